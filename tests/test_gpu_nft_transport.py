"""gpu_nft_transport against the reference's NFT transport (src/sim/nft.cpp:1028-1106).

1. Fixtures made by the reference (tests/golden/make_nft_golden.py, x86-64): arrays
   before one window's transport and after the reference's nft_transport<f32x8>, in
   its production FTZ/DAZ mode and in IEEE mode -- bit for bit, both modes.
2. Where the reference was compiled on this host (oracle/_ref/libref_nft.so): larger
   synthetic groups against the reference's transport run here, and the reference's
   own window driver with the GPU transport put in place of its transport, against
   nft_run<f32x8> (test_kinetics.cpp:503-511) -- the same system state bit for bit.
   The reference's denormal mode is FTZ/DAZ on x86-64 hosts and IEEE elsewhere
   (NftFlushDenormals is empty there), so the GPU runs in this host's mode."""
import os
import platform
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

import simstack_gb300 as sg  # noqa: E402
from oracle import oracle as O  # noqa: E402

G = np.load(os.path.join(HERE, "golden", "nft_transport.npz"))
CASES = sorted({k.split("/")[0] for k in G.files})
HOST_FTZ = platform.machine() in ("x86_64", "AMD64")
OUTPUTS = ("rows", "hot", "sites", "out_sum", "evap_kg")


def run_gpu(module, arrays, groups, cells, sites, site_offset, site_stride, ref, env, substeps, ftz):
    nt = sg.NftTransport(module, groups, cells, sites, site_offset, site_stride)
    for name in ("rows", "hot", "cold", "sites"):
        if name != "sites" or sites:
            nt.upload(name, arrays[name])
    ms = nt.run(ref, *env, substeps, flush_denormals=ftz)
    out = {n: nt.download(n) for n in ("rows", "hot", "out_sum", "evap_kg")}
    out["sites"] = nt.download("sites")[: groups * sites * 288]
    return out, ms


@pytest.mark.parametrize("mode", ["ftz", "ieee"])
@pytest.mark.parametrize("case", CASES)
def test_fixture_bit_identical(module, case, mode):
    c = {k.split("/", 1)[1]: G[k] for k in G.files if k.startswith(case + "/")}
    meta = {k: int(c[k]) for k in ("groups", "cells", "sites", "site_offset", "site_stride", "substeps")}
    arrays = {n: c[f"in_{n}"] for n in ("rows", "hot", "cold", "sites")}
    got, _ = run_gpu(module, arrays, meta["groups"], meta["cells"], meta["sites"], meta["site_offset"],
                     meta["site_stride"], c["ref"], c["env"], meta["substeps"], mode == "ftz")
    for n in OUTPUTS:
        want = c[f"{mode}_{n}"]
        assert got[n].tobytes() == want.tobytes(), \
            f"{case}/{mode} {n}: {np.count_nonzero(got[n].view(np.uint32) != want.view(np.uint32))} floats differ"
    module.reset_arena()


def test_fixture_modes_differ():
    """The fixtures exercise the denormal mode: FTZ and IEEE give different bits somewhere."""
    assert any(G[f"{c}/ftz_rows"].tobytes() != G[f"{c}/ieee_rows"].tobytes() for c in CASES)


def aligned32(a):
    a = np.ascontiguousarray(a, np.float32).ravel()
    raw = np.empty(a.size + 8, np.float32)
    off = (-raw.ctypes.data % 32) // 4
    out = raw[off:off + a.size]
    out[...] = a
    return out


@pytest.mark.parametrize("cells,sites,offset,stride,substeps", [(4096, 80, 25, 51, 3), (1000, 333, 0, 3, 9),
                                                                 (129, 43, 0, 3, 60)])
def test_live_reference_larger_groups(module, cells, sites, offset, stride, substeps):
    """Four synthetic groups per case against the reference's transport run on this host:
    channel lengths of the serving workload (4,096 cells), runs of several cells per
    thread, and a length one past a whole number of runs."""
    if not O.ref_nft_available():
        pytest.skip("reference sources not present: oracle/_ref/libref_nft.so was not built")
    rng = np.random.default_rng(cells + sites)
    groups = 4
    rows = rng.normal(0.0, 0.5, (groups, cells, 9, 8)).astype(np.float32)
    hot = np.zeros((groups, cells, 4, 8), np.float32)
    hot[:, :, 0] = rng.uniform(0.05, 0.9, (groups, cells, 8))
    hot[:, :, 3] = rng.uniform(0.0, 0.02, (groups, cells, 8))
    cold = np.zeros((groups, cells, 80), np.float32)
    for off, hi in ((24, 1e-3), (32, 1e-5), (40, 1e-6), (48, 1e-9)):
        cold[:, :, off:off + 8] = rng.uniform(0.0, hi, (groups, cells, 8))
    site_arr = np.zeros((groups, sites, 288), np.float32)
    site_arr[:, :, 24:88] = rng.uniform(0.0, 0.05, (groups, sites, 64))
    ref = np.array([21.0, 8.5, 140.0, 12.0, 45.0, 210.0, 150.0, 48.0, 64.0], np.float32)
    env = np.array([25.0, 120.0, 800.0, 150.0], np.float32)
    want = {n: [] for n in OUTPUTS}
    for g in range(groups):
        a = {"rows": aligned32(rows[g]), "hot": aligned32(hot[g]), "cold": aligned32(cold[g]), "sites": aligned32(site_arr[g])}
        out_sum, evap = O.ref_nft_transport_arrays(a["rows"], a["hot"], a["cold"], a["sites"], cells, sites, offset, stride,
                                                   ref, env, substeps)
        for n, v in (("rows", a["rows"]), ("hot", a["hot"]), ("sites", a["sites"]), ("out_sum", out_sum), ("evap_kg", evap)):
            want[n].append(v.copy())
    got, _ = run_gpu(module, {"rows": rows, "hot": hot, "cold": cold, "sites": site_arr}, groups, cells, sites, offset,
                     stride, ref, env, substeps, HOST_FTZ)
    for n in OUTPUTS:
        w = np.concatenate(want[n])
        assert got[n].tobytes() == w.tobytes(), f"{n}: {np.count_nonzero(got[n].view(np.uint32) != w.view(np.uint32))} differ"
    module.reset_arena()


def test_reference_window_driver_with_gpu_transport(module):
    """60 windows of the reference's NFT system (12 rails = 2 groups, the second half-padded,
    test_kinetics.cpp:520) with every window's transport on the GPU: the system state is the
    state nft_run<f32x8> reaches."""
    if not O.ref_nft_available():
        pytest.skip("reference sources not present: oracle/_ref/libref_nft.so was not built")
    want = O.RefNftSystem(12)
    want.run(60)
    s = O.RefNftSystem(12)
    nt = sg.NftTransport(module, s.groups, s.cells, s.sites, s.site_offset, s.site_stride)
    for _ in range(60):
        s.prepare()
        ref, env, substeps = s.inputs()
        views = [s.group_views(g) for g in range(s.groups)]
        for name in ("rows", "hot", "cold", "sites"):
            nt.upload(name, np.concatenate([v[name] for v in views]))
        nt.run(ref, *env, substeps, flush_denormals=HOST_FTZ)
        for name in ("rows", "hot", "sites", "out_sum", "evap_kg"):
            host = nt.download(name)
            per = host.size // s.groups
            for g, v in enumerate(views):
                v[name][...] = host[g * per:(g + 1) * per]
        s.finish()
    assert s.digest() == want.digest()
    s.close()
    want.close()
    module.reset_arena()


def test_rejects_bad_launches(module):
    """Null records, empty channels and misaligned arrays are refused before any launch."""
    import ctypes as C

    nt = sg.NftTransport(module, 1, 8, 2, 0, 3)
    L = sg.lib()
    assert L.gpu_nft_transport(None, None) != 0
    t = sg.GpuNftTransport()
    for name in ("rows", "hot", "cold", "sites", "out_sum", "evap_kg"):
        setattr(t, name, nt.dev[name])
    t.groups, t.cells, t.sites_count, t.site_offset, t.site_stride, t.substeps = 1, 8, 2, 0, 3, 4
    assert L.gpu_nft_transport(C.byref(t), None) == 0
    t.cells = 0
    assert L.gpu_nft_transport(C.byref(t), None) != 0
    t.cells = 8
    t.rows = nt.dev["rows"] + 4
    assert L.gpu_nft_transport(C.byref(t), None) != 0
    module.reset_arena()
