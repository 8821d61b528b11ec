"""Generate tests/golden/nft_transport.npz from the reference's NFT code.

    make -C oracle ref            # builds oracle/_ref/libref_nft.so from the reference sources
    python tests/golden/make_nft_golden.py

Run on an x86-64 host: there the reference's transport runs under FTZ/DAZ
(NftFlushDenormals, src/sim/nft.cpp:1130-1136), its production mode. Each case
holds a group set's arrays before one window's transport, the window's inputs,
and the arrays after the reference's nft_transport<f32x8> (nft.cpp:1028-1106),
both in that mode ("ftz_*") and without it ("ieee_*", as the reference runs on
hosts where NftFlushDenormals is empty).

Cases:
  run600   the reference's own system (nft_default_params, 12 rails = 2 groups,
           the second half-padded, as test_kinetics.cpp:520) after 600 windows of
           nft_run<f32x8> (test_kinetics.cpp:503-511), captured between the window's
           plants and its transport (the split the tests also replay);
  edge_*   one synthetic group each: a single cell; sites up to the last cell;
           a last site row beyond the channel (the reference then applies none);
           site stride 0; no sites; deltas near the bottom of the f32 range, so
           that FTZ and IEEE results differ within a few substeps.
"""
from __future__ import annotations

import os
import platform
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

ARRAYS = ("rows", "hot", "cold", "sites")
OUTPUTS = ("rows", "hot", "sites", "out_sum", "evap_kg")


def aligned32(a: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a, np.float32).ravel()
    raw = np.empty(a.size + 8, np.float32)
    off = (-raw.ctypes.data % 32) // 4
    out = raw[off:off + a.size]
    out[...] = a
    return out


def transport_groups(before: dict, groups: int, cells: int, sites: int, site_offset: int, site_stride: int,
                     ref, env, substeps: int, ieee: bool) -> dict:
    per = {n: before[n].size // groups for n in ARRAYS}
    out = {n: [] for n in OUTPUTS}
    for g in range(groups):
        arr = {n: aligned32(before[n][g * per[n]:(g + 1) * per[n]]) for n in ARRAYS}
        if sites == 0:
            arr["sites"] = aligned32(np.zeros(288, np.float32))
        out_sum, evap = O.ref_nft_transport_arrays(arr["rows"], arr["hot"], arr["cold"], arr["sites"], cells, sites,
                                                   site_offset, site_stride, ref, env, substeps, ieee=ieee)
        out["rows"].append(arr["rows"].copy())
        out["hot"].append(arr["hot"].copy())
        out["sites"].append(arr["sites"][:per["sites"]].copy())
        out["out_sum"].append(out_sum)
        out["evap_kg"].append(evap)
    return {n: np.concatenate(v) for n, v in out.items()}


def capture_run(windows: int) -> dict:
    s = O.RefNftSystem(12)
    s.run(windows)
    s.prepare()
    ref, env, substeps = s.inputs()
    before = {n: np.concatenate([s.group_views(g)[n].copy() for g in range(s.groups)]) for n in ARRAYS}
    s.transport()   # the reference's own split window, this host's mode
    after_sys = {n: np.concatenate([s.group_views(g)[n].copy() for g in range(s.groups)])
                 for n in ("rows", "hot", "sites", "out_sum", "evap_kg")}
    case = {"groups": s.groups, "cells": s.cells, "sites": s.sites, "site_offset": s.site_offset,
            "site_stride": s.site_stride, "substeps": substeps, "ref": ref, "env": env, "before": before}
    ftz = transport_groups(before, s.groups, s.cells, s.sites, s.site_offset, s.site_stride, ref, env, substeps, False)
    for n in OUTPUTS:   # the array entry point reproduces the system's own transport
        assert ftz[n].tobytes() == after_sys[n].tobytes(), n
    case["ftz"] = ftz
    case["ieee"] = transport_groups(before, s.groups, s.cells, s.sites, s.site_offset, s.site_stride, ref, env,
                                    substeps, True)
    s.close()
    return case


def capture_edge(seed: int, cells: int, sites: int, site_offset: int, site_stride: int, substeps: int,
                 scale: float = 1.0) -> dict:
    rng = np.random.default_rng(seed)
    rows = (rng.normal(0.0, 1.0, (cells, 9, 8)) * scale).astype(np.float32)
    rows[:, :, 6:] = 0.0   # two padding lanes, as in a half-padded group
    hot = np.zeros((cells, 4, 8), np.float32)
    hot[:, 0] = rng.uniform(0.05, 0.9, (cells, 8))     # Courant number
    hot[:, 3] = rng.uniform(0.0, 0.02, (cells, 8))     # O2 transfer per substep
    cold = np.zeros((cells, 80), np.float32)
    for off, lo, hi in ((24, 0.0, 1e-3), (32, 0.0, 1e-5), (40, 0.0, 1e-6), (48, 0.0, 1e-9)):   # kw, kr, ge, ev
        cold[:, off:off + 8] = rng.uniform(lo, hi, (cells, 8))
    site_arr = np.zeros((max(sites, 1), 288), np.float32)
    site_arr[:, 16 + 8:16 + 72] = rng.uniform(0.0, 0.05, (max(sites, 1), 64))   # drop[1..8]
    before = {"rows": rows.ravel(), "hot": hot.ravel(), "cold": cold.ravel(), "sites": site_arr[:sites].ravel()}
    ref = np.array([20.0, 8.0, 150.0, 10.0, 40.0, 200.0, 160.0, 50.0, 60.0], np.float32)
    env = np.array([24.0, 150.0, 900.0, 140.0], np.float32)
    case = {"groups": 1, "cells": cells, "sites": sites, "site_offset": site_offset, "site_stride": site_stride,
            "substeps": substeps, "ref": ref, "env": env, "before": before}
    case["ftz"] = transport_groups(before, 1, cells, sites, site_offset, site_stride, ref, env, substeps, False)
    case["ieee"] = transport_groups(before, 1, cells, sites, site_offset, site_stride, ref, env, substeps, True)
    return case


def main() -> None:
    if platform.machine() not in ("x86_64", "AMD64"):
        raise SystemExit("run on an x86-64 host: the fixtures record the reference's FTZ/DAZ mode")
    cases = {"run600": capture_run(600),
             "edge_one_cell": capture_edge(1, 1, 1, 0, 3, 17),
             "edge_last_cell_site": capture_edge(2, 40, 5, 3, 9, 23),
             "edge_site_beyond": capture_edge(3, 40, 5, 5, 9, 23),
             "edge_stride0": capture_edge(4, 30, 3, 7, 0, 11),
             "edge_no_sites": capture_edge(5, 30, 0, 0, 3, 11),
             "edge_denormal": capture_edge(6, 24, 0, 0, 3, 40, scale=1e-36)}
    out = {}
    for name, c in cases.items():
        for key in ("groups", "cells", "sites", "site_offset", "site_stride", "substeps"):
            out[f"{name}/{key}"] = np.array(c[key], np.uint32)
        out[f"{name}/ref"] = c["ref"]
        out[f"{name}/env"] = c["env"]
        for n, v in c["before"].items():
            out[f"{name}/in_{n}"] = v
        for mode in ("ftz", "ieee"):
            for n, v in c[mode].items():
                out[f"{name}/{mode}_{n}"] = v
        differ = sum(c["ftz"][n].tobytes() != c["ieee"][n].tobytes() for n in OUTPUTS)
        print(f"{name}: {c['groups']} groups x {c['cells']} cells, {c['substeps']} substeps; "
              f"outputs where FTZ and IEEE differ: {differ}")
    path = os.path.join(HERE, "nft_transport.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
