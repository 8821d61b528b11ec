"""The cooperative (one CTA per cell) kernels for mechanisms beyond the
reference's u16 tables. FP64: bit for bit against the reference's own outputs
(the 60-species / 300-reaction synthetic mechanism of tests/golden, run by the
reference's solver with enlarged capacities) and against the oracle (the
shipped mechanism; the 200-species / 1,200-reaction mechanism, where the
oracle is the reference's algorithm with 32-bit indices). Mixed: accuracy
against the FP64 path."""
import json
import os

import numpy as np
import pytest

import simstack_gb300 as sg

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
G = np.load(os.path.join(HERE, "golden", "golden_ref.npz"))
STATE = ("y", "h", "steps", "rejects", "pulses", "failed")


def synthetic_pair(oracle_lib, seed, species, reactions):
    pm = sg.Model.synthetic(seed=seed, species=species, reactions=reactions, bimolecular=0.7, products=1)
    om = oracle_lib.Mechanism()
    for s in range(species):
        om.add_species(f"S{s}", True)
    for r in range(pm.R):
        om.add_reaction(sg.model_equation(pm, r), "arr", (float(pm.k_const[r]), 0.0, 0.0))
    om.finalize()
    return pm, om


def assert_state(z, ref, cells=None):
    for name in STATE:
        a, b = z[name], ref[name]
        if cells is not None:
            a, b = a[..., :cells], b[..., :cells]
        assert np.ascontiguousarray(a).tobytes() == np.ascontiguousarray(b).tobytes(), \
            f"{name}: {np.count_nonzero(a != b)} entries differ"


def test_coop_f64_matches_reference_golden(module):
    """60 species / 300 reactions, 16 cells x 1 s: the reference's own outputs."""
    pm = sg.Model.synthetic(seed=7, species=60, reactions=300, bimolecular=0.7, products=1)
    module.coop_set_mech(pm, sg.method("rodas3"), sg.control(rtol=1e-4, atol=1e-12, max_steps=200000))
    info = module.coop_info()
    meta = json.load(open(os.path.join(HERE, "golden", "golden_meta.json")))["big_counts"]
    assert info["nnz"] == meta["nnz"] and info["l_entries"] == meta["lower"] and info["u_entries"] == meta["upper"]
    assert info["lu_updates"] == meta["updates"]
    z = sg.ZoneBlock(60, 300, 16, pad_to=16)
    for name in sg.ROWS_ORDER:
        z[name][...] = G[f"big_in_{name}"]
    module.coop_integrate(z, 1.0, precision=0)
    for name in STATE:
        assert z[name].tobytes() == G[f"big_out_{name}"].tobytes(), name
    module.reset_arena()


@pytest.mark.parametrize("method", ["rodas3", "ros3"])
def test_coop_f64_shipped_mechanism(module, oracle_lib, method):
    module.coop_set_mech(sg.Model.air(), sg.method(method), sg.control())
    z = sg.air_cells(100, seed=12)
    ref = z.copy()
    module.coop_integrate(z, 1.0, precision=0, lane_count=100)
    oracle_lib.Mechanism.air().advance(method, oracle_lib.control(), ref.as_dict(), ref.padded, 0, 100, 1.0, 0, 8)
    assert_state(z, ref, 100)
    module.reset_arena()


def test_coop_f64_pulsed_source(module, oracle_lib):
    """Discharge source and pulse trains through the segment machinery."""
    n = 16
    i = np.arange(n)
    zs = sg.dbd_zones(n, 300.0 + 10.0 * (i % 5), 0.005 * (i % 7), 0.05 + 0.1 * (i % 3), 5000.0 + 2500.0 * (i % 4))
    module.coop_set_mech(sg.Model.air(), sg.method("rodas3"), sg.control(rtol=1e-3, atol=1e8, max_steps=20000))
    ref = zs.copy()
    for step in range(3):
        t0, t1 = step * 1e-3, (step + 1) * 1e-3
        sg.dbd_prepare_source(zs, True, t0, t1)
        for name in ("src", "pulse", "period", "pulse_first", "pulse_count"):
            ref[name][...] = zs[name]
        module.coop_integrate(zs, t1 - t0, precision=0)
        oracle_lib.Mechanism.air().advance("rodas3", oracle_lib.control(rtol=1e-3, atol=1e8, max_steps=20000),
                                           ref.as_dict(), ref.padded, 0, ref.padded, t1 - t0, 0, 4)
        sg.dbd_commit_pulses(zs)
        ref.pulse_index = zs.pulse_index
        assert_state(zs, ref)
    assert zs["pulses"].min() > 0
    module.reset_arena()


def test_coop_f64_large_mechanism(module, oracle_lib):
    """200 species / 1,200 reactions (~1.76 M LU updates per factorisation), 3 cells x 0.05 s."""
    pm, om = synthetic_pair(oracle_lib, 4, 200, 1200)
    ctl = dict(rtol=1e-4, atol=1e-12, max_steps=200000)
    module.coop_set_mech(pm, sg.method("rodas3"), sg.control(**ctl))
    assert module.coop_info()["lu_updates"] == om.counts()["updates"]
    z = sg.synthetic_cells(pm, 3, seed=5)
    ref = z.copy()
    module.coop_integrate(z, 0.05, precision=0, lane_count=3)
    om.advance("rodas3", oracle_lib.control(**ctl), ref.as_dict(), ref.padded, 0, 3, 0.05, 0, 3)
    assert_state(z, ref, 3)
    module.reset_arena()


def test_coop_large_mechanism_64_cells(module, oracle_lib):
    """200 species / 1,200 reactions, 64 cells x 0.5 s (~475 steps per cell): the FP64 cooperative
    path bit for bit against the oracle, and the mixed cooperative path (FP32 LU in shared memory,
    FP64 refinement residual) within 1e-5 of it on every species of every cell (|a-b| / max(|b|,
    atol), no filter)."""
    pm, om = synthetic_pair(oracle_lib, 4, 200, 1200)
    ctl = dict(rtol=1e-4, atol=1e-12, max_steps=200000)
    module.coop_set_mech(pm, sg.method("rodas3"), sg.control(**ctl))
    z0 = sg.synthetic_cells(pm, 64, seed=5)
    z, zm, ref = z0.copy(), z0.copy(), z0.copy()
    module.coop_integrate(z, 0.5, precision=0, lane_count=64)
    module.coop_integrate(zm, 0.5, precision=2, lane_count=64)
    om.advance("rodas3", oracle_lib.control(**ctl), ref.as_dict(), ref.padded, 0, 64, 0.5, 0, 0)
    assert_state(z, ref, 64)
    a, b = zm["y"][:, :64], ref["y"][:, :64]
    rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-12)
    assert zm["failed"][:64].max() == 0.0 and rel.max() <= 1e-5, rel.max()
    module.reset_arena()


def test_coop_mixed_accuracy(module, oracle_lib):
    """Mixed cooperative path (FP32 LU in shared memory + FP64 refinement) vs FP64, 60-species mechanism."""
    pm = sg.Model.synthetic(seed=7, species=60, reactions=300, bimolecular=0.7, products=1)
    module.coop_set_mech(pm, sg.method("rodas3"), sg.control(rtol=1e-4, atol=1e-12, max_steps=200000))
    z = sg.synthetic_cells(pm, 256, seed=9)
    ref = z.copy()
    module.coop_integrate(z, 1.0, precision=2)
    module.coop_integrate(ref, 1.0, precision=0)
    a, b = z["y"], ref["y"]
    sig = b >= 1e-9 * b.sum(axis=0)
    rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
    assert z["failed"].max() == 0.0
    assert np.quantile(rel[sig], 0.99) < 1e-5 and rel[sig].max() < 1e-3, (rel[sig].max(), np.quantile(rel[sig], 0.99))
    module.reset_arena()


def test_coop_rejects_bad_launches(module):
    module.coop_set_mech(sg.Model.air(), sg.method("rodas3"), sg.control())
    z = sg.air_cells(8, seed=1)
    base = module.upload(z)
    for prec in (1, 3):
        with pytest.raises(sg.GpuError):
            module.coop_advance(z.launch(base, prec, 1.0))
    assert module.coop_advance(z.launch(base, 0, 0.0)) == 0.0
    module.reset_arena()
