"""The oracle pinned to the reference's own outputs (tests/golden/, produced by
tests/golden/make_golden.py from the reference's CPU solver). CPU only.

Every comparison of solver output is bit for bit: the oracle performs the
reference's IEEE operations in the reference's order."""
import json
import os

import numpy as np
import pytest

import simstack_gb300 as sg

HERE = os.path.dirname(os.path.abspath(__file__))
G = np.load(os.path.join(HERE, "golden", "golden_ref.npz"))
META = json.load(open(os.path.join(HERE, "golden", "golden_meta.json")))
STATE = ("y", "h", "steps", "rejects", "pulses", "failed")
BENCH_CTL = dict(rtol=1e-4, atol=6.02214076e8, h_min=1e-14, h_max=0.0, h_start=1e-9, max_steps=1_000_000)
DBD_CTL = dict(rtol=1e-3, atol=1e8, h_min=1e-14, h_max=0.0, h_start=1e-9, max_steps=20000)


def zone_from(prefix: str, n: int, R: int) -> sg.ZoneBlock:
    cells = G[f"{prefix}y"].shape[1]
    z = sg.ZoneBlock(n, R, cells, pad_to=cells)
    for name in sg.ROWS_ORDER:
        z[name][...] = G[f"{prefix}{name}"]
    return z


def assert_state(z, prefix):
    for name in STATE:
        got, want = z[name], G[f"{prefix}{name}"]
        assert got.tobytes() == want.tobytes(), f"{prefix}{name}: {np.count_nonzero(got != want)} entries differ"


def test_kinmech_bytes_and_signature(oracle_lib):
    ref = open(os.path.join(HERE, "golden", "air_kinmech.bin"), "rb").read()
    b, sig = oracle_lib.Mechanism.air().kinmech()
    assert b == ref
    assert f"0x{sig:016x}" == META["air_signature"] == "0x6f2a410e23c0192e"
    # the module's own symbolic phase produces the same record
    km = sg.Model.air().kinmech()
    assert sg.kinmech_bytes(km) == ref and f"0x{sg.signature(km):016x}" == META["air_signature"]


def test_rate_constants(oracle_lib):
    """Host libm: identical on the machine that made the fixtures; within 2 ulp elsewhere."""
    om, pm = oracle_lib.Mechanism.air(), sg.Model.air()
    for T, M, want in zip(G["rates_T"], G["rates_M"], G["rates_k"]):
        for got in (om.rate_constants(T, M), pm.rate_constants(T, M)):
            np.testing.assert_allclose(got, want, rtol=5e-16, atol=0)


def test_air_64_cells_f64x4(oracle_lib):
    z = zone_from("c1_in_", 17, 44)
    oracle_lib.Mechanism.air().advance("rodas3", oracle_lib.control(**BENCH_CTL), z.as_dict(), z.padded, 0, z.padded, 1.0, 0, 1)
    assert_state(z, "c1_out_")


def test_f32_lanes(oracle_lib):
    z = zone_from("f32_in_", 17, 44)
    oracle_lib.Mechanism.air().advance("rodas3", oracle_lib.control(**DBD_CTL), z.as_dict(), z.padded, 0, z.padded, 0.05, 1, 1)
    assert_state(z, "f32_out_")


@pytest.mark.parametrize("method", ["ros3", "ros2"])
def test_table_walk_methods(oracle_lib, method):
    z = zone_from(f"{method}_in_", 17, 44)
    oracle_lib.Mechanism.air().advance(method, oracle_lib.control(**BENCH_CTL), z.as_dict(), z.padded, 0, z.padded, 0.5, 0, 1)
    assert_state(z, f"{method}_out_")


def test_pulsed_dbd_zones(oracle_lib):
    z = zone_from("dbd_in_", 17, 44)
    m = oracle_lib.Mechanism.air()
    for step in range(5):
        for name in ("src", "pulse", "period", "pulse_first", "pulse_count"):
            z[name][...] = G[f"dbd_step{step}_{name}"]
        m.advance("rodas3", oracle_lib.control(**DBD_CTL), z.as_dict(), z.padded, 0, z.padded, 1e-3, 0, 1)
        assert_state(z, f"dbd_step{step}_out_")
    assert z["pulses"].min() > 0


@pytest.mark.parametrize("method", ["ros2", "ros3", "rodas3"])
def test_robertson(oracle_lib, method):
    O = oracle_lib
    m = O.Mechanism()
    for s in ("A", "B", "C"):
        m.add_species(s, True)
    m.add_reaction("A -> B", "arr", (0.04, 0, 0))
    m.add_reaction("B + B -> C + B", "arr", (3.0e7, 0, 0))
    m.add_reaction("B + C -> A + C", "arr", (1.0e4, 0, 0))
    m.finalize()
    ctl = O.control(rtol=1e-6, atol=1e-12, h_min=0.0, h_start=1e-6, max_steps=100000)
    y, t, h, st = m.integrate(method, ctl, m.rate_constants(300.0, 1.0), np.zeros(3), [1.0, 0.0, 0.0], 40.0)
    assert y.tobytes() == G[f"rob_{method}_y"].tobytes() and np.array_equal(st, G[f"rob_{method}_stats"])
    # and the reference's own accuracy check against the published solution (test_kinetics.cpp:164-177)
    ref = np.array([0.7158270687193267, 9.185534764557338e-06, 0.2841637457458339])
    assert t == 40.0 and np.all(np.abs(y - ref) / ref < 1e-4) and abs(y.sum() - 1.0) < 1e-12


def test_source_delta(oracle_lib):
    for j in range(len(G["src_energy"])):
        want = G["src_delta"][j]
        got_oracle = oracle_lib.source_delta(G["src_y"][j], G["src_energy"][j], G["src_T"][j])
        got_module = np.zeros(17)
        y = np.ascontiguousarray(G["src_y"][j])
        sg.lib().kin_air_source_delta(y.ctypes.data, 17, G["src_energy"][j], G["src_T"][j], got_module.ctypes.data)
        for got in (got_oracle, got_module):
            np.testing.assert_allclose(got, want, rtol=1e-14, atol=1e-300)


def test_synthetic_mechanism_tables_and_integration(oracle_lib):
    """60 species / 300 reactions: the wide-index oracle reproduces the reference's
    u16 tables (elimination lists op for op) and its integration bit for bit."""
    O = oracle_lib
    pm = sg.Model.synthetic(seed=7, species=60, reactions=300, bimolecular=0.7, products=1)
    om = O.Mechanism()
    for s in range(60):
        om.add_species(f"S{s}", True)
    for r in range(pm.R):
        om.add_reaction(sg.model_equation(pm, r), "arr", (float(pm.k_const[r]), 0.0, 0.0))
    om.finalize()
    c = om.counts()
    for key in ("n", "R", "nnz", "pivots", "updates", "lower", "upper"):
        assert c[key] == META["big_counts"][key], key
    piv, upd = om.lu_ops()
    assert np.array_equal(piv, G["big_pivots"]) and np.array_equal(upd, G["big_updates"])
    assert np.array_equal(pm.k_const, G["big_k"])
    z = zone_from("big_in_", 60, 300)
    om.advance("rodas3", O.control(rtol=1e-4, atol=1e-12, h_min=1e-14, h_start=1e-9, max_steps=200000), z.as_dict(),
               z.padded, 0, z.padded, 1.0, 0, 1)
    assert_state(z, "big_out_")
