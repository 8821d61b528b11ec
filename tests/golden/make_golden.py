"""Generate tests/golden/*.npz from the reference's own CPU solver.

    make -C oracle ref            # builds oracle/_ref/ from the reference sources
    python tests/golden/make_golden.py

Runs only where the reference sources were compiled into oracle/_ref/ (the
fixtures it writes are committed, so the tests need neither). Inputs are
generated with this repository's seeded workload generator and stored in the
fixtures next to the reference's outputs, so a test replays exactly the same
inputs through the oracle.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import simstack_gb300 as sg  # noqa: E402
from oracle import oracle as O  # noqa: E402

STATE = ("y", "h", "steps", "rejects", "pulses", "failed")
BENCH_CTL = dict(rtol=1e-4, atol=6.02214076e8, h_min=1e-14, h_max=0.0, h_start=1e-9, max_steps=1_000_000)
DBD_CTL = dict(rtol=1e-3, atol=1e8, h_min=1e-14, h_max=0.0, h_start=1e-9, max_steps=20000)


def block_arrays(z: sg.ZoneBlock, prefix: str) -> dict:
    out = {}
    for name in sg.ROWS_ORDER:
        out[f"{prefix}{name}"] = np.array(z[name])
    return out


def aligned_block(z: sg.ZoneBlock) -> dict:
    """Copies of the zone block's rows in 64-byte aligned arrays (the reference's f64x4 lanes need it)."""
    b = {}
    for name in sg.ROWS_ORDER:
        v = O.aligned_zeros(z[name].shape)
        v[...] = z[name]
        b[name] = v
    return b


def main() -> None:
    assert O.ref_available(), "build oracle/_ref first: make -C oracle ref"
    out = {}
    meta = {}

    # 1. mechanism tables and signature
    km, sig, gen_sig = O.ref_air_kinmech()
    with open(os.path.join(HERE, "air_kinmech.bin"), "wb") as f:
        f.write(km)
    meta["air_signature"] = f"0x{sig:016x}"
    meta["air_generated_signature"] = f"0x{gen_sig:016x}"

    # 2. rate constants on a temperature grid (1 atm)
    Ts = np.array([250.0, 288.0, 295.5, 303.0, 320.0, 350.0, 400.0])
    Ms = 101325.0 / (1.380649e-23 * Ts) * 1e-6
    out["rates_T"], out["rates_M"] = Ts, Ms
    out["rates_k"] = np.stack([O.ref_air_rate_constants(T, M) for T, M in zip(Ts, Ms)])

    # 3. humid-air sample: 64 cells, 1 s, rtol 1e-4, f64x4 generated (the production CPU path)
    z = sg.air_cells(64, seed=1)
    out.update(block_arrays(z, "c1_in_"))
    b = aligned_block(z)
    O.ref_air_advance("rodas3", O.control(**BENCH_CTL), b, z.padded, 0, z.padded, 1.0, "f64x4_gen")
    for name in STATE:
        out[f"c1_out_{name}"] = np.array(b[name])

    # 4. f32 Delta lanes (f32x8 generated) under the reference's DBD control, 0.05 s
    z = sg.air_cells(64, seed=3)
    out.update(block_arrays(z, "f32_in_"))
    b = aligned_block(z)
    O.ref_air_advance("rodas3", O.control(**DBD_CTL), b, z.padded, 0, z.padded, 0.05, "f32x8_gen")
    for name in STATE:
        out[f"f32_out_{name}"] = np.array(b[name])

    # 5. Ros3 and Ros2 through the reference's table walk (f64 scalar lanes), 0.5 s
    for meth in ("ros3", "ros2"):
        z = sg.air_cells(32, seed=9)
        out.update(block_arrays(z, f"{meth}_in_"))
        b = aligned_block(z)
        O.ref_air_advance(meth, O.control(**BENCH_CTL), b, z.padded, 0, z.padded, 0.5, "f64_table")
        for name in STATE:
            out[f"{meth}_out_{name}"] = np.array(b[name])

    # 6. pulsed DBD zones (the reference's test set-up), 5 master steps of 1 ms: per-step
    # source/pulse inputs are stored, the state after every step is the reference's
    n = 16
    i = np.arange(n)
    zs = sg.dbd_zones(n, 300.0 + 10.0 * (i % 5), 0.005 * (i % 7), 0.05 + 0.1 * (i % 3), 5000.0 + 2500.0 * (i % 4))
    out.update(block_arrays(zs, "dbd_in_"))
    b = aligned_block(zs)
    for step in range(5):
        t0, t1 = step * 1e-3, (step + 1) * 1e-3
        for name in sg.ROWS_ORDER:   # prepare_source reads the current state
            zs[name][...] = b[name]
        sg.dbd_prepare_source(zs, True, t0, t1)
        for name in ("src", "pulse", "period", "pulse_first", "pulse_count"):
            b[name][...] = zs[name]
            out[f"dbd_step{step}_{name}"] = np.array(zs[name])
        O.ref_air_advance("rodas3", O.control(**DBD_CTL), b, zs.padded, 0, zs.padded, t1 - t0, "f64x4_gen")
        sg.dbd_commit_pulses(zs)
        for name in STATE:
            out[f"dbd_step{step}_out_{name}"] = np.array(b[name])

    # 7. Robertson at t = 40, all three methods (test_kinetics.cpp:151-180 set-up)
    rob_ctl = O.control(rtol=1e-6, atol=1e-12, h_min=0.0, h_start=1e-6, max_steps=100000)
    for meth in ("ros2", "ros3", "rodas3"):
        y, st = O.ref_robertson(meth, rob_ctl, 40.0)
        out[f"rob_{meth}_y"], out[f"rob_{meth}_stats"] = y, st

    # 8. discharge source for a few compositions and energies
    rng = np.random.default_rng(5)
    ys = 10.0 ** rng.uniform(8, 19, size=(6, 17))
    en = np.array([0.0, 1e-6, 1e-4, 0.01, 0.5, 3.0])
    Tsrc = np.array([290.0, 300.0, 310.0, 330.0, 350.0, 400.0])
    out["src_y"], out["src_energy"], out["src_T"] = ys, en, Tsrc
    out["src_delta"] = np.stack([O.ref_air_source_delta(ys[j], en[j], Tsrc[j]) for j in range(6)])

    # 9. a synthetic abstract mechanism inside the reference's enlarged u16 tables:
    # 60 species, 300 reactions, 1 product; tables and an integration of 16 cells
    m = sg.Model.synthetic(seed=7, species=60, reactions=300, bimolecular=0.7, products=1)
    eqs = synthetic_equations(seed=7, species=60, reactions=300)
    rb = O.RefBigMechanism()
    for s in range(60):
        rb.add_species(f"S{s}", True)
    for eq, k in eqs:
        rb.add_reaction(eq, "arr", (k, 0.0, 0.0))
    rb.finalize()
    assert not rb.error, rb.error
    c = rb.counts()
    meta["big_counts"] = c
    piv, upd = rb.lu_ops()
    out["big_pivots"], out["big_updates"] = piv, upd
    zb = sg.synthetic_cells(m, 16, seed=8)
    out.update(block_arrays(zb, "big_in_"))
    b = aligned_block(zb)
    rb.advance("rodas3", O.control(rtol=1e-4, atol=1e-12, h_min=1e-14, h_start=1e-9, max_steps=200000), b, zb.padded, 0,
               zb.padded, 1.0, variant=0)
    for name in STATE:
        out[f"big_out_{name}"] = np.array(b[name])
    out["big_k"] = m.k_const

    np.savez_compressed(os.path.join(HERE, "golden_ref.npz"), **out)
    with open(os.path.join(HERE, "golden_meta.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print("wrote", os.path.join(HERE, "golden_ref.npz"), sum(v.nbytes for v in out.values()), "bytes raw")


def synthetic_equations(seed: int, species: int, reactions: int):
    """The equations and rate constants of sg.Model.synthetic (the module's generator)."""
    m = sg.Model.synthetic(seed=seed, species=species, reactions=reactions, bimolecular=0.7, products=1)
    return [(sg.model_equation(m, r), float(m.k_const[r])) for r in range(m.R)]


if __name__ == "__main__":
    main()
