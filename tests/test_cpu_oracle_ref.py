"""The oracle against the reference's own CPU solver, live (compiled from the
reference sources into oracle/_ref/ where they are present; skipped elsewhere,
where tests/golden/ carries the pin). CPU only."""
import numpy as np
import pytest

import simstack_gb300 as sg
from oracle import oracle as O

pytestmark = pytest.mark.skipif(not O.ref_available(), reason="oracle/_ref not built (reference sources absent)")

STATE = ("y", "h", "steps", "rejects", "pulses", "failed")


def aligned(z):
    b = {}
    for name in sg.ROWS_ORDER:
        v = O.aligned_zeros(z[name].shape)
        v[...] = z[name]
        b[name] = v
    return b


@pytest.mark.parametrize("variant,precision,ctl", [
    ("f64x4_gen", 0, {}), ("f64x4_table", 0, {}), ("f64_table", 0, {}),
    ("f32x8_gen", 1, dict(rtol=1e-3, atol=1e8, max_steps=20000)), ("f32_gen", 1, dict(rtol=1e-3, atol=1e8, max_steps=20000)),
])
@pytest.mark.parametrize("seed", [11, 12])
def test_oracle_matches_reference_variants(oracle_lib, variant, precision, ctl, seed):
    dur = 1.0 if precision == 0 else 0.05
    z = sg.air_cells(128, seed=seed)
    b = aligned(z)
    O.ref_air_advance("rodas3", O.control(**ctl), b, z.padded, 0, z.padded, dur, variant)
    O.Mechanism.air().advance("rodas3", O.control(**ctl), z.as_dict(), z.padded, 0, z.padded, dur, precision, 1)
    for name in STATE:
        assert z[name].tobytes() == b[name].tobytes(), name


def test_rate_constants_and_source_match_reference(oracle_lib):
    m = O.Mechanism.air()
    rng = np.random.default_rng(2)
    for T in rng.uniform(250, 450, 20):
        M = 101325.0 / (1.380649e-23 * T) * 1e-6
        assert np.array_equal(m.rate_constants(T, M), O.ref_air_rate_constants(T, M))
    for _ in range(20):
        y = 10.0 ** rng.uniform(6, 19, 17)
        e, T = 10.0 ** rng.uniform(-8, 1), rng.uniform(280, 420)
        assert np.array_equal(O.source_delta(y, e, T), O.ref_air_source_delta(y, e, T))


def test_threaded_reference_path_and_module_free_inputs(oracle_lib):
    """The CPU baselines' inputs (oracle.air_block: no GPU module) equal the module's workload
    generator bit for bit, rate constants from the reference included; the reference's threaded
    production path (dbd_advance_threads) gives the oracle's bits on them."""
    b, P, used = O.air_block(1000, seed=9, first_cell=77)
    z = sg.air_cells(1000, seed=9, first_cell=77)
    assert used == "reference" and P == z.padded
    for name in sg.ROWS_ORDER:
        assert b[name].tobytes() == np.ascontiguousarray(z[name]).tobytes(), name
    O.ref_air_advance_threads("rodas3", O.control(), b, P, 0, P, 1.0, 4)
    O.Mechanism.air().advance("rodas3", O.control(), z.as_dict(), z.padded, 0, z.padded, 1.0, 0, 2)
    for name in STATE:
        assert z[name].tobytes() == b[name].tobytes(), name
