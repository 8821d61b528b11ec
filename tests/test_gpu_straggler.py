"""Straggler hand-off: FP64 cells still stepping after a budget of step attempts
are parked by the lane kernels and finished by the cooperative kernel, keeping
every bit of the oracle (the reference's algorithm)."""
import numpy as np
import pytest

import simstack_gb300 as sg

pytestmark = pytest.mark.gpu


@pytest.fixture
def budget(module, request):
    module.set_straggler_budget(request.param)
    yield request.param
    module.set_straggler_budget(sg.DEFAULT_STRAGGLER_BUDGET)


def source_cells(cells, seed=3):
    z = sg.air_cells(cells, seed=seed)
    sg.air_source(z, seed=seed, P0=1e-2, decades=3.0)
    return z


@pytest.mark.parametrize("budget", [40, 150], indirect=True)
@pytest.mark.parametrize("kind", [0, 2])
def test_f64_handoff_bit_identical(module, oracle_lib, budget, kind):
    """Uneven stiffness (discharge source over 3 decades of power), 1,024 cells x 5 s."""
    module.set_mech(sg.Model.air().kinmech(), sg.method("rodas3"), sg.control())
    module.set_tuning(kind=kind)
    z = source_cells(1024)
    ref = z.copy()
    module.integrate(z, 5.0, precision=0)
    parked = module.parked_cells()
    oracle_lib.Mechanism.air().advance("rodas3", oracle_lib.control(), ref.as_dict(), ref.padded, 0, ref.padded, 5.0, 0, 0)
    module.set_tuning()
    assert parked > 0
    for name in ("y", "h", "steps", "rejects", "pulses", "failed"):
        assert z[name].tobytes() == ref[name].tobytes(), f"{name}: {np.count_nonzero(z[name] != ref[name])} differ"


@pytest.mark.parametrize("budget", [40], indirect=True)
def test_f64_handoff_pulsed_zones(module, oracle_lib, budget):
    """Pulse segments continue across the hand-off."""
    n = 64
    i = np.arange(n)
    zs = sg.dbd_zones(n, 300.0 + 10.0 * (i % 5), 0.005 * (i % 7), 0.05 + 0.1 * (i % 3), 5000.0 + 2500.0 * (i % 4))
    ctl = dict(rtol=1e-3, atol=1e8, max_steps=20000)
    module.set_mech(sg.Model.air().kinmech(), sg.method("rodas3"), sg.control(**ctl))
    ref = zs.copy()
    for step in range(3):
        t0, t1 = step * 1e-3, (step + 1) * 1e-3
        sg.dbd_prepare_source(zs, True, t0, t1)
        for name in ("src", "pulse", "period", "pulse_first", "pulse_count"):
            ref[name][...] = zs[name]
        module.integrate(zs, t1 - t0, precision=0)
        oracle_lib.Mechanism.air().advance("rodas3", oracle_lib.control(**ctl), ref.as_dict(), ref.padded, 0, ref.padded,
                                           t1 - t0, 0, 0)
        sg.dbd_commit_pulses(zs)
        for name in ("y", "h", "steps", "rejects", "pulses", "failed"):
            assert zs[name].tobytes() == ref[name].tobytes(), (step, name)
    assert zs["pulses"].min() > 0


@pytest.mark.parametrize("budget", [40], indirect=True)
def test_mixed_keeps_its_cells(module, oracle_lib, budget):
    """The mixed path does not hand off (its FP32-pipe lane steps are shorter than the
    cooperative FP64 steps): the same bits with and without a budget."""
    module.set_mech(sg.Model.air().kinmech(), sg.method("rodas3"), sg.control())
    z = source_cells(512, seed=4)
    a = z.copy()
    module.integrate(a, 2.0, precision=2)
    module.set_straggler_budget(0)
    b = z.copy()
    module.integrate(b, 2.0, precision=2)
    for name in ("y", "h", "steps", "rejects", "failed"):
        assert a[name].tobytes() == b[name].tobytes(), name
