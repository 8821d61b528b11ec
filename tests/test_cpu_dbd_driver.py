"""The DBD zone driver (src/sim/dbd.cpp:118-158, 466-483) restated on the host -- the
discharge source and pulse schedule, the pulse commit, the plug flow -- against the
reference's own driver (oracle/_ref, ref_dbd_run), bit for bit, with the oracle doing the
advance. This pins the host-side sequence that the device driver's GPU test compares
with where the reference is not built. CPU only."""
import numpy as np
import pytest

import simstack_gb300 as sg
from oracle import oracle as O

pytestmark = pytest.mark.skipif(not O.ref_available(), reason="oracle/_ref not built (reference sources absent)")

CTL = dict(rtol=1e-3, atol=1e8, h_min=1e-14, h_start=1e-9, max_steps=20000)


def zones(n=24):
    i = np.arange(n)
    return sg.dbd_zones(n, 300.0 + 10.0 * (i % 5), 0.005 * (i % 7), 0.05 + 0.1 * (i % 3), 5000.0 + 2500.0 * (i % 4))


def flow_exchange_host(z, residence_s, dt):
    """dbd.cpp:468-483, back to front so every zone sees its neighbour's old state."""
    a = dt * z.cells / residence_s
    y = z["y"]
    for i in range(z.cells - 1, -1, -1):
        if i == 0:
            total = z.p_Pa[0] / (sg.BOLTZMANN_J_K * z.T[0]) * 1e-6
            dry = 1.0 - z.x_H2O[0]
            up = np.zeros(17)
            up[sg.AIR_N2], up[sg.AIR_O2], up[sg.AIR_H2O] = total * dry * 0.79, total * dry * 0.21, total * z.x_H2O[0]
        else:
            up = y[:, i - 1].copy()
        y[:, i] = y[:, i] + a * (up - y[:, i])


def host_driver(z, pulsed, steps, dt, chained=False, residence_s=0.0):
    t = 0.0
    for _ in range(steps):
        t0, t1 = t, t + dt
        sg.dbd_prepare_source(z, pulsed, t0, t1)
        O.Mechanism.air().advance("rodas3", O.control(**CTL), z.as_dict(), z.padded, 0, z.padded, dt, 0, 1)
        sg.dbd_commit_pulses(z)
        if chained:
            flow_exchange_host(z, residence_s, dt)
        t = t1


@pytest.mark.parametrize("pulsed,chained", [(True, False), (False, False), (False, True), (True, True)],
                         ids=["pulsed", "averaged", "averaged-chained", "pulsed-chained"])
def test_host_driver_matches_reference_driver(oracle_lib, pulsed, chained):
    a = zones()
    b = a.copy()
    b.pulse_index = a.pulse_index.copy()
    for name in ("T", "x_H2O", "power", "freq", "p_Pa"):
        setattr(b, name, getattr(a, name))
    host_driver(a, pulsed, 4, 1e-3, chained, residence_s=0.5)
    blk = sg.dbd_block(b)
    O.ref_dbd_run(blk, b.cells, b.padded, pulsed, 4, 1e-3, O.control(**CTL), chained, 0.5)
    ref = blk[: a.rows]
    assert ref.tobytes() == a.block.tobytes()
    assert blk[a.rows].tobytes() == a.pulse_index.tobytes()   # the pulse clock
    if pulsed:
        assert a["pulses"].min() > 0
