"""The DBD zone driver on the device (gpu_dbd_*): source and pulse schedule, advance,
pulse commit and plug flow as kernels over a zone block that stays in device memory
-- uploaded once, never between master steps -- against the reference's own zone
driver (ref_dbd_run, where oracle/_ref is built) or the host restatement that
tests/test_cpu_dbd_driver.py pins to it: bit for bit, FP64 lanes and f32 Delta lanes,
and the mixed path against its model."""
import ctypes as C

import numpy as np
import pytest

import simstack_gb300 as sg
from oracle import oracle as O

from test_cpu_dbd_driver import CTL, flow_exchange_host, zones

pytestmark = pytest.mark.gpu


def host_driver(z, pulsed, steps, dt, precision, chained, residence_s, variant):
    t = 0.0
    for _ in range(steps):
        t0, t1 = t, t + dt
        sg.dbd_prepare_source(z, pulsed, t0, t1)
        if precision == 2:
            O.advance_mixed(O.Mechanism.air(), "rodas3", O.control(**CTL), z.as_dict(), z.padded, 0, z.padded, dt,
                            sweeps=1, variant=variant)
        else:
            O.Mechanism.air().advance("rodas3", O.control(**CTL), z.as_dict(), z.padded, 0, z.padded, dt, precision, 1)
        sg.dbd_commit_pulses(z)
        if chained:
            flow_exchange_host(z, residence_s, dt)
        t = t1


@pytest.mark.parametrize("precision", [0, 1, 2], ids=["f64", "f32-delta", "mixed"])
@pytest.mark.parametrize("pulsed,chained", [(True, False), (False, False), (False, True), (True, True)],
                         ids=["pulsed", "averaged", "averaged-chained", "pulsed-chained"])
def test_device_driver_matches_host_driver(module, pulsed, chained, precision):
    module.set_mech(sg.Model.air().kinmech(), sg.method("rodas3"), sg.control(**CTL))
    steps, dt, residence = 5, 1e-3, 0.5
    a = zones()
    b = zones()
    dev = sg.DeviceZones(module, a)
    t = 0.0
    for _ in range(steps):
        dev.step(t, dt, pulsed, precision=precision, chained=chained, residence_s=residence)
        t = t + dt
    got = dev.download()
    if precision == 0 and O.ref_available():   # the reference's own driver, end to end
        blk = sg.dbd_block(b)
        O.ref_dbd_run(blk, b.cells, b.padded, pulsed, steps, dt, O.control(**CTL), chained, residence)
        assert got[: b.rows + 1].tobytes() == blk[: b.rows + 1].tobytes()
    else:
        host_driver(b, pulsed, steps, dt, precision, chained, residence, module.mixed_variant())
        assert got[: b.rows].tobytes() == b.block.tobytes()
        assert got[b.rows].tobytes() == b.pulse_index.tobytes()
    if pulsed:
        assert got[b.row_offset["pulses"]].min() > 0
    module.reset_arena()


def test_device_driver_rejects_unstable_flow(module):
    module.set_mech(sg.Model.air().kinmech(), sg.method("rodas3"), sg.control(**CTL))
    dev = sg.DeviceZones(module, zones())
    L = sg.lib()
    # dt * zones / residence > 1: the explicit exchange would be unstable (dbd.cpp:472)
    assert L.gpu_dbd_flow_exchange(C.byref(dev.g), 0.01, 1e-3) != 0
    ms = C.c_float()
    assert L.gpu_dbd_step(C.byref(dev.g), None, 0, 0.0, 1e-3, 0, 1, 0.01, C.byref(ms)) != 0
    bad = sg.GpuDbdZones.from_buffer_copy(dev.g)
    bad.source_temp = None
    assert L.gpu_dbd_prepare_source(C.byref(bad), None, 1, 0.0, 1e-3) != 0
    module.reset_arena()
