"""Bounded device waits give up with an error status, never a hang or a fault.

The table-driven kernels stage a mechanism's tables into shared memory with a
TMA bulk copy and wait for it on an mbarrier with a poll limit. With the limit
set to zero (gpu_kin_set_wait_limit) every such wait gives up at once: the CTA
lets its copy land, records the error flag and returns before touching a lane,
and the advance returns cudaErrorTimeout. Nothing faults, and the context
stays usable: the next advance at the normal limit runs as usual."""
import ctypes as C

import pytest

import simstack_gb300 as sg

pytestmark = pytest.mark.gpu

CUDA_ERROR_TIMEOUT = 909
OUT = ("y", "h", "steps", "rejects", "pulses", "failed")


@pytest.mark.parametrize("precision", [0, 2])
@pytest.mark.parametrize("entry", ["gpu_kin_advance", "gpu_kin_advance_queue"])
def test_timeout_returns_error_and_leaves_block_untouched(module, precision, entry):
    module.set_mech(sg.Model.air().kinmech(), sg.method("ros3"), sg.control())   # ros3: table-driven kernels
    z = sg.air_cells(700, seed=41)
    base = module.upload(z)
    before = z.copy()
    L = sg.lib()
    ms = C.c_float()
    assert L.gpu_kin_set_wait_limit(0) == 0
    try:
        rc = getattr(L, entry)(C.byref(z.launch(base, precision, 0.25)), C.byref(ms))
    finally:
        L.gpu_kin_set_wait_limit(1 << 24)
    assert rc == CUDA_ERROR_TIMEOUT, L.gpu_error_string(rc).decode()
    module.download(z, base)
    for name in OUT:
        assert z[name].tobytes() == before[name].tobytes(), f"{name} was written"
    # the context is still usable and the flag was cleared: a normal advance succeeds
    rc = getattr(L, entry)(C.byref(z.launch(base, precision, 0.25)), C.byref(ms))
    assert rc == 0, L.gpu_error_string(rc).decode()
    module.download(z, base)
    assert z["steps"][:700].min() > 0
    module.set_mech(sg.Model.air().kinmech(), sg.method("rodas3"), sg.control())
