"""gpu_kin_advance_noalloc: the advance for callers that cannot allocate device
memory (a caller whose device memory all belongs to its own arena, a caller
recording into a CUDA graph, a real-time loop that may not synchronise the
device). It keeps the work queue's scratch in a static device array instead of
module-allocated memory, so it must produce exactly what the regular
persistent-queue entry point (gpu_kin_advance_queue) produces.

This file is named to be collected last: if it fails, a run that stops at the
first failure has already run every other test. It passes on its own in a
fresh process and after the other tests alike (it initialises the module
itself and restores nothing it does not own).
"""
import ctypes as C

import numpy as np
import pytest

import simstack_gb300 as sg

pytestmark = pytest.mark.gpu

OUT = ("y", "h", "steps", "rejects", "pulses", "failed")


def _advance_twice_noalloc(z, km, meth, ctl, base, precision, duration):
    L = sg.lib()
    for _ in range(2):   # two calls in a row: the second starts from the first one's state
        launch = z.launch(base, precision, duration)
        rc = L.gpu_kin_advance_noalloc(C.byref(km), C.byref(meth), C.byref(ctl), C.byref(launch), None, 1)
        assert rc == 0, L.gpu_error_string(rc).decode()


def _advance_twice_queue(z, base, precision, duration):
    L = sg.lib()
    for _ in range(2):
        launch = z.launch(base, precision, duration)
        ms = C.c_float()
        rc = L.gpu_kin_advance_queue(C.byref(launch), C.byref(ms))
        assert rc == 0, L.gpu_error_string(rc).decode()


@pytest.mark.parametrize("method,precision", [("rodas3", 0), ("rodas3", 2), ("ros3", 0)],
                         ids=["generated-f64", "generated-mixed", "table-f64"])
def test_noalloc_matches_queue_entry_point(method, precision):
    """Same outputs, bit for bit (the FP64 and mixed paths are deterministic), as
    gpu_kin_advance_queue on the same zone block, over two consecutive calls."""
    mod = sg.Module(0, 256 << 20)
    km, meth, ctl = sg.Model.air().kinmech(), sg.method(method), sg.control()
    mod.set_mech(km, meth, ctl)
    z0 = sg.air_cells(3000, seed=17)
    a, b = z0.copy(), z0.copy()
    base_a = mod.upload(a)
    base_b = mod.upload(b)
    used_before = sg.lib().gpu_arena_used()
    _advance_twice_noalloc(a, km, meth, ctl, base_a, precision, 0.5)
    assert sg.lib().gpu_arena_used() == used_before   # it takes nothing from the module's arena either
    _advance_twice_queue(b, base_b, precision, 0.5)
    mod.download(a, base_a)
    mod.download(b, base_b)
    for name in OUT:
        assert a[name].tobytes() == b[name].tobytes(), f"{name} differs"
    assert a["steps"].min() > 0
