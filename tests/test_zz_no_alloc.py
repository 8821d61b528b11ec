"""gpu_kin_advance_noalloc: the advance for callers that cannot allocate device
memory (a caller whose device memory all belongs to its own arena, or a
real-time loop that may not take cudaMalloc's device-wide synchronisation). It
keeps the work queue's scratch in a static device array instead of
module-allocated memory, and launches the same kernel at the same shape as the
regular persistent-queue entry point (gpu_kin_advance_queue), so it must
produce exactly what that entry point produces.

This file is named to be collected last: if it fails, a run that stops at the
first failure has already run every other test. It passes on its own in a
fresh process and after the other tests alike (it initialises the module
itself and restores every module setting it changes).
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

import simstack_gb300 as sg

pytestmark = pytest.mark.gpu

OUT = ("y", "h", "steps", "rejects", "pulses", "failed")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_ERROR_TIMEOUT = 909
CUDA_ERROR_LAUNCH_OUT_OF_RESOURCES = 701


def _advance_twice_noalloc(z, km, meth, ctl, base, precision, duration, stream=None, wait=1):
    L = sg.lib()
    for _ in range(2):   # two calls in a row: the second starts from the first one's state
        launch = z.launch(base, precision, duration)
        rc = L.gpu_kin_advance_noalloc(C.byref(km), C.byref(meth), C.byref(ctl), C.byref(launch), stream, wait)
        assert rc == 0, L.gpu_error_string(rc).decode()


def _advance_twice_queue(z, base, precision, duration):
    L = sg.lib()
    for _ in range(2):
        launch = z.launch(base, precision, duration)
        ms = C.c_float()
        rc = L.gpu_kin_advance_queue(C.byref(launch), C.byref(ms))
        assert rc == 0, L.gpu_error_string(rc).decode()


TABLE_FRAME_BYTES = 10752   # the table-driven kernels' largest per-thread frame (the generated ones fit gpu_init's 3,840)


def _setup(method):
    mod = sg.Module(0, 256 << 20)
    km, meth, ctl = sg.Model.air().kinmech(), sg.method(method), sg.control()
    mod.set_mech(km, meth, ctl)
    if method != "rodas3":   # set-up for the table-driven kernels: a stack reservation that covers their frame
        assert sg.lib().gpu_stack_limit(TABLE_FRAME_BYTES, None) == 0
    return mod, km, meth, ctl


@pytest.mark.parametrize("method,precision", [("rodas3", 0), ("rodas3", 2), ("ros3", 0), ("ros3", 2)],
                         ids=["generated-f64", "generated-mixed", "table-f64", "table-mixed"])
def test_noalloc_matches_queue_entry_point(method, precision):
    """Same outputs, bit for bit (both paths are deterministic), as
    gpu_kin_advance_queue on the same zone block, over two consecutive calls."""
    mod, km, meth, ctl = _setup(method)
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


def test_noalloc_on_a_caller_stream_without_waiting():
    """Enqueued on the caller's own stream with wait = 0, then synchronised by the
    caller: the same bits as the queue entry point."""
    torch = pytest.importorskip("torch")
    mod, km, meth, ctl = _setup("rodas3")
    z0 = sg.air_cells(2000, seed=23)
    a, b = z0.copy(), z0.copy()
    base_a, base_b = mod.upload(a), mod.upload(b)
    stream = torch.cuda.Stream()
    _advance_twice_noalloc(a, km, meth, ctl, base_a, 0, 0.5, stream=C.c_void_p(stream.cuda_stream), wait=0)
    stream.synchronize()
    _advance_twice_queue(b, base_b, 0, 0.5)
    mod.download(a, base_a)
    mod.download(b, base_b)
    for name in OUT:
        assert a[name].tobytes() == b[name].tobytes(), f"{name} differs"


def test_noalloc_reports_a_bounded_wait_that_ran_out():
    """The table path stages its tables with a bounded wait; with the poll limit at
    zero the wait gives up at once, the error flag in the static array is set, and
    the call returns cudaErrorTimeout with the zone block untouched. The next call
    clears the flag and runs normally."""
    mod, km, meth, ctl = _setup("ros3")
    z = sg.air_cells(1000, seed=29)
    base = mod.upload(z)
    before = z.copy()
    L = sg.lib()
    assert L.gpu_kin_set_wait_limit(0) == 0
    try:
        launch = z.launch(base, 0, 0.5)
        rc = L.gpu_kin_advance_noalloc(C.byref(km), C.byref(meth), C.byref(ctl), C.byref(launch), None, 1)
        assert rc == CUDA_ERROR_TIMEOUT, L.gpu_error_string(rc).decode()
    finally:
        L.gpu_kin_set_wait_limit(1 << 24)
    mod.download(z, base)
    for name in OUT:
        assert z[name].tobytes() == before[name].tobytes(), f"{name} was written"
    launch = z.launch(base, 0, 0.5)
    assert L.gpu_kin_advance_noalloc(C.byref(km), C.byref(meth), C.byref(ctl), C.byref(launch), None, 1) == 0
    mod.download(z, base)
    assert z["steps"].min() > 0


_FRESH = r"""
import ctypes as C, sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
import simstack_gb300 as sg
L = sg.lib()
km, meth, ctl = sg.Model.air().kinmech(), sg.method("rodas3"), sg.control()
z = sg.air_cells(1500, seed=31)
dev = torch.from_numpy(z.block.copy()).cuda()          # the caller's own device memory
launch = z.launch(dev.data_ptr(), 0, 0.5)
# set-up: without gpu_init the stack reservation is the context's default, too small
rc = L.gpu_kin_advance_noalloc(C.byref(km), C.byref(meth), C.byref(ctl), C.byref(launch), None, 1)
first = rc
assert L.gpu_stack_limit(3840, None) == 0
for _ in range(2):
    rc = L.gpu_kin_advance_noalloc(C.byref(km), C.byref(meth), C.byref(ctl), C.byref(launch), None, 1)
    assert rc == 0, L.gpu_error_string(rc).decode()
np.save(sys.argv[2], dev.cpu().numpy())
print("first", first)
"""


def test_noalloc_in_a_fresh_process_without_gpu_init(tmp_path):
    """A process that never calls gpu_init: the first call refuses to launch until the
    stack reservation is set (instead of letting the driver grow it), then two calls
    give the queue entry point's bits."""
    pytest.importorskip("torch")
    out = tmp_path / "fresh.npy"
    r = subprocess.run([sys.executable, "-c", _FRESH, ROOT, str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert f"first {CUDA_ERROR_LAUNCH_OUT_OF_RESOURCES}" in r.stdout, r.stdout
    mod, km, meth, ctl = _setup("rodas3")
    z = sg.air_cells(1500, seed=31)
    base = mod.upload(z)
    _advance_twice_queue(z, base, 0, 0.5)
    mod.download(z, base)
    got = np.load(out)
    for name in OUT:
        r0 = z.row_offset[name]
        rows = z[name].reshape(-1, z.padded)
        assert got[r0:r0 + rows.shape[0]].tobytes() == rows.tobytes(), f"{name} differs"
