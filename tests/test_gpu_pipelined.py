"""gpu_kin_advance_pipelined: the host-buffer advance with the zone block split
into lane chunks whose uploads, kernels and downloads overlap. Every cell's
result is the one the plain upload / advance / download gives (src/sim/dbd.cpp:272-295
is the reference's host-buffer call sequence)."""
import numpy as np
import pytest

import simstack_gb300 as sg

pytestmark = pytest.mark.gpu

FIELDS = ("y", "h", "steps", "rejects", "pulses", "failed")


@pytest.mark.parametrize("precision", [0, 2])
@pytest.mark.parametrize("chunks", [1, 3, 16])
def test_pipelined_same_bits_as_plain(module, precision, chunks):
    """1,000 cells (not a multiple of the chunk count; the padded lanes beyond them are not
    integrated by the pipelined call) x 0.5 s."""
    module.set_mech(sg.Model.air().kinmech(), sg.method("rodas3"), sg.control())
    z = sg.air_cells(1000, seed=21)
    ref = z.copy()
    module.integrate(ref, 0.5, precision=precision)
    base = module.alloc(z.nbytes)
    ms = module.integrate_pipelined(z, 0.5, precision=precision, chunks=chunks, device_base=base)
    assert ms > 0.0
    for name in FIELDS:
        a, b = z[name][..., :1000], ref[name][..., :1000]
        assert a.tobytes() == b.tobytes(), f"{name}: {np.count_nonzero(a != b)} differ"


def test_pipelined_matches_oracle_f64(module, oracle_lib):
    module.set_mech(sg.Model.air().kinmech(), sg.method("rodas3"), sg.control())
    z = sg.air_cells(700, seed=22)
    ref = z.copy()
    module.integrate_pipelined(z, 1.0, precision=0, chunks=4)
    oracle_lib.Mechanism.air().advance("rodas3", oracle_lib.control(), ref.as_dict(), ref.padded, 0, ref.padded, 1.0, 0, 0)
    for name in FIELDS:
        assert z[name][..., :700].tobytes() == ref[name][..., :700].tobytes(), name


def test_pipelined_rejects_bad_arguments(module):
    module.set_mech(sg.Model.air().kinmech(), sg.method("rodas3"), sg.control())
    z = sg.air_cells(64, seed=23)
    for chunks in (0, 17):
        with pytest.raises(sg.GpuError):
            module.integrate_pipelined(z, 0.1, precision=0, chunks=chunks)


def test_pipelined_f64_concurrent_chunks(module, oracle_lib):
    """With the straggler hand-off off, FP64 chunk kernels also run on two streams at once."""
    module.set_mech(sg.Model.air().kinmech(), sg.method("rodas3"), sg.control())
    module.set_straggler_budget(0)
    try:
        z = sg.air_cells(900, seed=24)
        ref = z.copy()
        module.integrate_pipelined(z, 1.0, precision=0, chunks=5)
    finally:
        module.set_straggler_budget(sg.DEFAULT_STRAGGLER_BUDGET)
    oracle_lib.Mechanism.air().advance("rodas3", oracle_lib.control(), ref.as_dict(), ref.padded, 0, ref.padded, 1.0, 0, 0)
    for name in FIELDS:
        assert z[name][..., :900].tobytes() == ref[name][..., :900].tobytes(), name
