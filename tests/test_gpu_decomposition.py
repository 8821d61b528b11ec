"""The cells-per-warp axis: the reference's warp-per-cell mode (gpu_kin_set_mode(1),
src/gpu/gpu_api.h:108-110) and the cooperative decomposition as tuning kind 3 (one cell
per CTA of 32..256 threads). FP64 keeps the reference's bits whatever the decomposition;
the mixed path stays within its 1e-5 bound; the autotuner's kind 4 chooses among the
lane kernels and the cooperative shapes by measurement."""
import numpy as np
import pytest

import simstack_gb300 as sg

from test_gpu_parity import MIXED_BOUND, assert_bits, mixed_errors, oracle_run

pytestmark = pytest.mark.gpu


@pytest.fixture
def restore_tuning(module):
    yield
    sg.lib().gpu_kin_set_mode(0)
    module.set_tuning()


def test_warp_per_cell_mode_keeps_the_bits(module, oracle_lib, restore_tuning):
    module.set_mech(sg.Model.air().kinmech(), sg.method("rodas3"), sg.control())
    assert sg.lib().gpu_kin_set_mode(1) == 0
    z = sg.air_cells(512, seed=21)
    ref = z.copy()
    module.integrate(z, 1.0, precision=0)
    oracle_run(oracle_lib, ref, 1.0)
    assert_bits(z, ref)


@pytest.mark.parametrize("block", [32, 64, 128])
def test_cooperative_kind_keeps_the_bits(module, oracle_lib, restore_tuning, block):
    module.set_mech(sg.Model.air().kinmech(), sg.method("rodas3"), sg.control())
    module.set_tuning(kind=3, block=block, variant=0, ctas_per_sm=0)
    z = sg.air_cells(600, seed=22)
    ref = z.copy()
    module.integrate(z, 1.0, precision=0)
    oracle_run(oracle_lib, ref, 1.0)
    assert_bits(z, ref)


def test_cooperative_mixed_within_bound(module, oracle_lib, restore_tuning):
    module.set_mech(sg.Model.air().kinmech(), sg.method("rodas3"), sg.control())
    module.set_tuning(kind=3, block=64, variant=0, ctas_per_sm=0)
    z = sg.air_cells(600, seed=23)
    ref = z.copy()
    module.integrate(z, 1.0, precision=2)
    oracle_run(oracle_lib, ref, 1.0)
    _, floored = mixed_errors(z, ref)
    assert floored.max() <= MIXED_BOUND, floored.max()


def test_autotune_across_decompositions(module, restore_tuning):
    module.set_mech(sg.Model.air().kinmech(), sg.method("rodas3"), sg.control())
    z = sg.air_cells(4096, seed=24)
    base = module.upload(z)
    t = module.autotune(z.launch(base, 0, 0.2), kind=4)
    assert t.kind in (2, 3) and t.ms > 0
    after = z.copy()
    module.download(after, base)
    assert after["y"].tobytes() == z["y"].tobytes()   # the caller's block is restored
    module.reset_arena()
