"""The reference's own GPU test against this module.

oracle/_ref/ref_gpu_tests is the reference's test translation unit
(tests/test_kinetics.cpp) compiled from the reference sources, running its
test_gpu (test_kinetics.cpp:1086-1243) with the reference's own module loader
(platform/linux_gpu.cpp:7-31) pointed at libsimstack_gpu.so. Its checks, all bit
for bit against the reference's CPU lanes on this host:
  - FP64 lanes, pulsed and averaged discharge, 12 zones x 5 x 1 ms;
  - f32 lanes (precision 1), both modes, 16 zones x 5 ms;
  - ten 20 ms steps with an upload every step, FP64 and f32, 64 zones;
  - warp per zone (gpu_kin_set_mode(1)), both precisions and modes, 24 zones;
  - the hybrid driver dbd_advance_hybrid (dbd.cpp:336-463): lanes split
    0/8/24/40/64 of 64 zones between this module (gpu_kin_advance_async +
    gpu_kin_wait on a page-locked block) and the reference's threaded CPU path.
The executable is built by `make -C oracle ref` wherever the reference sources
are present (the staged copy travels with the working tree)."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "oracle", "_ref", "ref_gpu_tests")

EXPECTED = [
    "pulsed  , 12 zones x 5 ms: CUDA vs AVX2 bit-identical",
    "averaged, 12 zones x 5 ms: CUDA vs AVX2 bit-identical",
    "pulsed  , 16 zones x 5 ms, f32 lanes: CUDA vs AVX2 bit-identical",
    "averaged, 16 zones x 5 ms, f32 lanes: CUDA vs AVX2 bit-identical",
    "f64 lanes, 64 zones x 10 x 20 ms (upload every step): CUDA vs AVX2 bit-identical",
    "f32 lanes, 64 zones x 10 x 20 ms (upload every step): CUDA vs AVX2 bit-identical",
    "warp per zone, f64 lanes, pulsed  , 24 zones x 5 ms: CUDA vs AVX2 bit-identical",
    "warp per zone, f64 lanes, averaged, 24 zones x 5 ms: CUDA vs AVX2 bit-identical",
    "warp per zone, f32 lanes, pulsed  , 24 zones x 5 ms: CUDA vs AVX2 bit-identical",
    "warp per zone, f32 lanes, averaged, 24 zones x 5 ms: CUDA vs AVX2 bit-identical",
    "hybrid CUDA+CPU, f64 lanes, splits 0/8/24/40/64 of 64 zones: all bit-identical to the CPU",
    "hybrid CUDA+CPU, f32 lanes, splits 0/8/24/40/64 of 64 zones: all bit-identical to the CPU",
]


def test_reference_gpu_suite_passes_against_this_module():
    if not os.path.exists(EXE):
        pytest.skip("reference sources not present: oracle/_ref/ref_gpu_tests was not built")
    r = subprocess.run([EXE], capture_output=True, text=True, timeout=900, cwd=os.path.dirname(EXE))
    out = r.stdout + r.stderr
    assert r.returncode == 0, out
    for line in EXPECTED:
        assert line in out, f"missing: {line}\n{out}"
    assert " 0 failed" in out, out
