"""The reference's hybrid CPU+GPU zone driver with this module (dbd.cpp:336-463).

dbd_advance_hybrid gives lanes [0, split) to the module (gpu_kin_advance_async on a
page-locked block, gpu_kin_wait) while the reference's threaded CPU path takes
[split, padded). The reference's rule: the result is bit-identical to either device
alone for ANY split, so the split can follow timings. Checked here for fixed splits and
for the driver's own measured search, FP64 and f32 lanes, against the reference's
CPU-only zone driver (oracle/_ref), on a 16 x 16 sweep grid. Each hybrid run is a child
process (oracle/hybrid_sweep.py), because the reference's loader calls gpu_init."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from oracle.hybrid_sweep import sweep_zones  # noqa: E402

import simstack_gb300 as sg  # noqa: E402

SIDE, STEPS, DT = 16, 6, 1e-3


@pytest.mark.parametrize("precision", [0, 1], ids=["f64", "f32"])
@pytest.mark.parametrize("pulsed", [True, False], ids=["pulsed", "averaged"])
def test_hybrid_splits_match_cpu_only_reference(tmp_path, precision, pulsed):
    if not O.ref_available():
        pytest.skip("reference sources not present: oracle/_ref was not built")
    splits = "0,8,64,136,256,adaptive"
    cmd = [sys.executable, "-m", "oracle.hybrid_sweep", "--side", str(SIDE), "--steps", str(STEPS), "--dt", str(DT),
           "--precision", str(precision), "--threads", "4", "--splits", splits, "--save", str(tmp_path)]
    if pulsed:
        cmd.append("--pulsed")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stdout + r.stderr
    runs = [json.loads(line) for line in r.stdout.splitlines() if line.startswith("{")]
    assert [x["split"] for x in runs] == splits.split(",")
    # the CPU-only reference zone driver on the same inputs
    z = sweep_zones(SIDE)
    ref = sg.dbd_block(z)
    O.ref_dbd_run(ref, z.cells, z.padded, pulsed, STEPS, DT,
                  O.control(rtol=1e-3, atol=1e8, h_min=1e-14, h_start=1e-9, max_steps=20000),
                  threads=4, f32_lanes=bool(precision))
    solver_rows = z.mutable_rows
    for name in splits.split(","):
        got = np.load(tmp_path / f"{name}.npy")
        assert got[:solver_rows].tobytes() == ref[:solver_rows].tobytes(), f"split {name}: solver rows differ"
        assert got.tobytes() == ref.tobytes(), f"split {name}: host rows differ"
    adaptive = runs[-1]["lanes_on_gpu"]
    # the driver's start-up: a CPU-only step, then GPU probes of 8 and padded/2 lanes
    assert adaptive[:3] == [0, 8, 128], adaptive
    for x in runs[:-1]:
        want = int(x["split"])
        assert set(x["lanes_on_gpu"]) == {want}
