"""bench.py's command line and the algorithmic constants its roofline uses (no GPU): every named
workload parses and has its runner; the shipped mechanism's flops per Rodas3 step and HBM bytes
per cell-integration are the counts derived from the reference's tables (6,032 and 808); the
served request stream is seeded and within its stated ranges."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


@pytest.mark.parametrize("workload", list(bench.WORKLOADS))
def test_every_workload_parses(monkeypatch, workload):
    monkeypatch.setattr(sys, "argv", ["bench.py", "--workload", workload, "--steps", "2", "--warmup", "3"])
    a = bench.parse()
    assert a.workload == workload and a.steps == 2 and a.warmup == 3 and a.gpus == 1 and a.impl == "ours"


def test_defaults_are_the_headline(monkeypatch):
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench.parse()
    assert a.workload == "air-1048576x10s" and a.cells == 1 << 20 and a.duration == 10.0 and a.precision == "mixed"
    assert a.warmup >= 3


def test_runners_exist():
    for name in ("run_ours", "run_reference", "run_uneven_stiffness", "run_large_mechanism", "run_serving",
                 "run_profile_case", "run_dbd_sweep"):
        assert callable(getattr(bench, name))


def test_algorithmic_counts_of_the_shipped_mechanism():
    import simstack_gb300 as sg

    f = bench.flops_per_step(sg.Model.air())
    assert f["total"] == 6032 and f["executed_f64"] == 5639   # the FP64 path reuses f(y) at Rodas3's stage 2
    assert (f["fun"], f["neg_jac"], f["factor"], f["solve"]) == (393, 694, 1552, 409)
    assert bench.hbm_bytes_per_cell(17, 44) == 808


def test_mixed_error_definition():
    """Every entry counts; relative to max(|b|, atol); the filtered figure is reported beside it."""
    b = np.array([[1e12, 1e12], [1e3, 1e3]])
    a = b.copy()
    a[1, 0] += 6.02214076e8 * 1e-6   # a tiny species off by 1e-6 atol
    e = bench.mixed_errors(a, b)
    assert abs(e["max"] - 1e-6) < 1e-12 and e["max_species_above_1e-3_ppm"] == 0.0


def test_served_stream_is_seeded_and_in_range():
    a, b = bench.serve_sample(1, 48), bench.serve_sample(1, 48)
    assert a == b and len(a) == 48
    t = np.array([r["arrival_s"] for r in a])
    assert np.all(np.diff(t) > 0)
    assert all(1024 <= r["cells"] <= 65536 and 1 <= r["steps"] <= 600 and 256 <= r["channel_cells"] <= 4096
               and 0.01 <= r["velocity"] <= 0.1 for r in a)
    assert bench.serve_sample(2, 48) != a
