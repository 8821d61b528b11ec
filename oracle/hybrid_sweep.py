"""TEST AND BASELINE INFRASTRUCTURE -- NOT PART OF THE PRODUCT.

The reference's hybrid CPU+GPU zone driver (dbd_advance_hybrid, src/sim/dbd.cpp:336-463,
compiled from the reference sources into oracle/_ref/libref.so) running with this
repository's module, which the reference's own loader (platform/linux_gpu.cpp:7-31)
loads from simstack_gb300/libsimstack_gpu.so: the integration a maintainer gets by
dropping the module in. Each run is dbd_scene_step's sequence (dbd_scene.cpp:232-265):
host source, hybrid advance, pulse commit.

Runs in its own process (the loader calls gpu_init). Prints one JSON line per split
setting; --save writes the final zone blocks for bit comparisons.

    python -m oracle.hybrid_sweep --side 64 --pulsed --steps 12 --precision 1
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def sweep_zones(side: int):
    """The reference's DBD sweep grid: power 0.01-0.5 W/cm^3 (log) x H2O 0-4 %, 310 K, 10 kHz."""
    import simstack_gb300 as sg

    n = side * side
    fx = (np.arange(n) % side) / (side - 1)
    fy = (np.arange(n) // side) / (side - 1)
    return sg.dbd_zones(n, 310.0, 0.04 * fy, 0.01 * np.power(50.0, fx), 10000.0)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--side", type=int, default=64)
    ap.add_argument("--pulsed", action="store_true")
    ap.add_argument("--steps", type=int, default=12)
    ap.add_argument("--dt", type=float, default=0.02)
    ap.add_argument("--precision", type=int, default=1, choices=[0, 1])
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--splits", default="cpu,gpu,adaptive",
                    help="comma list: cpu (split 0), gpu (all lanes), adaptive (the driver's search), or a lane count")
    ap.add_argument("--save", default=None, help="directory for the final blocks (<split>.npy)")
    a = ap.parse_args(argv)
    sys.path.insert(0, ROOT)
    import simstack_gb300 as sg
    from oracle import oracle as O

    O.ref_gpu_load(sg.LIB_PATH, 1 << 30)
    ctl = O.control(rtol=1e-3, atol=1e8, h_min=1e-14, h_start=1e-9, max_steps=20000)
    for name in a.splits.split(","):
        z = sweep_zones(a.side)
        blk = sg.dbd_block(z)
        force = {"cpu": 0, "gpu": z.padded, "adaptive": -1}.get(name)
        force = int(name) if force is None else force
        split, step_ms, gpu_ms = O.ref_dbd_hybrid_run(blk, z.cells, z.padded, a.pulsed, a.steps, a.dt, ctl, a.threads,
                                                      a.precision, force_split=force)
        tail = max(1, a.steps // 2)   # the second half: past the adaptive search's start-up probes
        rec = {"split": name, "zones": z.cells, "mode": "pulsed" if a.pulsed else "averaged", "dt": a.dt,
               "steps": a.steps, "precision": a.precision, "threads": a.threads,
               "sim_s_per_wall_s": a.steps * a.dt / (float(step_ms.sum()) * 1e-3),
               "sim_s_per_wall_s_second_half": tail * a.dt / (float(step_ms[-tail:].sum()) * 1e-3),
               "lanes_on_gpu": [int(v) for v in split], "step_ms": [round(float(v), 3) for v in step_ms],
               "gpu_ms": [round(float(v), 3) for v in gpu_ms]}
        print(json.dumps(rec), flush=True)
        if a.save:
            os.makedirs(a.save, exist_ok=True)
            np.save(os.path.join(a.save, f"{name}.npy"), blk)
    return 0


if __name__ == "__main__":
    sys.exit(main())
