"""The served workload's large mechanism needs its own step control (CPU, oracle).

The serving engine integrates every request of a mechanism under one KinControl. The
shipped mechanism's absolute tolerance is 6.022e8 molecules/cm^3 (1e-12 mol/L); the
200-species synthetic mechanism works in its own units (concentrations 1e-10 .. 1e-3),
where that atol leaves some cells to the step limit. The benchmark therefore gives the
large mechanism its own control (gpu_serve_set_coop_mech), the one its own workload
uses. This test pins both facts on a served request's cells with the oracle (the
reference's FP64 algorithm), so that a change of either control shows up here.
"""
import numpy as np

import bench
import simstack_gb300 as sg
from oracle import oracle as O


def _large_mechanism():
    big = sg.Model.synthetic(seed=1, species=200, reactions=1200, bimolecular=0.7, products=1)
    om = O.Mechanism()
    for sp in range(big.n):
        om.add_species(f"S{sp}", True)
    for r in range(big.R):
        om.add_reaction(sg.model_equation(big, r), "arr", (float(big.k_const[r]), 0.0, 0.0))
    om.finalize()
    return big, om


def test_large_mechanism_needs_its_own_control():
    big, om = _large_mechanism()
    req = bench.serve_sample(1, 48)[2]   # a 200-species request of the served stream
    assert req["mechanism"] == 2
    cap = 3000
    cells = 32                           # cell 30 is one that the shipped control leaves to the cap
    attempts = {}
    for name, ctl in (("shipped", O.control(max_steps=cap)),
                      ("own", O.control(**dict(bench.MECH200_CONTROL, max_steps=cap)))):
        z = sg.synthetic_cells(big, cells, seed=req["seed"])
        om.advance("rodas3", ctl, z.as_dict(), z.padded, 0, cells, 1.0, 0, 8)
        attempts[name] = (z["steps"][:cells] + z["rejects"][:cells], z["failed"][:cells])
    steps, failed = attempts["shipped"]
    assert failed.any() and steps.max() == cap
    steps, failed = attempts["own"]
    assert not failed.any() and steps.max() < cap / 4
