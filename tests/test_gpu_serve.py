"""Film advection and the serving engine against the oracle (chemistry by the
oracle's restatement of the reference's solver, advection by its FP64
restatement of the upwind formula of src/sim/nft.cpp:1066-1079), bit for bit;
plus the engine's own guarantees: a request's result is the same alone and in
a mix, admission respects the HBM budget, cancellation."""
import ctypes as C

import numpy as np
import pytest

import simstack_gb300 as sg

pytestmark = pytest.mark.gpu


def oracle_coupled(O, z, cells, channel_cells, steps, courant, substeps, method="rodas3", precision=0, mech=None):
    """The served computation on the CPU: per coupling step, chemistry over 1 s
    on cells [0, cells), then upwind advection of every channel (inlet = the
    request's cell-0 initial state)."""
    mech = mech if mech is not None else O.Mechanism.air()
    ctl = O.control()
    inlet = np.array(z["y"][:, 0])
    for _ in range(steps):
        if precision == 2:   # the module's current mixed variant
            O.advance_mixed(mech, method, ctl, z.as_dict(), z.padded, 0, cells, 1.0, sweeps=1,
                            variant=int(sg.lib().gpu_kin_get_mixed_variant()))
        else:
            mech.advance(method, ctl, z.as_dict(), z.padded, 0, cells, 1.0, precision, 1)
        y = z["y"]
        for b in range(0, cells, channel_cells):
            e = min(cells, b + channel_cells)
            row = np.ascontiguousarray(y[:, b:e])
            O.advect(row, inlet, courant, substeps)
            y[:, b:e] = row


def test_advect_matches_oracle(module, oracle_lib):
    species, cells, cc, padded = 5, 1000, 256, 1024
    rng = np.random.default_rng(4)
    x = rng.uniform(0.0, 1e15, size=(species, padded))
    inlet = rng.uniform(0.0, 1e15, size=species)
    dev = module.alloc(x.nbytes)
    dinlet = module.alloc(inlet.nbytes)
    L = sg.lib()
    sg.check(L.gpu_copy_to_device(dev, x.ctypes.data, x.nbytes), "copy")
    sg.check(L.gpu_copy_to_device(dinlet, inlet.ctypes.data, inlet.nbytes), "copy")
    courant, substeps = 0.1 * (1.0 / 3) / 0.05, 3
    sg.check(L.gpu_advect(dev, padded, species, cells, cc, dinlet, courant, substeps, L.gpu_stream()), "gpu_advect")
    sg.check(L.gpu_sync(), "gpu_sync")
    got = np.zeros_like(x)
    sg.check(L.gpu_copy_to_host(got.ctypes.data, dev, x.nbytes), "copy")
    want = x.copy()
    for b in range(0, cells, cc):
        row = np.ascontiguousarray(want[:, b:min(cells, b + cc)])
        oracle_lib.advect(row, inlet, courant, substeps)
        want[:, b:min(cells, b + cc)] = row
    assert got.tobytes() == want.tobytes()   # columns >= cells untouched too
    module.reset_arena()


@pytest.mark.parametrize("precision", [0, 2])
def test_served_request_matches_oracle(oracle_lib, precision):
    cells, cc, steps, v = 700, 256, 3, 0.1
    z = sg.air_cells(cells, seed=21)
    with sg.Server() as srv:
        rid = srv.submit(z["y"][:, :cells], z["k"][:, :cells], steps, cc, v, precision=precision)
        srv.drain(timeout_s=300)
        st = srv.poll(rid)
        assert st["state"] == "done" and st["steps_completed"] == steps, st
        assert st["substeps"] == 3 and st["latency_s"] >= st["admit_s"] >= 0.0
        y, nsteps, failed = srv.result(rid)
    ref = z.copy()
    oracle_coupled(oracle_lib, ref, cells, cc, steps, st["courant"], st["substeps"], precision=precision)
    assert y.tobytes() == np.ascontiguousarray(ref["y"][:, :cells]).tobytes()
    assert nsteps.tobytes() == np.ascontiguousarray(ref["steps"][:cells]).tobytes()
    assert not failed.any()


def test_served_table_mechanism(oracle_lib):
    """mechanism = 1: the table-driven kernels (here the shipped mechanism's
    tables with Ros3, which the generated code does not cover)."""
    cells, cc, steps, v = 300, 128, 2, 0.04
    z = sg.air_cells(cells, seed=22)
    with sg.Server() as srv:
        srv.set_mech(sg.Model.air().kinmech(), sg.method("ros3"))
        rid = srv.submit(z["y"][:, :cells], z["k"][:, :cells], steps, cc, v, mechanism=1)
        srv.drain(timeout_s=300)
        st = srv.poll(rid)
        assert st["state"] == "done", st
        y, nsteps, _ = srv.result(rid)
    ref = z.copy()
    oracle_coupled(oracle_lib, ref, cells, cc, steps, st["courant"], st["substeps"], method="ros3")
    assert y.tobytes() == np.ascontiguousarray(ref["y"][:, :cells]).tobytes()
    assert nsteps.tobytes() == np.ascontiguousarray(ref["steps"][:cells]).tobytes()


MIX = [  # (cells, channel_cells, coupling steps, v, precision, seed)
    (1024, 256, 2, 0.05, 0, 31),
    (3000, 1024, 1, 0.1, 2, 32),
    (257, 4096, 3, 0.01, 0, 33),
    (2048, 512, 2, 0.08, 2, 34),
]


def serve_all(reqs, budget=0):
    out = []
    with sg.Server(budget) as srv:
        ids = []
        for cells, cc, steps, v, prec, seed in reqs:
            z = sg.air_cells(cells, seed=seed)
            ids.append(srv.submit(z["y"][:, :cells], z["k"][:, :cells], steps, cc, v, precision=prec))
        max_running = 0
        import time
        t_end = time.monotonic() + 300
        while True:
            running, waiting, _ = srv.progress()
            max_running = max(max_running, running)
            if running == 0 and waiting == 0:
                break
            assert time.monotonic() < t_end
            time.sleep(2e-4)
        for rid in ids:
            assert srv.poll(rid)["state"] == "done"
            out.append(srv.result(rid))
        stats = srv.stats()
    return out, max_running, stats


def test_same_alone_and_in_the_mix():
    together, max_running, stats = serve_all(MIX)
    assert max_running >= 2 and stats["graph_launches"] == sum(r[2] for r in MIX)
    for req, got in zip(MIX, together):
        alone, _, _ = serve_all([req])
        for a, b in zip(alone[0], got):
            assert a.tobytes() == b.tobytes()


def test_admission_respects_budget():
    # footprint of a 1,024-cell shipped-mechanism request: 103 rows of 1,024 doubles, inlet, queue header, table image
    one = 103 * 1024 * 8 + 17 * 8 + 256 + 30112
    reqs = [(1024, 256, 1, 0.05, 0, 40 + i) for i in range(4)]
    _, max_running, stats = serve_all(reqs, budget=one + one // 2)
    assert max_running == 1 and stats["peak_bytes"] <= stats["budget_bytes"]
    with sg.Server(one) as srv:   # a request that could never fit is refused at submit
        z = sg.air_cells(2048, seed=1)
        with pytest.raises(sg.GpuError) as e:
            srv.submit(z["y"][:, :2048], z["k"][:, :2048], 1, 256, 0.05)
        assert e.value.code == 2   # cudaErrorMemoryAllocation


def test_cancel_waiting_and_running():
    z = sg.air_cells(1024, seed=50)
    one = 103 * 1024 * 8 + 17 * 8 + 256 + 30112
    with sg.Server(one) as srv:
        a = srv.submit(z["y"], z["k"], 50, 256, 0.05)
        b = srv.submit(z["y"], z["k"], 50, 256, 0.05)
        srv.progress()                        # a admitted, b waits for memory
        assert srv.poll(a)["state"] == "running" and srv.poll(b)["state"] == "waiting"
        srv.cancel(b)
        assert srv.poll(b)["state"] == "cancelled"
        srv.cancel(a)
        srv.drain(timeout_s=120)
        sa = srv.poll(a)
        assert sa["state"] == "cancelled" and sa["steps_completed"] < 50
        assert srv.stats()["in_use_bytes"] == 0
        with pytest.raises(sg.GpuError):
            srv.result(a)


def test_invalid_requests():
    z = sg.air_cells(64, seed=1)
    with sg.Server() as srv:
        bad = [dict(channel_cells=0), dict(channel_cells=5000), dict(dt=0.0), dict(velocity_m_s=-1.0),
               dict(precision=3), dict(mechanism=2), dict(coupling_steps=0)]
        for kw in bad:
            args = dict(coupling_steps=1, channel_cells=64, velocity_m_s=0.05)
            args.update(kw)
            with pytest.raises(sg.GpuError):
                srv.submit(z["y"][:, :64], z["k"][:, :64], **args)
        assert srv.stats()["waiting"] == 0


@pytest.mark.parametrize("precision", [0, 2])
def test_served_large_mechanism(oracle_lib, precision):
    """mechanism = 2: a 60-species / 300-reaction synthetic mechanism through the
    cooperative kernel inside the coupling graph; FP64 bit for bit against the
    oracle's coupled computation, mixed within tolerance. The engine keeps its
    default control (the shipped mechanism's atol in molecules/cm^3); the large
    mechanism's requests run under the control given with it (atol 1e-12 in its
    own units), which the bit-for-bit comparison checks."""
    pm = sg.Model.synthetic(seed=7, species=60, reactions=300, bimolecular=0.7, products=1)
    om = oracle_lib.Mechanism()
    for s in range(60):
        om.add_species(f"S{s}", True)
    for r in range(pm.R):
        om.add_reaction(sg.model_equation(pm, r), "arr", (float(pm.k_const[r]), 0.0, 0.0))
    om.finalize()
    cells, cc, steps, v = 40, 16, 2, 0.05
    z = sg.synthetic_cells(pm, cells, seed=8)
    ctl = sg.control(rtol=1e-4, atol=1e-12, max_steps=200000)
    with sg.Server(0) as srv:
        srv.set_coop_mech(pm, sg.method("rodas3"), ctl)
        rid = srv.submit(z["y"][:, :cells], z["k"][:, :cells], steps, cc, v, precision=precision, mechanism=2)
        srv.drain(timeout_s=300)
        st = srv.poll(rid)
        assert st["state"] == "done", st
        y, nsteps, failed = srv.result(rid)
    ref = z.copy()
    inlet = np.array(ref["y"][:, 0])
    octl = oracle_lib.control(rtol=1e-4, atol=1e-12, max_steps=200000)
    for _ in range(steps):
        om.advance("rodas3", octl, ref.as_dict(), ref.padded, 0, cells, 1.0, 0, 1)
        for b in range(0, cells, cc):
            e = min(cells, b + cc)
            row = np.ascontiguousarray(ref["y"][:, b:e])
            oracle_lib.advect(row, inlet, st["courant"], st["substeps"])
            ref["y"][:, b:e] = row
    want = np.ascontiguousarray(ref["y"][:, :cells])
    assert not failed.any()
    if precision == 0:
        assert y.tobytes() == want.tobytes()
        assert nsteps.tobytes() == np.ascontiguousarray(ref["steps"][:cells]).tobytes()
    else:
        sig = want >= 1e-9 * want.sum(axis=0)
        rel = np.abs(y - want)[sig] / want[sig]
        assert rel.max() < 1e-6, rel.max()
