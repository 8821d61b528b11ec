"""Host-side mechanism compiler (the module's kin_model_*) against the oracle's
restatement of the reference's builder, and the reference's numerical unit
tests (test_kinetics.cpp:44-211) run on the oracle. CPU only."""
import ctypes as C

import numpy as np
import pytest

import simstack_gb300 as sg


def both_synthetic(oracle_lib, seed, species, reactions, products=1):
    pm = sg.Model.synthetic(seed=seed, species=species, reactions=reactions, bimolecular=0.7, products=products)
    om = oracle_lib.Mechanism()
    for s in range(species):
        om.add_species(f"S{s}", True)
    for r in range(pm.R):
        om.add_reaction(sg.model_equation(pm, r), "arr", (float(pm.k_const[r]), 0.0, 0.0))
    om.finalize()
    return pm, om


@pytest.mark.parametrize("seed,species,reactions,products", [(1, 10, 30, 1), (2, 40, 150, 2), (3, 200, 1200, 1)])
def test_symbolic_phase_matches_oracle(oracle_lib, seed, species, reactions, products):
    """Same counts as the oracle's restatement (pattern, fill-in, op lists), up to
    the 200-species / 1,200-reaction synthetic mechanism."""
    pm, om = both_synthetic(oracle_lib, seed, species, reactions, products)
    pc, oc = pm.counts(), om.counts()
    for key, okey in (("n", "n"), ("R", "R"), ("nnz", "nnz"), ("divs", "pivots"), ("subs", "updates"), ("lower", "lower"),
                      ("upper", "upper")):
        assert pc[key] == oc[okey], key
    if species <= 32 and reactions <= 96:
        b, _ = om.kinmech()
        assert sg.kinmech_bytes(pm.kinmech()) == b


def test_synthetic_large_mechanism_fill(oracle_lib):
    """The 200-species synthetic mechanism: Jacobian fill before LU and after."""
    pm, om = both_synthetic(oracle_lib, 3, 200, 1200, 1)
    pat = om.pattern()
    fill_after = pat.mean()
    assert 0.5 < fill_after < 0.95   # the natural-order no-pivot LU fills most of the matrix
    c = pm.counts()
    assert c["subs"] > 1_000_000      # beyond the reference's u16 op tables (KIN_MAX_LU_SUB)


@pytest.mark.parametrize("equation,reason", [
    ("O + O2 -> O2 + O2", "element balance"),
    ("O + X -> O3", "unknown species"),
    ("O + O + O + O -> O2 + O2", "too many reactants"),
    ("-> O3", "needs reactants"),
])
def test_builder_rejects(oracle_lib, equation, reason):
    """The reference's builder rejects these (kin_build.cpp:100-148); so do both restatements."""
    pm = sg.Model.new()
    om = oracle_lib.Mechanism()
    for s in ("O", "O2", "O3"):
        pm.add_species(s)
        om.add_species(s)
    pm.add_reaction(equation)
    om.add_reaction(equation)
    assert reason in pm.error and reason in om.error


def test_reverse_must_follow_forward():
    pm = sg.Model.new()
    for s in ("N2O5", "NO2", "NO3"):
        pm.add_species(s)
    pm.add_reaction("N2O5 -> NO2 + NO3", "eqrev", (2.7e-27, 11000.0), ref=0)
    assert "reverse reaction must follow" in pm.error


def test_jacobian_vs_finite_differences(oracle_lib):
    """test_kinetics.cpp:61-102: analytic J vs central differences, < 1e-8 of row scale."""
    m = oracle_lib.Mechanism.air()
    n = 17
    T, total = 320.0, 101325.0 / (1.380649e-23 * 320.0) * 1e-6
    y = np.zeros(n)
    y[14], y[15], y[16] = total * 0.98 * 0.79, total * 0.98 * 0.21, total * 0.02
    for s in range(n):
        if y[s] == 0.0:
            y[s] = total * 1e-6 * (1.0 + 0.37 * s)
    k = m.rate_constants(T, total)
    jac = m.jac(k, y)
    pat = m.pattern()
    # map compact index -> (i, j)
    slot = -np.ones((n, n), int)
    idx = 0
    for i in range(n):
        for j in range(n):
            if pat[i, j]:
                slot[i, j] = idx
                idx += 1
    src = np.zeros(n)
    gross = np.zeros(n)
    for j in range(n):
        d = y[j] * 1e-4
        yp, ym = y.copy(), y.copy()
        yp[j] += d
        ym[j] -= d
        gross = np.maximum(gross, np.abs(m.fun(k, src, yp)))
    worst = 0.0
    for j in range(n):
        d = y[j] * 1e-4
        yp, ym = y.copy(), y.copy()
        yp[j] += d
        ym[j] -= d
        fd = (m.fun(k, src, yp) - m.fun(k, src, ym)) / (2 * d)
        for i in range(n):
            an = jac[slot[i, j]] if slot[i, j] >= 0 else 0.0
            worst = max(worst, abs(an - fd[i]) * y[j] / (gross[i] + 1e-300))
    assert worst < 1e-6


def test_sparse_lu_vs_dense(oracle_lib):
    """test_kinetics.cpp:105-148: no-pivot sparse solve vs dense partial-pivot solve."""
    m = oracle_lib.Mechanism.air()
    n = 17
    total = 101325.0 / (1.380649e-23 * 300.0) * 1e-6
    y = np.full(n, total * 1e-7)
    y[14], y[15], y[16] = total * 0.99 * 0.79, total * 0.99 * 0.21, total * 0.01
    k = m.rate_constants(300.0, total)
    jac = m.jac(k, y)
    pat = m.pattern()
    J = np.zeros((n, n))
    idx = 0
    for i in range(n):
        for j in range(n):
            if pat[i, j]:
                J[i, j] = jac[idx]
                idx += 1
    worst = 0.0
    for hstep in (1e-12, 1e-9, 1e-6, 1e-3, 1.0):
        ghinv = 1.0 / (hstep * 0.5)
        b = 1.0 + 0.25 * np.arange(n)
        x, _ = m.decomp_solve(jac, ghinv, b)
        xr = np.linalg.solve(np.eye(n) * ghinv - J, b)
        worst = max(worst, np.max(np.abs(x - xr) / np.maximum(np.abs(x), np.abs(xr))))
    assert worst < 1e-9


@pytest.mark.parametrize("method,order", [("ros2", 2), ("ros3", 3), ("rodas3", 3)])
def test_fixed_step_order(oracle_lib, method, order):
    """test_kinetics.cpp:183-211: A + B -> C, fixed steps, observed order."""
    O = oracle_lib
    m = O.Mechanism()
    for s in ("A", "B", "C"):
        m.add_species(s, True)
    m.add_reaction("A + B -> C", "arr", (1.0, 0, 0))
    m.finalize()
    A0, B0, T = 2.0, 1.0, 2.0
    d = A0 - B0
    exact = d / (1.0 - (B0 / A0) * np.exp(-d * T))
    errs = []
    for steps in (10, 20, 40, 80):
        ctl = O.control(rtol=1.0, atol=1.0, h_min=0.0, h_start=0.0, max_steps=1000, fixed_step=1)
        y, t, h, st = m.integrate(method, ctl, [1.0], np.zeros(3), [A0, B0, 0.0], T, h0=T / steps)
        errs.append(abs(y[0] - exact))
    assert abs(np.log2(errs[2] / errs[3]) - order) < 0.3


def coop_image(model=None, km=None) -> bytes:
    L = sg.lib()
    if model is not None:
        size = L.kin_model_coop_image(model.h, None, 0)
        buf = (C.c_uint8 * size)()
        assert L.kin_model_coop_image(model.h, buf, size) == size
    else:
        size = L.kin_mech_coop_image(C.byref(km), None, 0)
        buf = (C.c_uint8 * size)()
        assert L.kin_mech_coop_image(C.byref(km), buf, size) == size
    return bytes(buf)


@pytest.mark.parametrize("which", ["air", "synthetic"])
def test_coop_image_same_from_model_and_kinmech(which):
    """The cooperative kernels' image is the same bytes whether it is built from
    the model or from the reference-layout KinMech (the straggler hand-off builds
    it from the KinMech that gpu_kin_set_mech receives)."""
    pm = sg.Model.air() if which == "air" else sg.Model.synthetic(seed=5, species=24, reactions=80, bimolecular=0.7,
                                                                  products=1)
    a = coop_image(model=pm)
    b = coop_image(km=pm.kinmech())
    assert len(a) > 0 and a == b


def test_coop_image_counts_large_mechanism(oracle_lib):
    """Header counts of the 200-species image against the oracle's symbolic phase."""
    pm, om = both_synthetic(oracle_lib, 3, 200, 1200, 1)
    img = coop_image(model=pm)
    n, R, ld, nj, fun_terms, jac_terms, l_entries, u_entries = np.frombuffer(img[:32], dtype=np.uint32)
    lu_updates = np.frombuffer(img[32:40], dtype=np.uint64)[0]
    oc = om.counts()
    assert (n, R, ld) == (200, 1200, 201)
    assert l_entries == oc["lower"] and u_entries == oc["upper"] and lu_updates == oc["updates"]
