"""The NumPy oracle against golden vectors of the reference's own code.

``tests/golden/golden_*.npz`` hold outputs of the reference's unmodified
simple.py, bicgsolver.py, cgsolver.py, debug/karman_taichi.py,
karman_taichi.py and debug/ti_bicg_test.py, run under a NumPy stand-in for
the Taichi API (``tests/golden/make_golden.py``, ``ti_standin.py``).  These
tests pin the oracle (``oracle/np_oracle.py``) to them; the GPU path is
checked against the same vectors in ``test_gpu_golden.py``.

Tolerances: expressions evaluated in the reference's operation order are
compared bit for bit (coefficients, masks, initial fields); linear-solver
results differ by summation order only (the stand-in sums serially, NumPy
pairwise), so iteration counts agree to +-1 and solutions to ~1e-10
relative; fields after SIMPLE iterations, whose solves stop at a relative
residual, agree to 1e-6 relative -- the FP64 field tolerance of this
library.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import np_oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(case):
    path = os.path.join(GOLDEN, f"golden_{case}.npz")
    if not os.path.exists(path):
        pytest.skip(f"{path} not generated")
    d = np.load(path)
    return d, json.loads(str(d["meta"]))


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


# ---- solvers ---------------------------------------------------------------------------------------
def test_oracle_bicgstab_matches_reference_kat():
    """debug/ti_bicg_test.py:21-98 run through debug/linalg.py's bicgstab (right Jacobi with M = A)."""
    d, m = load("solvers")
    k = m["kat"]
    n = k["n"]
    assert k["allclose"] == 2          # the script's own two np.allclose checks printed True
    coef, b = d["kat_coef"], d["kat_b"]
    r = O.bicgstab(coef, b, k["S"], eps=k["eps"], max_iter=100 * n, x0=np.zeros(n), M=coef[0].copy(),
                   omega_break=True, order="karman")
    assert r.status == O.OK
    assert abs(r.iters - k["iters"]) <= 1
    assert rel(r.x, d["kat_x"]) < 1e-10
    assert rel(r.x, d["kat_xnp"]) < 1e-6


def test_oracle_bicgsolver_matches_reference():
    """BICGSolver.solve (bicgsolver.py:88-135) on the padded [NX, NY, 5] layout."""
    d, m = load("solvers")
    NX, NY = m["bicg"]["NX"], m["bicg"]["NY"]
    coef = np.moveaxis(d["bicg_coef"], -1, 0).reshape(5, -1)
    r = O.bicgstab(coef, d["bicg_b"], NY, eps=m["bicg"]["eps"], max_iter=NX * NY)
    assert r.status == O.OK
    assert abs(r.iters - m["bicg"]["iters"]) <= 1
    assert rel(r.x.reshape(NX, NY), d["bicg_x"]) < 1e-10


def test_oracle_cgsolver_matches_reference():
    """CGSolver.solve (cgsolver.py:83-114) and its convergence history (cgsolver.py:88, 111)."""
    d, m = load("solvers")
    NX, NY = m["cg"]["NX"], m["cg"]["NY"]
    coef = np.moveaxis(d["cg_coef"], -1, 0).reshape(5, -1)
    r = O.cg(coef, d["cg_b"], NY, eps=m["cg"]["eps"], max_iter=NX * NY)
    assert r.status == O.OK
    hist = d["cg_history"]
    assert abs(len(r.history) - len(hist)) <= 1
    k = min(len(r.history), len(hist))
    # the reference records 7 significant digits; CG's residual norms are sensitive to the
    # summation order once orthogonality degrades, so later entries only follow the same curve
    np.testing.assert_allclose(r.history[:20], hist[:20], rtol=2e-6)
    np.testing.assert_allclose(r.history[:k], hist[:k], rtol=0.15)
    assert rel(r.x.reshape(NX, NY), d["cg_x"]) < 1e-10


# ---- simple.py cavity --------------------------------------------------------------------------------
def test_oracle_simple_cavity_matches_reference():
    """SIMPLESolver(1, 1, 30, 30) with lid velocity 0.1 (simple.py:288-303), 5 steps of simple.py:270-281:
    coefficients of the first step bit for bit, fields of every step to 1e-6, solver iterations +-1."""
    d, m = load("simple_cavity")
    o = O.SimpleOracle(m["lx"], m["ly"], m["nx"], m["ny"])
    o.bc["n"][1] = m["bc_n_tangential"]
    o.init()
    for step in range(m["n_steps"]):
        ru, rv = o.solve_momentum_eqn(1)
        o.compute_mdiv()
        if step == 0:
            for name in ("coef_u", "coef_v"):
                assert np.array_equal(np.moveaxis(getattr(o, name), 0, -1), d[f"step0_{name}"]), name
            for name in ("b_u", "b_v"):
                assert np.array_equal(getattr(o, name), d[f"step0_{name}"]), name
            assert rel(o.u_mid, d["step0_u_mid"]) < 1e-10
            assert rel(o.u, d["step0_u_relaxed"]) < 1e-10
        rp = o.solve_pcorrection_eqn()
        if step == 0:
            assert np.array_equal(np.moveaxis(o.coef_p, 0, -1), d["step0_coef_p"])
            # b_p = mdiv of the relaxed velocities, which come out of the solves: not bit for bit
            assert rel(o.b_p, d["step0_b_p"]) < 1e-8
        o.correct_pressure(); o.correct_velocity(); o.compute_mdiv()
        ref = m["steps"][step]
        assert abs(ru.iters - ref["it_u"]) <= 1 and abs(rv.iters - ref["it_v"]) <= 1, (step, ru.iters, rv.iters, ref)
        assert abs(rp.iters - ref["it_p"]) <= 1, (step, rp.iters, ref)
        for name in ("u", "v", "p", "pcor"):
            assert rel(getattr(o, name), d[f"step{step + 1}_{name}"]) < 1e-6, (step, name)


# ---- karman_taichi.py ---------------------------------------------------------------------------------
def test_oracle_karman_640x128_fills_match_reference():
    """karman_taichi.py at its own 640 x 128 size: init (mask, pressure ramp) and fill_Au / fill_Av /
    fill_Ap on seeded perturbed fields, bit for bit (SHA-256 of every plane, b and M)."""
    d, m = load("karman_640x128_fills")
    o = O.KarmanOracle(nx=m["nx"], ny=m["ny"])
    assert np.array_equal(o.ct.astype(np.int8), d["ct"])
    dig = m["digests"]
    assert digest(o.p) == dig["p"]
    rng = np.random.default_rng(m["seed"])
    for name in ("u", "v", "u0", "v0"):
        setattr(o, name, rng.standard_normal(getattr(o, name).shape))
    o.fill_Au(); o.fill_Av(); o.fill_Ap()
    ny = m["ny"]
    for name, A, b, M, S in (("u", o.Au, o.bu, o.Mu, ny), ("v", o.Av, o.bv, o.Mv, ny + 1), ("p", o.Ap, o.bp, o.Mp, ny)):
        planes = A.planes(S)
        for c in range(5):
            assert digest(planes[c]) == dig[f"A{name}{c}"], (name, c)
        assert digest(b) == dig[f"b{name}"], name
        assert digest(np.array([M[k, k] for k in range(b.size)])) == dig[f"M{name}"], name


def test_oracle_karman_320x64_matches_reference():
    """debug/karman_taichi.py (the 320 x 64 geometry): init and two sub-iterations of the __main__ loop
    (karman_taichi.py:633-653).  Assembled systems bit for bit; solves, corrected fields and pcor_max to
    1e-6 relative; momentum BiCGSTAB iterations +-1, the p' solve's within 10 %."""
    d, m = load("karman_320x64")
    o = O.KarmanOracle(nx=m["nx"], ny=m["ny"])
    assert np.array_equal(o.ct.astype(np.int8), d["init_ct"])
    assert np.array_equal(o.p, d["init_p"])
    ny = m["ny"]
    for sub in range(m["n_sub"]):
        r = o.substep()
        ref = m["subs"][sub]
        assert abs(r["it_u"] - ref["it_u"]) <= 1 and abs(r["it_v"] - ref["it_v"]) <= 1, (sub, r, ref)
        # the p' solve takes several hundred iterations; BiCGSTAB's count there moves by a few
        # percent with the summation order of its dot products
        assert abs(r["it_p"] - ref["it_p"]) <= 0.1 * ref["it_p"], (sub, r, ref)
        assert r["pcor_max"] == pytest.approx(ref["pcor"], rel=1e-6)
        for name in ("u", "v", "p", "pcor"):
            assert rel(getattr(o, name), d[f"sub{sub}_{name}"]) < 1e-6, (sub, name)
        assert rel(o.xp, d[f"sub{sub}_xp"]) < 1e-6
        # the momentum systems of the first sub-iteration (assembled from the initial state), bit for bit
        if sub == 0:
            dig = m["digests"]
            for name, A, b, M, S in (("u", o.Au, o.bu, o.Mu, ny), ("v", o.Av, o.bv, o.Mv, ny + 1)):
                planes = A.planes(S)
                for c in range(5):
                    assert digest(planes[c]) == dig[f"sub0_A{name}{c}"], (name, c)
                assert digest(b) == dig[f"sub0_b{name}"], name
                assert digest(np.array([M[k, k] for k in range(b.size)])) == dig[f"sub0_M{name}"], name


def test_oracle_karman_320x64_fills_from_reference_state():
    """The second sub-iteration's systems assembled from the reference's own fields after the first
    (float64 in the fixture): u and v systems and the p' operator bit for bit (SHA-256)."""
    d, m = load("karman_320x64")
    o = O.KarmanOracle(nx=m["nx"], ny=m["ny"])
    o.u, o.v, o.p = d["sub0_u"].copy(), d["sub0_v"].copy(), d["sub0_p"].copy()
    o.u0[...] = 0.0
    o.v0[...] = 0.0
    o.fill_Au(); o.fill_Av(); o.fill_Ap()
    dig, ny = m["digests"], m["ny"]
    for name, A, b, M, S in (("u", o.Au, o.bu, o.Mu, ny), ("v", o.Av, o.bv, o.Mv, ny + 1), ("p", o.Ap, o.bp, o.Mp, ny)):
        planes = A.planes(S)
        for c in range(5):
            assert digest(planes[c]) == dig[f"sub1_A{name}{c}"], (name, c)
        assert digest(np.array([M[k, k] for k in range(b.size)])) == dig[f"sub1_M{name}"], name
        if name != "p":
            assert digest(b) == dig[f"sub1_b{name}"], name


# ---- jacosimp.py / bicgsimp.py cavities ------------------------------------------------------------------
def test_oracle_jacosimp_cavity_matches_reference():
    """jacosimp.py's cavity (SIMPLESolver(1, 1, 51, 51), lid 1.0): 20 steps of its solve loop
    (jacosimp.py:249-272), lexicographic relaxation sweeps in place; the restatement sweeps by
    anti-diagonals and matches the reference bit for bit."""
    d, m = load("jacosimp_cavity")
    o = O.JacoSimpleOracle(m["lx"], m["ly"], m["nx"], m["ny"])
    o.bc["n"][1] = m["bc_n_tangential"]
    o.init()
    for step in range(m["n_steps"]):
        o.jaco_momentum()
        if step == 0:
            assert np.array_equal(o.u_mid, d["step0_u_mid"]) and np.array_equal(o.v_mid, d["step0_v_mid"])
            assert np.array_equal(o.u, d["step0_u_sweep"]) and np.array_equal(o.v, d["step0_v_sweep"])
        o.jaco_pcorrection(); o.update_pressure(); o.jaco_update_velocity(); o.compute_mdiv()
        if step in m["saved_steps"]:
            for name in ("u", "v", "p", "pcor", "mdiv"):
                assert np.array_equal(getattr(o, name), d[f"step{step}_{name}"]), (step, name)


def test_oracle_bicgsimp_cavity_matches_reference():
    """bicgsimp.py's cavity (SIMPLESolver(1, 1, 50, 50), lid 1.0): the first substeps of its SIMPLE loop
    (bicgsimp.py:302-326) with its persistent solvers: the momentum residual (max |u_mid - u| of
    bicgsimp.py:212-225) and the continuity residual (max |mdiv|, bicgsimp.py:114-122) its stop rule
    tests, and the fields.  bicgsimp.py solves the momentum equations only to a relative residual of
    1e-4 (bicgsimp.py:206-208), so two correct implementations that sum in different orders stop on
    iterates ~1e-4 apart, which the outer loop carries: residuals and u, v, p agree to 1e-3, p' (a
    correction shrinking towards zero) to 1e-2."""
    d, m = load("bicgsimp_cavity")
    o = O.SimpleOracle(m["lx"], m["ly"], m["nx"], m["ny"], bicgsimp=True)
    o.bc["n"][1] = m["bc_n_tangential"]
    o.init()
    for sub in range(m["n_sub"]):
        _, _ = o.solve_momentum_eqn(1, eps=1e-4)
        mres = o.last_momentum_residual
        o.solve_pcorrection_eqn(eps=1e-8)
        o.correct_pressure(); o.correct_velocity()
        cres = o.compute_mdiv()
        ref = m["subs"][sub]
        assert mres == pytest.approx(ref["momentum_residual"], rel=1e-3), sub
        assert cres == pytest.approx(ref["continuity_residual"], rel=1e-3), sub
        if f"sub{sub}_u" in d:
            for name in ("u", "v", "p", "pcor"):
                assert rel(getattr(o, name), d[f"sub{sub}_{name}"]) < (1e-2 if name == "pcor" else 1e-3), (sub, name)
