"""The CUDA path against golden vectors of the reference's own code.

The vectors (``tests/golden/golden_*.npz``, made by
``tests/golden/make_golden.py``) are outputs of the reference's unmodified
simple.py, bicgsolver.py, cgsolver.py, debug/karman_taichi.py,
karman_taichi.py and debug/ti_bicg_test.py.  Everything here runs through
the drop-in modules and the C ABI of libkarman_gb300.so.

Tolerances: karman_taichi.py's assembled systems, the cell types, the
initial pressure and the cell-centre velocities are compared bit for bit;
the simple.py coefficients (a reduced form of the momentum rows' central
part) to 1e-14 relative; linear solves, whose FP64 sums run in another
order than the reference's serial loops, to 1e-8 relative with iteration
counts +-1; fields after whole SIMPLE iterations to 1e-6 relative.
"""
import hashlib
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

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


def T(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def test_bicgstab_matches_reference_kat(dev):
    """debug/ti_bicg_test.py:21-98: the banded n = 320 system (offsets +-1, +-3), right Jacobi with
    M = A, solved by the device BiCGSTAB through the C ABI."""
    import torch
    from karman_taichi_gb300 import linalg
    d, m = load("solvers")
    k = m["kat"]
    coef = T(d["kat_coef"], dev)
    x = torch.zeros(k["n"], dtype=torch.float64, device=dev)
    info = linalg.bicgstab(linalg.Stencil(coef, stride=k["S"]), T(d["kat_b"], dev), x, eps=k["eps"],
                           max_iter=100 * k["n"], warm=True, M=coef[0].clone(), omega_break=True)
    assert info.ok, info
    assert abs(info.iters - k["iters"]) <= 1
    assert rel(x.cpu().numpy(), d["kat_x"]) < 1e-8


@pytest.mark.parametrize("persistent", [True, False])
def test_bicgsolver_matches_reference(dev, persistent):
    """BICGSolver (bicgsolver.py:88-135) on the reference's [NX, NY, 5] layout, read in place."""
    import torch
    from karman_taichi_gb300.bicgsolver import BICGSolver
    d, m = load("solvers")
    coef = T(d["bicg_coef"], dev)
    x = torch.zeros(coef.shape[:2], dtype=torch.float64, device=dev)
    s = BICGSolver(coef, T(d["bicg_b"], dev), x)
    if not persistent:
        from karman_taichi_gb300 import linalg
        info = linalg.bicgstab(s._A(), s.b, s.x, eps=m["bicg"]["eps"], max_iter=s.steps, persistent=False)
    else:
        info = s.solve(eps=m["bicg"]["eps"])
    assert info.ok, info
    assert abs(info.iters - m["bicg"]["iters"]) <= 1
    assert rel(x.cpu().numpy(), d["bicg_x"]) < 1e-8


def test_cgsolver_matches_reference(dev):
    """CGSolver (cgsolver.py:83-114): solution and recorded residual history (cgsolver.py:88, 111)."""
    import torch
    from karman_taichi_gb300.cgsolver import CGSolver
    d, m = load("solvers")
    coef = T(d["cg_coef"], dev)
    x = torch.zeros(coef.shape[:2], dtype=torch.float64, device=dev)
    s = CGSolver(coef, T(d["cg_b"], dev), x)
    info = s.solve(eps=m["cg"]["eps"])
    assert info.ok, info
    assert abs(info.iters - m["cg"]["iters"]) <= 1
    assert rel(x.cpu().numpy(), d["cg_x"]) < 1e-8
    hist = np.array([float(h) for h in s.history])
    ref = d["cg_history"]
    np.testing.assert_allclose(hist[:20], ref[:20], rtol=2e-6)
    k = min(len(hist), len(ref))
    np.testing.assert_allclose(hist[:k], ref[:k], rtol=0.15)


def test_simple_cavity_matches_reference(dev):
    """simple.py's cavity (SIMPLESolver(1, 1, 30, 30), lid 0.1, simple.py:288-303): 5 steps of
    simple.py:270-281 against the reference's fields after every step."""
    from karman_taichi_gb300.simple import SIMPLESolver
    d, m = load("simple_cavity")
    g = SIMPLESolver(m["lx"], m["ly"], m["nx"], m["ny"], device=dev)
    g.bc["n"][1] = m["bc_n_tangential"]
    seen = []

    def check(step, mres, cres):
        if step == 0:
            for name in ("coef_u", "coef_v"):
                a = getattr(g, name).cpu().numpy()
                a = np.moveaxis(a, 0, -1) if a.shape[0] == 5 else a
                assert rel(a, d[f"step0_{name}"]) <= 1e-14, name
        for name in ("u", "v", "p", "pcor"):
            assert rel(getattr(g, name).cpu().numpy(), d[f"step{step + 1}_{name}"]) < 1e-6, (step, name)
        seen.append(step)

    g.solve(n_steps=m["n_steps"], callback=check)
    assert seen == list(range(m["n_steps"]))
    its = [e for e in g.log]
    for step, ref in enumerate(m["steps"]):
        mom, pc = its[2 * step], its[2 * step + 1]
        assert abs(mom[1] - ref["it_u"]) <= 1 and abs(mom[2] - ref["it_v"]) <= 1, (step, mom, ref)
        assert abs(pc[1] - ref["it_p"]) <= 1, (step, pc, ref)


def test_karman_640x128_fills_match_reference(dev):
    """karman_taichi.py at its own 640 x 128 size: cell types, pressure ramp and the assembled u, v and
    p' systems (fill_Au / fill_Av / fill_Ap on seeded perturbed fields), bit for bit."""
    import torch
    from karman_taichi_gb300 import karman_taichi as K
    from karman_taichi_gb300.config import KarmanConfig
    d, m = load("karman_640x128_fills")
    st = K.KarmanState(KarmanConfig(nx=m["nx"], ny=m["ny"]), device=dev)
    K.init(st)
    assert np.array_equal(st.ct.cpu().numpy().astype(np.int8), d["ct"])
    dig = m["digests"]
    assert digest(st.p.cpu().numpy()) == dig["p"]
    rng = np.random.default_rng(m["seed"])
    for name in ("u", "v", "u0", "v0"):
        t = getattr(st, name)
        t.copy_(torch.from_numpy(rng.standard_normal(tuple(t.shape))))
    K.fill_Au(st); K.fill_Av(st); K.fill_Ap(st)
    for name in ("u", "v", "p"):
        A, b, M = (getattr(st, f"A{name}").cpu().numpy(), getattr(st, f"b{name}").cpu().numpy(),
                   getattr(st, f"M{name}").cpu().numpy())
        for c in range(5):
            assert digest(A[c]) == dig[f"A{name}{c}"], (name, c)
        assert digest(b) == dig[f"b{name}"], name
        assert digest(M) == dig[f"M{name}"], name


def test_karman_320x64_matches_reference(dev):
    """debug/karman_taichi.py (320 x 64): init and two sub-iterations of the __main__ loop
    (karman_taichi.py:633-653) through the drop-in module: systems bit for bit, solves to 1e-6 with
    iteration counts +-1 (10 % for the several-hundred-iteration p' solve, whose count moves with the
    summation order of BiCGSTAB's dot products), corrected fields and pcor_max to 1e-6, cell-centre
    velocities bit for bit from the reference's own fields."""
    import torch
    from karman_taichi_gb300 import karman_taichi as K
    from karman_taichi_gb300.config import KARMAN_PRESETS
    d, m = load("karman_320x64")
    cfg = KARMAN_PRESETS["karman_320x64"]
    assert (cfg.nx, cfg.ny) == (m["nx"], m["ny"])
    st = K.KarmanState(cfg, device=dev)
    K.init(st)
    assert np.array_equal(st.ct.cpu().numpy().astype(np.int8), d["init_ct"])
    assert np.array_equal(st.p.cpu().numpy(), d["init_p"])
    for sub in range(m["n_sub"]):
        ref = m["subs"][sub]
        st.solves.clear()
        pc = K.substep(st)
        its = {w: info.iters for w, info in st.solves}
        assert abs(its["u"] - ref["it_u"]) <= 1 and abs(its["v"] - ref["it_v"]) <= 1, (sub, its, ref)
        assert abs(its["p"] - ref["it_p"]) <= 0.1 * ref["it_p"], (sub, its, ref)
        assert pc == pytest.approx(ref["pcor"], rel=1e-6)
        for name in ("xu", "xv", "xp"):
            assert rel(getattr(st, name).cpu().numpy(), d[f"sub{sub}_{name}"]) < 1e-6, (sub, name)
        for name in ("u", "v", "p", "pcor"):
            assert rel(getattr(st, name).cpu().numpy(), d[f"sub{sub}_{name}"]) < 1e-6, (sub, name)
    # assembly from the reference's own state after the first sub-iteration (float64 in the fixture):
    # the second sub-iteration's u and v systems bit for bit, and its p' operator (its links and
    # diagonal come from the momentum diagonals and the cell types; its b from the momentum solution)
    dig = m["digests"]
    for name in ("u", "v", "p"):
        getattr(st, name).copy_(T(d[f"sub0_{name}"], dev))
    st.u0.zero_(); st.v0.zero_()
    K.fill_Au(st); K.fill_Av(st); K.fill_Ap(st)
    for name in ("u", "v", "p"):
        A = getattr(st, f"A{name}").cpu().numpy()
        for c in range(5):
            assert digest(A[c]) == dig[f"sub1_A{name}{c}"], (name, c)
        assert digest(getattr(st, f"M{name}").cpu().numpy()) == dig[f"sub1_M{name}"], name
        if name != "p":
            assert digest(getattr(st, f"b{name}").cpu().numpy()) == dig[f"sub1_b{name}"], name
    # cell-centre velocities of the reference's fields after the first sub-iteration (karman_taichi.py:547-550)
    post = K.post_process_field(st, canvases=False)
    assert digest(post["u_post"].cpu().numpy()) == dig["sub0_u_post"]
    assert digest(post["v_post"].cpu().numpy()) == dig["sub0_v_post"]
    torch.cuda.synchronize()
