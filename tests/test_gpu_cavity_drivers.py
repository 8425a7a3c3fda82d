"""The cavity drivers bicgsimp.py and jacosimp.py on the GPU, against the
reference's own runs (golden vectors from the unmodified files,
tests/golden/make_golden.py).

jacosimp.py relaxes instead of solving: one in-place lexicographic sweep per
equation and step.  The GPU sweeps by anti-diagonal wavefronts, the serial
sweep's values exactly; the momentum coefficients come from the assembly
kernel whose central part is an algebraically reduced form (<= 5e-16 of the
row's largest coefficient), so fields agree to 1e-12 relative after the first
sweep and to 1e-10 after 20 steps.

bicgsimp.py keeps persistent solvers (bicgsimp.py:260-262): BiCGSTAB to 1e-4
for u and v, CG to 1e-8 for p' pinned at (1, 1), and reports the momentum and
continuity residuals its stop rule tests (bicgsimp.py:326).  The first 8
substeps are compared.  The momentum solves stop at a relative residual of
1e-4 (bicgsimp.py:206-208), so two correct implementations that sum in
different orders stop on iterates ~1e-4 apart: residuals and u, v, p agree to
1e-3, p' (a correction shrinking towards zero) to 1e-2.  At these settings
(lid 1.0, alpha_m 0.05) the reference's stop rule "momentum < 1e-2 and
continuity < 1e-6" (bicgsimp.py:326) is never met: the restatement ran 20,000
substeps with the momentum residual still 1-20 and continuity ~1e-3, so the
reference driver always runs to its 10,000-substep cap.
"""
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


def test_jacosimp_cavity_matches_reference(dev):
    from karman_taichi_gb300.jacosimp import SIMPLESolver
    d, m = load("jacosimp_cavity")
    g = SIMPLESolver(m["lx"], m["ly"], m["nx"], m["ny"], device=dev)
    g.bc["n"][1] = m["bc_n_tangential"]
    g.init()
    for step in range(m["n_steps"]):
        g.solve_momentum_eqn()
        if step == 0:
            for name, key in (("u_mid", "step0_u_mid"), ("v_mid", "step0_v_mid"), ("u", "step0_u_sweep"),
                              ("v", "step0_v_sweep")):
                assert rel(getattr(g, name).cpu().numpy(), d[key]) <= 1e-12, name
        g.solve_pcorrection_eqn(); g.update_pressure(); g.update_velocity(); g.compute_mdiv()
        if step in m["saved_steps"]:
            for name in ("u", "v", "p", "pcor"):
                assert rel(getattr(g, name).cpu().numpy(), d[f"step{step}_{name}"]) <= 1e-10, (step, name)


def test_lex_sweep_is_the_serial_sweep(dev):
    """kc_lex_sweep on a seeded random system equals the restatement's diagonal-by-diagonal sweep
    (itself the serial Python loop's order) bit for bit, in place and relaxed."""
    import torch
    from karman_taichi_gb300 import _lib as L
    from karman_taichi_gb300.linalg import stream_handle
    from oracle import np_oracle as O
    rng = np.random.default_rng(4)
    NX, NY = 37, 29
    c = -rng.uniform(0.1, 1.0, (5, NX, NY))
    c[0] = -c[1:].sum(axis=0) + 0.3
    b = rng.standard_normal((NX, NY))
    x0 = rng.standard_normal((NX, NY))
    for relax, box in ((True, (2, NX - 1, 1, NY - 1)), (False, (1, NX - 1, 2, NY - 2))):
        xr = x0.copy()
        xm = np.zeros_like(x0)
        O.lex_sweep(c, b, xr, box, 0.37, relax, xm)
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
        ct, bt, xt, xmt = t(c), t(b), t(x0), t(np.zeros_like(x0))
        L.check(L.load().kc_lex_sweep(ct.data_ptr(), NX * NY, 1, NX, NY, *box, bt.data_ptr(), xt.data_ptr(),
                                      xmt.data_ptr(), 0.37, int(relax), stream_handle(dev)), "kc_lex_sweep")
        assert np.array_equal(xt.cpu().numpy(), xr)
        if relax:
            assert np.array_equal(xmt.cpu().numpy(), xm)


def test_bicgsimp_cavity_matches_reference(dev):
    from karman_taichi_gb300.simple import SIMPLESolver
    d, m = load("bicgsimp_cavity")
    g = SIMPLESolver(m["lx"], m["ly"], m["nx"], m["ny"], device=dev, bicgsimp=True)
    g.bc["n"][1] = m["bc_n_tangential"]
    g.init()
    for sub in range(m["n_sub"]):
        mres = g.bicg_solve_momentum_eqn(1)
        g.bicg_solve_pcorrection_eqn(1e-8)
        g.correct_pressure()
        g.correct_velocity()
        cres = g.compute_mdiv()
        ref = m["subs"][sub]
        assert mres == pytest.approx(ref["momentum_residual"], rel=1e-3), sub
        assert cres == pytest.approx(ref["continuity_residual"], rel=1e-3), sub
        if f"sub{sub}_u" in d:
            for name in ("u", "v", "p", "pcor"):
                assert rel(getattr(g, name).cpu().numpy(), d[f"sub{sub}_{name}"]) <= (1e-2 if name == "pcor" else 1e-3), \
                    (sub, name)


def test_bicgsimp_cavity_runs_to_its_stop_rule(dev):
    """bicgsimp.py's own case (50 x 50, lid u = 1, Re 100) to its stop rule: the substeps, the
    final residuals and the centreline profiles its plot compares with Ghia et al. (1982) are those
    committed by tests/golden/make_cavity_profiles.py (which compare_ghia.py sets against the
    reference's data file: within 0.004 in u and 0.009 in v of the lid velocity)."""
    import os
    import numpy as np
    import torch
    from karman_taichi_gb300.simple import SIMPLESolver
    ref = np.load(os.path.join(os.path.dirname(__file__), "golden", "cavity_bicgsimp_50x50_profiles.npz"))
    s = SIMPLESolver(1.0, 1.0, 50, 50, device=dev, bicgsimp=True)
    s.bc["n"][1] = 1.0
    last = {}
    s.solve(n_steps=10000, callback=lambda step, m, c: last.update(step=step, m=m, c=c))
    torch.cuda.synchronize()
    assert last["step"] + 1 == int(ref["substeps"])
    assert last["m"] < 1e-2 and last["c"] < 1e-6
    u = s.u.cpu().numpy()[26, 1:51]
    v = s.v.cpu().numpy()[1:51, 26]
    assert np.abs(u - ref["u_at_x05"]).max() <= 1e-9
    assert np.abs(v - ref["v_at_y05"]).max() <= 1e-9
