"""Golden vectors from the reference's own code.

Runs the reference's unmodified source files -- simple.py, bicgsolver.py,
cgsolver.py, karman_taichi.py (and its 320 x 64 copy debug/karman_taichi.py),
debug/linalg.py, debug/ti_bicg_test.py -- under ``ti_standin`` (a NumPy
stand-in for the Taichi API they use; Taichi itself is not installable
here) and writes the results to ``tests/golden/*.npz``.

It needs the reference tree (``KARMAN_TAICHI_REF``, default the read-only
mount this repository was built beside) and runs only where that tree is;
the tests read the committed ``.npz`` files and never import the reference.

Usage:  python tests/golden/make_golden.py [case ...]
Cases:  solvers  simple_cavity  bicgsimp_cavity  jacosimp_cavity  karman_320x64
        karman_640x128_fills
        (default: all; each writes golden_<case>.npz)

What is run, and what is skipped, per case:

* ``solvers`` -- debug/ti_bicg_test.py executed as a script with numpy's
  global generator seeded (its matrix comes from unseeded np.random.rand);
  BICGSolver (bicgsolver.py) and CGSolver (cgsolver.py) on seeded 5-point
  systems in the reference's padded [NX, NY, 5] layout.
* ``simple_cavity`` -- simple.py's class definitions (its module-level demo,
  simple.py:288-303, is not executed: it runs 2000 steps and writes CSV/PNG
  files); the demo's cavity SIMPLESolver(1.0, 1.0, 30, 30) with lid
  tangential velocity 0.1 is stepped 5 times through the body of
  SIMPLESolver.solve (simple.py:270-281) without its every-10-steps dumps.
* ``karman_320x64`` -- debug/karman_taichi.py imported as a module (its
  ``__main__`` block is not run); init() and two SIMPLE sub-iterations of the
  ``__main__`` loop (karman_taichi.py:633-653): solve_momentum_bicgstab(1e-8,
  1, 0, 1), correct_conserv(), solve_pcorrection_bicgstab(1e-8, 1),
  puv_correction(), post_process_field().
* ``karman_640x128_fills`` -- karman_taichi.py (640 x 128, the reference's
  own driver constants) imported as a module; init(), then seeded
  perturbations of u, v, u0, v0 written with from_numpy, then fill_Au,
  fill_Av, fill_Ap; SHA-256 digests of the resulting 5-point planes.
"""
from __future__ import annotations

import ast
import contextlib
import hashlib
import importlib.util
import io
import json
import os
import re
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("KARMAN_TAICHI_REF", "/root/reference")


def install_standin():
    sys.path.insert(0, HERE)
    import ti_standin
    sys.modules["taichi"] = ti_standin
    return ti_standin


def load_module(name, path, keep_demo=True):
    """Import a reference file.  keep_demo=False executes only its imports,
    the ti.init call and its def/class statements (the module-level demo run
    is skipped; the skipped line ranges are returned)."""
    with open(path) as f:
        src = f.read()
    tree = ast.parse(src, filename=path)
    skipped = []
    if not keep_demo:
        body = []
        for node in tree.body:
            keep = isinstance(node, (ast.Import, ast.ImportFrom, ast.FunctionDef, ast.ClassDef))
            if (isinstance(node, ast.Expr) and isinstance(node.value, ast.Call)
                    and ast.unparse(node.value.func) == "ti.init"):
                keep = True
            if keep:
                body.append(node)
            else:
                skipped.append((node.lineno, node.end_lineno))
        tree.body = body
    mod = types.ModuleType(name)
    mod.__file__ = path
    sys.modules[name] = mod
    exec(compile(tree, path, "exec"), mod.__dict__)
    return mod, skipped


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def sparse_planes(field, n, S):
    """5-point planes [A(k,k), A(k,k-S), A(k,k+S), A(k,k+1), A(k,k-1)] of the
    rows 0..n-1 of a pointer-sparse n x n matrix field; asserts that no
    nonzero entry lies off that pattern."""
    c = np.zeros((5, n))
    slot = {0: 0, -S: 1, S: 2, 1: 3, -1: 4}
    for (r, col), val in field.entries().items():
        if r >= n or col >= n:
            continue
        off = col - r
        if off in slot:
            c[slot[off], r] = val
        elif val != 0.0:
            raise AssertionError(f"entry off the 5-point pattern at {(r, col)}: {val}")
    return c


def diag(field, n):
    e = field.entries()
    return np.array([e.get((k, k), 0.0) for k in range(n)])


def count(pattern, text):
    return len(re.findall(pattern, text))


def karman_solve_iters(text):
    """Iterations of each bicgstab call in printed output (karman_taichi.py:438-454 prints one
    'Iteration' line per iteration and ends a call with 'has converged', 'failed' or 'Omega')."""
    out, k = [], 0
    for line in text.splitlines():
        if ">> Iteration" in line:
            k += 1
        elif "has converged" in line or "Bicgstab failed" in line or "Omega = 0.0" in line:
            out.append(k)
            k = 0
    return out


def save(case, arrays, meta):
    """Writes golden_<case>.npz: the arrays and the JSON metadata."""
    meta = dict(meta)
    meta["case"] = case
    meta["generated_by"] = "tests/golden/make_golden.py"
    path = os.path.join(HERE, f"golden_{case}.npz")
    np.savez_compressed(path, meta=np.array(json.dumps(meta, sort_keys=True)), **arrays)
    print(f"wrote {path} ({os.path.getsize(path)} bytes)")


# ---- cases ----------------------------------------------------------------------------------------
def case_solvers():
    ti = install_standin()
    sys.path.insert(0, REF)
    arrays, meta = {}, {}

    # debug/ti_bicg_test.py as a script (it imports debug/linalg.py's bicgstab)
    sys.path.insert(0, os.path.join(REF, "debug"))
    sys.modules.pop("linalg", None)
    np.random.seed(20220301)
    g = {"__name__": "__main__"}
    buf = io.StringIO()
    with open(os.path.join(REF, "debug", "ti_bicg_test.py")) as f:
        code = compile(f.read(), os.path.join(REF, "debug", "ti_bicg_test.py"), "exec")
    with contextlib.redirect_stdout(buf):
        exec(code, g)
    out = buf.getvalue()
    n = g["n"]
    Anp = g["Anp"]
    planes = np.zeros((5, n))        # S = 3: offsets 0, -3, +3, +1, -1
    for c, off in ((0, 0), (1, -3), (2, 3), (3, 1), (4, -1)):
        for r in range(n):
            if 0 <= r + off < n:
                planes[c, r] = Anp[r, r + off]
    arrays.update(kat_coef=planes, kat_b=g["bnp"], kat_x=g["x"].to_numpy(), kat_xnp=g["xnp"])
    meta["kat"] = dict(n=n, S=3, eps=g["eps"], iters=count(r"Iteration", out), np_seed=20220301,
                       allclose=out.count("True"), source="debug/ti_bicg_test.py:21-98, debug/linalg.py:106-226")
    sys.path.pop(0)

    from bicgsolver import BICGSolver
    from cgsolver import CGSolver

    # BICGSolver on a seeded non-symmetric, diagonally dominant system in the padded layout
    # (zero halo rows and links into the halo zeroed, as simple.py's coefficient fields are)
    rng = np.random.default_rng(7)
    NX, NY = 34, 26
    coef = np.zeros((NX, NY, 5))
    inner = (slice(1, NX - 1), slice(1, NY - 1))
    for c in range(1, 5):
        coef[inner + (c,)] = -rng.uniform(0.2, 1.0, (NX - 2, NY - 2))
    coef[1, :, 1] = 0.0; coef[NX - 2, :, 2] = 0.0; coef[:, NY - 2, 3] = 0.0; coef[:, 1, 4] = 0.0
    coef[inner + (0,)] = -coef[inner].sum(axis=-1)[..., ] * 1.0 + 0.3 + rng.uniform(0, 0.2, (NX - 2, NY - 2))
    b = np.zeros((NX, NY))
    b[inner] = rng.standard_normal((NX - 2, NY - 2))
    fc, fb, fx = ti.field(ti.f64, shape=(NX, NY, 5)), ti.field(ti.f64, shape=(NX, NY)), ti.field(ti.f64, shape=(NX, NY))
    fc.from_numpy(coef); fb.from_numpy(b)
    s = BICGSolver(fc, fb, fx)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        s.solve(eps=1e-10, quiet=False)
    arrays.update(bicg_coef=coef, bicg_b=b, bicg_x=fx.to_numpy())
    meta["bicg"] = dict(NX=NX, NY=NY, eps=1e-10, iters=count(r"Iter =", buf.getvalue()),
                        source="bicgsolver.py:88-135")

    # CGSolver on a seeded SPD system: symmetric links, diagonal = -sum(links) + shift
    NX, NY = 30, 22
    w = np.zeros((NX + 1, NY))            # face weights between (i-1, j) and (i, j)
    h = np.zeros((NX, NY + 1))            # face weights between (i, j-1) and (i, j)
    w[2:NX - 1, 1:NY - 1] = rng.uniform(0.5, 2.0, (NX - 3, NY - 2))
    h[1:NX - 1, 2:NY - 1] = rng.uniform(0.5, 2.0, (NX - 2, NY - 3))
    coef = np.zeros((NX, NY, 5))
    coef[:, :, 1] = -w[:NX, :]            # aW: link to (i-1, j)
    coef[:, :, 2] = -w[1:, :]             # aE: link to (i+1, j)
    coef[:, :, 3] = -h[:, 1:]             # aN: link to (i, j+1)
    coef[:, :, 4] = -h[:, :NY]            # aS: link to (i, j-1)
    inner = (slice(1, NX - 1), slice(1, NY - 1))
    coef[inner + (0,)] = -coef[inner][..., 1:].sum(axis=-1) + 0.05
    b = np.zeros((NX, NY))
    b[inner] = rng.standard_normal((NX - 2, NY - 2))
    fc, fb, fx = ti.field(ti.f64, shape=(NX, NY, 5)), ti.field(ti.f64, shape=(NX, NY)), ti.field(ti.f64, shape=(NX, NY))
    fc.from_numpy(coef); fb.from_numpy(b)
    s = CGSolver(fc, fb, fx)
    s.solve(eps=1e-10, quiet=True)
    hist = np.array([float(t) for t in s.history])
    arrays.update(cg_coef=coef, cg_b=b, cg_x=fx.to_numpy(), cg_history=hist)
    meta["cg"] = dict(NX=NX, NY=NY, eps=1e-10, iters=len(hist), source="cgsolver.py:83-114")
    save("solvers", arrays, meta)


def case_simple_cavity(n_steps=5):
    install_standin()
    sys.path.insert(0, REF)
    mod, skipped = load_module("simple", os.path.join(REF, "simple.py"), keep_demo=False)
    s = mod.SIMPLESolver(1.0, 1.0, 30, 30)          # simple.py:288
    s.bc["n"][1] = 0.1                              # simple.py:300
    arrays, steps = {}, []
    s.init()
    for step in range(n_steps):                      # body of simple.py:270-281
        buf = io.StringIO()
        with contextlib.redirect_stdout(buf):
            s.solve_momentum_eqn(1)
            s.compute_mdiv()
            out_m = buf.getvalue()
            if step == 0:
                for name in ("coef_u", "b_u", "coef_v", "b_v"):
                    arrays[f"step0_{name}"] = getattr(s, name).to_numpy()
                arrays["step0_u_mid"] = s.u_mid.to_numpy(); arrays["step0_v_mid"] = s.v_mid.to_numpy()
                arrays["step0_u_relaxed"] = s.u.to_numpy(); arrays["step0_v_relaxed"] = s.v.to_numpy()
            s.solve_pcorrection_eqn()
            if step == 0:
                for name in ("coef_p", "b_p", "pcor", "mdiv"):
                    arrays[f"step0_{name}"] = getattr(s, name).to_numpy()
            s.correct_pressure()
            s.correct_velocity()
            s.compute_mdiv()
        out = buf.getvalue()
        parts = out_m.split(">>> Initial residual")
        it_u = count(r"Iter =", parts[1]) if len(parts) > 1 else 0
        it_v = count(r"Iter =", parts[2]) if len(parts) > 2 else 0
        it_p = count(r"Iter =", out[len(out_m):]) + (1 if "converged" in out[len(out_m):] else 0)
        steps.append(dict(it_u=it_u, it_v=it_v, it_p=it_p))
        for name in ("u", "v", "p", "pcor", "mdiv"):
            arrays[f"step{step + 1}_{name}"] = getattr(s, name).to_numpy()
    meta = dict(lx=1.0, ly=1.0, nx=30, ny=30, bc_n_tangential=0.1, n_steps=n_steps, steps=steps,
                skipped_lines=skipped, source="simple.py:11-285 (demo 288-303 not executed)")
    save("simple_cavity", arrays, meta)


def case_karman_320x64(n_sub=2):
    install_standin()
    sys.path.insert(0, REF)
    path = os.path.join(REF, "debug", "karman_taichi.py")
    spec = importlib.util.spec_from_file_location("karman_taichi_320x64", path)
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    nx, ny = m.nx, m.ny
    nu, nv, n_p = (nx + 1) * ny, nx * (ny + 1), nx * ny
    arrays, subs = {}, []
    m.init()
    arrays["init_ct"] = m.ct.to_numpy().astype(np.int8)
    arrays["init_p"] = m.p.to_numpy()
    pcor_max = 0.0
    t0 = time.time()
    for sub in range(n_sub):                                  # karman_taichi.py:633-653
        buf = io.StringIO()
        with contextlib.redirect_stdout(buf):
            m.solve_momentum_bicgstab(1e-8, 1, 0, 1)
        iters_u_v = karman_solve_iters(buf.getvalue())
        # planes of this sub-iteration's momentum systems
        arrays[f"sub{sub}_Au"] = sparse_planes(m.Au, nu, ny)
        arrays[f"sub{sub}_bu"] = m.bu.to_numpy()
        arrays[f"sub{sub}_Mu"] = diag(m.Mu, nu)
        arrays[f"sub{sub}_Av"] = sparse_planes(m.Av, nv, ny + 1)
        arrays[f"sub{sub}_bv"] = m.bv.to_numpy()
        arrays[f"sub{sub}_Mv"] = diag(m.Mv, nv)
        arrays[f"sub{sub}_xu"] = m.xu.to_numpy()
        arrays[f"sub{sub}_xv"] = m.xv.to_numpy()
        m.correct_conserv()
        arrays[f"sub{sub}_u_conserv"] = m.u.to_numpy()
        arrays[f"sub{sub}_udiv_conserv"] = m.udiv.to_numpy()
        buf = io.StringIO()
        with contextlib.redirect_stdout(buf):
            m.solve_pcorrection_bicgstab(1e-8, 1)
        it_p = karman_solve_iters(buf.getvalue())[0]
        arrays[f"sub{sub}_Ap"] = sparse_planes(m.Ap, n_p, ny)
        arrays[f"sub{sub}_bp"] = m.bp.to_numpy()
        arrays[f"sub{sub}_Mp"] = diag(m.Mp, n_p)
        arrays[f"sub{sub}_xp"] = m.xp.to_numpy()
        r = m.puv_correction()
        if sub == 0:
            pcor_max = float(r)
        for name in ("u", "v", "p", "pcor"):
            arrays[f"sub{sub}_{name}"] = getattr(m, name).to_numpy()
        m.post_process_field()
        arrays[f"sub{sub}_u_post"] = m.u_post.to_numpy()
        arrays[f"sub{sub}_v_post"] = m.v_post.to_numpy()
        arrays[f"sub{sub}_udiv"] = m.udiv.to_numpy()
        subs.append(dict(it_u=iters_u_v[0], it_v=iters_u_v[1], it_p=it_p,
                         pcor=float(r), seconds=round(time.time() - t0, 1)))
        print(subs[-1], flush=True)
    # display canvases are large; their digests are kept
    meta = dict(nx=nx, ny=ny, n_sub=n_sub, subs=subs, pcor_max_first=pcor_max,
                canvas_digest={name: digest(getattr(m, name).to_numpy())
                               for name in ("u_disp", "v_disp", "p_disp", "pcor_disp", "udiv_disp")},
                source="debug/karman_taichi.py (the 320 x 64 copy of karman_taichi.py), main loop :633-653")
    save("karman_320x64", *compact_karman(arrays, meta))


# arrays of the karman case kept whole in float64: the cell types, the initial pressure and the
# fields after the first sub-iteration (inputs of the bit-exact assembly and post-processing checks)
KARMAN_F64 = ("init_ct", "init_p", "sub0_u", "sub0_v", "sub0_p")
# compared bit for bit: only their SHA-256 digests are kept
KARMAN_DIGEST = ("_Au", "_Av", "_Ap", "_bu", "_bv", "_bp", "_Mu", "_Mv", "_Mp", "_u_post", "_v_post")


def compact_karman(arrays, meta):
    """Keeps the karman fixture small: assembled systems and post-processed fields as digests
    (rows of planes: one digest per plane), the tolerance-compared fields rounded to float32 (the
    tests' field tolerance, 1e-6 relative, is far above float32 rounding), the inputs of the
    bit-exact checks in float64; intermediate arrays no test reads are dropped."""
    out, dig = {}, {}
    for k, a in arrays.items():
        if k in KARMAN_F64:
            out[k] = a
        elif k.endswith(KARMAN_DIGEST):
            if a.ndim == 2 and a.shape[0] == 5 and k.endswith(("_Au", "_Av", "_Ap")):
                for c in range(5):
                    dig[f"{k}{c}"] = digest(a[c])
            else:
                dig[k] = digest(a)
        elif k.endswith(("_u", "_v", "_p", "_pcor", "_xu", "_xv", "_xp")):
            out[k] = a.astype(np.float32)
    meta = dict(meta, digests=dig, float32_fields="fields other than " + ", ".join(KARMAN_F64))
    return out, meta


def case_karman_640x128_fills(seed=11):
    install_standin()
    sys.path.insert(0, REF)
    path = os.path.join(REF, "karman_taichi.py")
    spec = importlib.util.spec_from_file_location("karman_taichi_640x128", path)
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    nx, ny = m.nx, m.ny
    m.init()
    ct, p = m.ct.to_numpy(), m.p.to_numpy()
    rng = np.random.default_rng(seed)
    for name in ("u", "v", "u0", "v0"):
        f = getattr(m, name)
        f.from_numpy(rng.standard_normal(f.shape))
    m.fill_Au(); m.fill_Av(); m.fill_Ap()
    nu, nv, n_p = (nx + 1) * ny, nx * (ny + 1), nx * ny
    dig = dict(ct=hashlib.sha256(np.ascontiguousarray(ct, dtype="<i4").tobytes()).hexdigest(), p=digest(p))
    for name, A, b, M, n, S in (("u", m.Au, m.bu, m.Mu, nu, ny), ("v", m.Av, m.bv, m.Mv, nv, ny + 1),
                                ("p", m.Ap, m.bp, m.Mp, n_p, ny)):
        planes = sparse_planes(A, n, S)
        for c in range(5):
            dig[f"A{name}{c}"] = digest(planes[c])
        dig[f"b{name}"] = digest(b.to_numpy())
        dig[f"M{name}"] = digest(diag(M, n))
    meta = dict(nx=nx, ny=ny, seed=seed, perturb="u, v, u0, v0 = default_rng(seed).standard_normal(shape), in that order",
                digests=dig, source="karman_taichi.py:130-154, 162-339")
    save("karman_640x128_fills", {"ct": ct.astype(np.int8)}, meta)


def case_bicgsimp_cavity(n_sub=8):
    """bicgsimp.py's cavity (SIMPLESolver(1.0, 1.0, 50, 50), lid tangential velocity 1.0,
    bicgsimp.py:333-371) stepped through the body of its SIMPLE loop (bicgsimp.py:302-326) with the
    persistent solvers of bicgsimp.py:260-262; the matplotlib and GUI lines of solve() and the
    module-level demo are not executed."""
    install_standin()
    sys.path.insert(0, REF)
    mod, skipped = load_module("bicgsimp", os.path.join(REF, "bicgsimp.py"), keep_demo=False)
    from bicgsolver import BICGSolver
    from cgsolver import CGSolver
    s = mod.SIMPLESolver(1.0, 1.0, 50, 50)
    s.bc["n"][1] = 1.0
    s.init()
    s.u_momentum_solver = BICGSolver(s.coef_u, s.b_u, s.u_mid)
    s.v_momentum_solver = BICGSolver(s.coef_v, s.b_v, s.v_mid)
    s.p_correction_solver = CGSolver(s.coef_p, s.b_p, s.pcor)
    arrays, subs = {}, []
    for sub in range(n_sub):
        mres = s.bicg_solve_momentum_eqn(1)
        s.bicg_solve_pcorrection_eqn(1e-8)
        s.correct_pressure()
        s.correct_velocity()
        cres = s.compute_mdiv()
        subs.append(dict(momentum_residual=float(mres), continuity_residual=float(cres),
                         cg_iters=len(s.p_correction_solver.history) - 1))
        print(sub, subs[-1], flush=True)
        if sub in (0, n_sub - 1):
            for name in ("u", "v", "p", "pcor"):
                arrays[f"sub{sub}_{name}"] = getattr(s, name).to_numpy()
    meta = dict(lx=1.0, ly=1.0, nx=50, ny=50, bc_n_tangential=1.0, n_sub=n_sub, subs=subs, skipped_lines=skipped,
                source="bicgsimp.py:258-330 (loop body :302-326), persistent solvers :260-262")
    save("bicgsimp_cavity", arrays, meta)


def case_jacosimp_cavity(n_steps=20):
    """jacosimp.py's cavity (SIMPLESolver(1.0, 1.0, 51, 51), lid tangential velocity 1.0,
    jacosimp.py:274-290): n_steps steps of its solve() loop (jacosimp.py:249-272) without the
    every-100-steps dumps and its prints; the module-level demo is not executed."""
    install_standin()
    sys.path.insert(0, REF)
    mod, skipped = load_module("jacosimp", os.path.join(REF, "jacosimp.py"), keep_demo=False)
    s = mod.SIMPLESolver(1.0, 1.0, 51, 51)
    s.bc["n"][1] = 1.0
    s.init()
    arrays = {}
    for step in range(n_steps):
        s.solve_momentum_eqn()
        if step == 0:
            arrays["step0_u_mid"] = s.u_mid.to_numpy()
            arrays["step0_v_mid"] = s.v_mid.to_numpy()
            arrays["step0_u_sweep"] = s.u.to_numpy()
            arrays["step0_v_sweep"] = s.v.to_numpy()
        s.solve_pcorrection_eqn()
        s.update_pressure()
        s.update_velocity()
        s.compute_mdiv()
        if step in (0, 4, n_steps - 1):
            for name in ("u", "v", "p", "pcor", "mdiv"):
                arrays[f"step{step}_{name}"] = getattr(s, name).to_numpy()
    meta = dict(lx=1.0, ly=1.0, nx=51, ny=51, bc_n_tangential=1.0, n_steps=n_steps, saved_steps=[0, 4, n_steps - 1],
                skipped_lines=skipped, source="jacosimp.py:11-272 (solve loop :249-272)")
    save("jacosimp_cavity", arrays, meta)


CASES = {"solvers": case_solvers, "bicgsimp_cavity": case_bicgsimp_cavity, "jacosimp_cavity": case_jacosimp_cavity, "simple_cavity": case_simple_cavity, "karman_320x64": case_karman_320x64,
         "karman_640x128_fills": case_karman_640x128_fills}

if __name__ == "__main__":
    if not os.path.isdir(REF):
        sys.exit(f"reference tree not found at {REF} (set KARMAN_TAICHI_REF)")
    for c in (sys.argv[1:] or list(CASES)):
        t = time.time()
        CASES[c]()
        print(f"{c}: {time.time() - t:.1f} s", flush=True)
