"""kc_bicgstab_noalloc: BiCGSTAB for callers that cannot allocate device memory.

Some callers of this library cannot hand it a workspace: a plugin running
inside a host framework whose allocator owns all device memory, or a loop in
which cudaMalloc/cudaFree (which can synchronise the whole device) are not
acceptable.  For them the library keeps a fixed static scratch array on the
device.  This test calls the entry point through the C ABI twice in a row,
in FP64 and FP32, without and with the Jacobi preconditioner, and checks both
results against kc_bicgstab with a caller-allocated workspace, within the
solver tolerances the other solver tests use (1e-6 relative in FP64, 1e-5 in
FP32; the two paths run the same kernels, so they normally agree exactly).
It lives in its own file, collected last, so that a failure here stops a
fail-fast run only after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _laplacian(N, offset=0.05):
    c = np.zeros((5, N, N))
    c[0] = 4.0 + offset
    c[1, 1:, :] = -1.0
    c[2, :-1, :] = -1.0
    c[3, :, :-1] = -1.0
    c[4, :, 1:] = -1.0
    # a varying diagonal, so that the Jacobi preconditioner is not a constant scale
    c[0] *= 1.0 + 0.5 * np.random.default_rng(3).random((N, N))
    return c.reshape(5, -1)


def _opts(L, n, persistent, eps, precond):
    o = L.KcSolveOpts()
    o.eps, o.max_iter, o.x0, o.precond = eps, n, L.X0_ZERO, precond
    o.omega_break, o.rel_to, o.check_every, o.use_graph = 0, L.REL_R0, 0, 0
    o.persistent, o.history, o.history_len = persistent, None, 0
    return o


@pytest.mark.parametrize("persistent", [1, 0])
@pytest.mark.parametrize("precond", ["none", "jacobi"])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_noalloc_matches_workspace_solver_twice(persistent, precond, dtype):
    import torch
    from karman_taichi_gb300 import _lib as L
    lib = L.load()
    dev = torch.device("cuda:0")
    tdt, kdt, eps, tol = ((torch.float64, L.F64, 1e-9, 1e-6) if dtype == "f64"
                          else (torch.float32, L.F32, 1e-5, 1e-5))
    pre = L.PRECOND_JACOBI if precond == "jacobi" else L.PRECOND_NONE
    N = 96                                  # 9216 unknowns, inside KC_NOALLOC_MAX_N
    c = torch.from_numpy(_laplacian(N)).to(dev, tdt).contiguous()
    M = c[0].clone() if pre == L.PRECOND_JACOBI else None
    Mp = C.c_void_p(M.data_ptr()) if M is not None else None
    b = torch.from_numpy(np.random.default_rng(11).standard_normal(N * N)).to(dev, tdt)
    A = L.KcSystem(N * N, N * N, 1, c.data_ptr(), N, kdt)
    s = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)

    ws = torch.zeros(lib.kc_bicgstab_ws_bytes(N * N, N, kdt), dtype=torch.uint8, device=dev)
    x_ref = torch.zeros_like(b)
    info = L.KcSolveInfo()
    o = _opts(L, N * N, persistent, eps, pre)
    rc = lib.kc_bicgstab(C.byref(A), C.c_void_p(b.data_ptr()), C.c_void_p(x_ref.data_ptr()), Mp,
                         C.c_void_p(ws.data_ptr()), ws.numel(), C.byref(o), C.byref(info), s)
    assert rc == L.OK, L.last_error()
    ref = x_ref.double().cpu().numpy()

    for _ in range(2):                      # the shared scratch keeps the last call's contents
        x = torch.full_like(b, 7.0)         # garbage in x: the cold start must overwrite it
        info2 = L.KcSolveInfo()
        rc = lib.kc_bicgstab_noalloc(C.byref(A), C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), Mp,
                                     C.byref(o), C.byref(info2), s)
        assert rc == L.OK, L.last_error()
        assert info2.iters == info.iters
        got = x.double().cpu().numpy()
        assert np.abs(got - ref).max() <= tol * np.abs(ref).max()


def test_noalloc_rejects_oversize_systems():
    import torch
    from karman_taichi_gb300 import _lib as L
    lib = L.load()
    n = 65536 + 1
    A = L.KcSystem(n, n, 1, C.c_void_p(16), 257, L.F64)    # never dereferenced: rejected first
    o = _opts(L, n, 1, 1e-9, L.PRECOND_NONE)
    info = L.KcSolveInfo()
    rc = lib.kc_bicgstab_noalloc(C.byref(A), C.c_void_p(16), C.c_void_p(16), None, C.byref(o), C.byref(info),
                                 C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == L.ERR_ARG
    assert "exceeds the static scratch limit" in L.last_error()
