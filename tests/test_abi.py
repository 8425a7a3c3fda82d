"""The C ABI library loads and exports every symbol include/karman_gb300.h
declares (no compute calls: this runs without a GPU)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_symbols():
    txt = open(os.path.join(ROOT, "include", "karman_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(kc_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_the_hot_path():
    syms = _header_symbols()
    for s in ("kc_spmv", "kc_bicgstab", "kc_cg", "kc_dot", "kc_assemble_momentum", "kc_assemble_pcorr",
              "kc_correct", "kc_karman_fill_u", "kc_karman_puv_correction", "kc_bicgstab_refined"):
        assert s in syms


def test_library_exports_every_header_symbol(lib):
    import ctypes
    from karman_taichi_gb300 import _lib as L
    raw = ctypes.CDLL(L.LIB_PATH)
    missing = [s for s in _header_symbols() if not hasattr(raw, s)]
    assert not missing, missing
    assert set(_header_symbols()) == set(L.SIGNATURES), set(_header_symbols()) ^ set(L.SIGNATURES)


def test_status_strings_and_version(lib):
    from karman_taichi_gb300 import _lib as L
    assert lib.kc_version() >= 10000
    for rc in (L.OK, L.MAXITER, L.BREAKDOWN_RHO, L.BREAKDOWN_OMEGA, L.NONFINITE, L.STALL, L.ERR_ARG):
        assert lib.kc_status_str(rc)
    assert lib.kc_status_str(999) == b"unknown status"


def test_workspace_sizes_are_pure_host_queries(lib):
    n, S = 2050 * 514, 514
    b64 = lib.kc_bicgstab_ws_bytes(n, S, 0)
    b32 = lib.kc_bicgstab_ws_bytes(n, S, 1)
    assert b64 > 7 * 8 * n and b32 > 7 * 4 * n and b64 > b32
    assert lib.kc_refined_ws_bytes(n, S) > b32
    assert lib.kc_reduce_ws_bytes() > 0
    assert lib.kc_bicgstab_ws_bytes(0, 1, 0) == 0


def test_argument_errors_need_no_gpu(lib):
    from karman_taichi_gb300 import _lib as L
    assert lib.kc_spmv(None, None, None, None) == L.ERR_ARG
    assert lib.kc_karman_fill_u(None, *([None] * 9)) == L.ERR_ARG
    assert b"null" in lib.kc_last_error()


def test_library_has_no_cpu_fallback_symbols(lib):
    """The product must fail loudly when its library is missing."""
    from karman_taichi_gb300 import _lib as L
    old = L._lib
    try:
        L._lib = None
        real = L.LIB_PATH
        L.LIB_PATH = real + ".missing"
        with pytest.raises(L.KcLibraryMissing):
            L.load()
    finally:
        L.LIB_PATH = real
        L._lib = old


def test_struct_layouts_match_the_header():
    """ctypes mirrors of the ABI structs have the C sizes (kc_struct_size)."""
    import ctypes as C
    from karman_taichi_gb300 import _lib as L
    lib = L.load()
    for name, cls in (("kc_system", L.KcSystem), ("kc_solve_opts", L.KcSolveOpts), ("kc_solve_info", L.KcSolveInfo),
                      ("kc_mg_opts", L.KcMgOpts), ("kc_phys", L.KcPhys), ("kc_karman", L.KcKarman),
                      ("kc_channel", L.KcChannel), ("kc_channel_stats", L.KcChannelStats),
                      ("kc_unet_net", L.KcUnetNet), ("kc_flex_info", L.KcFlexInfo),
                      ("kc_recycle_state", L.KcRecycleState)):
        assert lib.kc_struct_size(name.encode()) == C.sizeof(cls), name
    assert lib.kc_struct_size(b"nope") == 0
