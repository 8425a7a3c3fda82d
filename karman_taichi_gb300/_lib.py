"""ctypes binding of libkarman_gb300.so (declarations in include/karman_gb300.h).

The library is the only compute path: importing an op whose library is
missing raises ``KcLibraryMissing`` -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libkarman_gb300.so")

# status codes (karman_gb300.h)
OK, MAXITER, BREAKDOWN_RHO, BREAKDOWN_OMEGA, NONFINITE, STALL = 0, 1, 2, 3, 4, 5
ERR_ARG, ERR_CUDA, ERR_WORKSPACE, ERR_UNSUPPORTED = -1, -2, -3, -4
F64, F32 = 0, 1
X0_ZERO, X0_WARM = 0, 1
PRECOND_NONE, PRECOND_JACOBI = 0, 1
REL_R0, REL_B = 0, 1
MODE_SIMPLE, MODE_BICGSIMP, MODE_CHANNEL = 0, 1, 2

STATUS_NAMES = {OK: "OK", MAXITER: "MAXITER", BREAKDOWN_RHO: "BREAKDOWN_RHO",
                BREAKDOWN_OMEGA: "BREAKDOWN_OMEGA", NONFINITE: "NONFINITE", STALL: "STALL"}


class KcLibraryMissing(RuntimeError):
    pass


class KcError(RuntimeError):
    def __init__(self, rc, what, detail):
        super().__init__(f"{what} failed with status {rc}: {detail}")
        self.rc = rc


class KcSystem(C.Structure):
    _fields_ = [("n", C.c_longlong), ("cs", C.c_longlong), ("es", C.c_longlong),
                ("coef", C.c_void_p), ("stride", C.c_int), ("dtype", C.c_int),
                ("form", C.c_int), ("pad_", C.c_int)]


FORM_STANDARD, FORM_LAPLACIAN = 0, 1


class KcSolveOpts(C.Structure):
    _fields_ = [("eps", C.c_double), ("max_iter", C.c_longlong), ("x0", C.c_int),
                ("precond", C.c_int), ("omega_break", C.c_int), ("rel_to", C.c_int),
                ("check_every", C.c_int), ("use_graph", C.c_int),
                ("persistent", C.c_int), ("pad_", C.c_int),
                ("history", C.c_void_p), ("history_len", C.c_longlong)]


class KcSolveInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("refinements", C.c_int), ("iters", C.c_longlong),
                ("rel_res", C.c_double), ("r0", C.c_double)]


class KcPhys(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("mode", C.c_int), ("pad_", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double), ("rho", C.c_double), ("mu", C.c_double),
                ("dt", C.c_double), ("U", C.c_double), ("bc", (C.c_double * 2) * 4),
                ("alpha_m", C.c_double), ("alpha_u", C.c_double), ("alpha_p", C.c_double)]


MOMENTUM_BICGSTAB, MOMENTUM_RBGS, MOMENTUM_RBGS_REFINED = 0, 1, 2


class KcMgOpts(C.Structure):
    _fields_ = [("nu_pre", C.c_int), ("nu_post", C.c_int), ("coarsest_sweeps", C.c_int), ("max_levels", C.c_int),
                ("tail", C.c_int), ("big_cells", C.c_int), ("nu_coarse", C.c_int), ("omega", C.c_float * 16),
                ("alpha", C.c_float * 16)]


class KcChannel(C.Structure):
    _fields_ = [("phys", KcPhys),
                ("precision", C.c_int), ("max_outer", C.c_int), ("use_graph", C.c_int), ("persistent", C.c_int),
                ("momentum", C.c_int), ("check_every_p", C.c_int),
                ("mass_tol", C.c_double), ("eps", C.c_double), ("eps_inner", C.c_double), ("eps_inner_p", C.c_double)]
    _fields_ += [(k, C.c_void_p) for k in ("u", "v", "p", "u0", "v0", "pcor", "u_mid", "v_mid", "solid",
                                          "coef_u", "b_u", "coef_v", "b_v", "coef_p", "b_p",
                                          "coef_u32", "b_u32", "coef_v32", "b_v32", "coef_p32", "b_p32",
                                          "mass", "pmax", "rws", "ws_u", "ws_v", "ws_p")]
    _fields_ += [("ws_u_bytes", C.c_size_t), ("ws_v_bytes", C.c_size_t), ("ws_p_bytes", C.c_size_t),
                 ("mg_ws", C.c_void_p), ("mg_ws_bytes", C.c_size_t), ("mg_opts", KcMgOpts),
                 ("learned", C.c_void_p), ("ws_flex", C.c_void_p), ("ws_flex_bytes", C.c_size_t),
                 ("recycle", C.c_int), ("pad2_", C.c_int), ("ws_recycle", C.c_void_p),
                 ("ws_recycle_bytes", C.c_size_t), ("rstate", C.c_void_p)]


class KcRecycleState(C.Structure):
    _fields_ = [("count", C.c_int), ("head", C.c_int)]


class KcChannelStats(C.Structure):
    _fields_ = [("outer", C.c_int), ("fallbacks", C.c_int), ("status", C.c_int), ("pad_", C.c_int),
                ("it_u", C.c_longlong), ("it_v", C.c_longlong), ("it_p", C.c_longlong), ("mass", C.c_double),
                ("learned", C.c_int), ("learned_rejected", C.c_int)]


class KcUnetNet(C.Structure):
    _fields_ = [("NX", C.c_int), ("NY", C.c_int), ("params", C.c_void_p), ("params16", C.c_void_p),
                ("ws", C.c_void_p), ("ws_bytes", C.c_size_t)]


class KcFlexInfo(C.Structure):
    _fields_ = [("learned_used", C.c_int), ("learned_rejected", C.c_int), ("outer", C.c_int), ("pad_", C.c_int)]


class KcKarman(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("dx", C.c_double), ("dy", C.c_double),
                ("rho", C.c_double), ("mu", C.c_double), ("dt", C.c_double),
                ("velo_rel", C.c_double), ("p_rel", C.c_double)]


P_ = C.c_void_p
I_ = C.c_int
L_ = C.c_longlong
S_ = C.c_size_t
D_ = C.c_double
PD = C.POINTER(C.c_double)

# name -> (restype, argtypes); every symbol declared in include/karman_gb300.h
SIGNATURES = {
    "kc_version": (I_, []),
    "kc_status_str": (C.c_char_p, [I_]),
    "kc_last_error": (C.c_char_p, []),
    "kc_device_count": (I_, []),
    "kc_launch_count": (L_, []),
    "kc_struct_size": (S_, [C.c_char_p]),
    "kc_graph_cache_size": (S_, []),
    "kc_graph_cache_limit": (S_, [S_]),
    "kc_debug_barrier_spin_limit": (C.c_uint, [C.c_uint]),
    "kc_device_loop": (I_, [I_]),
    "kc_spmv": (I_, [C.POINTER(KcSystem), P_, P_, P_]),
    "kc_dot_ws_bytes": (S_, [L_]),
    "kc_dot": (I_, [I_, L_, P_, P_, P_, P_, S_, P_]),
    "kc_bicgstab_ws_bytes": (S_, [L_, I_, I_]),
    "kc_bicgstab": (I_, [C.POINTER(KcSystem), P_, P_, P_, P_, S_, C.POINTER(KcSolveOpts),
                         C.POINTER(KcSolveInfo), P_]),
    "kc_bicgstab_noalloc": (I_, [C.POINTER(KcSystem), P_, P_, P_, C.POINTER(KcSolveOpts),
                                 C.POINTER(KcSolveInfo), P_]),
    "kc_cg_ws_bytes": (S_, [L_, I_, I_]),
    "kc_cg": (I_, [C.POINTER(KcSystem), P_, P_, P_, S_, C.POINTER(KcSolveOpts),
                   C.POINTER(KcSolveInfo), P_]),
    "kc_jacobi_ws_bytes": (S_, []),
    "kc_jacobi": (I_, [C.POINTER(KcSystem), P_, P_, P_, D_, I_, I_, I_, I_, P_, P_, S_, P_]),
    "kc_refined_ws_bytes": (S_, [L_, I_]),
    "kc_rbgs_ws_bytes": (S_, [L_, I_]),
    "kc_rbgs": (I_, [C.POINTER(KcSystem), P_, P_, P_, S_, C.POINTER(KcSolveOpts), C.POINTER(KcSolveInfo), P_]),
    "kc_bicgstab_refined": (I_, [C.POINTER(KcSystem), C.POINTER(KcSystem), P_, P_, P_, S_,
                                 C.POINTER(KcSolveOpts), D_, I_, C.POINTER(KcSolveInfo), P_]),
    "kc_rbgs_refined": (I_, [C.POINTER(KcSystem), C.POINTER(KcSystem), P_, P_, P_, S_,
                             C.POINTER(KcSolveOpts), D_, I_, C.POINTER(KcSolveInfo), P_]),
    "kc_mg_default_opts": (None, [C.POINTER(KcMgOpts)]),
    "kc_mg_ws_bytes": (S_, [L_, I_, C.POINTER(KcMgOpts)]),
    "kc_mg_setup": (I_, [C.POINTER(KcSystem), P_, S_, C.POINTER(KcMgOpts), P_]),
    "kc_mg_apply": (I_, [C.POINTER(KcSystem), P_, C.POINTER(KcMgOpts), P_, P_, P_]),
    "kc_pbicgstab_ws_bytes": (S_, [L_, I_]),
    "kc_pbicgstab_refined": (I_, [C.POINTER(KcSystem), C.POINTER(KcSystem), P_, P_, P_, P_, C.POINTER(KcMgOpts),
                                  P_, S_, C.POINTER(KcSolveOpts), D_, I_, C.POINTER(KcSolveInfo), P_]),
    "kc_pcg_refined": (I_, [C.POINTER(KcSystem), C.POINTER(KcSystem), P_, P_, P_, P_, C.POINTER(KcMgOpts),
                            P_, S_, C.POINTER(KcSolveOpts), D_, I_, C.POINTER(KcSolveInfo), P_]),
    "kc_pcg_flexible_ws_bytes": (S_, [L_]),
    "kc_pcg_flexible": (I_, [C.POINTER(KcSystem), C.POINTER(KcSystem), P_, P_, C.POINTER(KcUnetNet), P_,
                             C.POINTER(KcMgOpts), P_, S_, P_, S_, C.POINTER(KcSolveOpts), D_, I_,
                             C.POINTER(KcSolveInfo), C.POINTER(KcFlexInfo), P_]),
    "kc_unet_param_count": (L_, []),
    "kc_unet_predict_ws_bytes": (S_, [I_, I_]),
    "kc_unet_predict": (I_, [C.POINTER(KcUnetNet), P_, P_, P_, P_]),
    "kc_lex_sweep": (I_, [P_, L_, L_, I_, I_, I_, I_, I_, I_, P_, P_, P_, D_, I_, P_]),
    "kc_recycle_ws_bytes": (S_, [L_, I_]),
    "kc_recycle_guess": (I_, [C.POINTER(KcSystem), P_, P_, I_, P_, P_, S_, C.POINTER(C.c_int), P_]),
    "kc_channel_recycle_ws_bytes": (S_, [L_, I_]),
    "kc_reduce_ws_bytes": (S_, []),
    "kc_assemble_momentum": (I_, [C.POINTER(KcPhys)] + [P_] * 14 + [P_]),
    "kc_apply_bc_values": (I_, [C.POINTER(KcPhys), P_, P_, P_]),
    "kc_relax_velocity": (I_, [C.POINTER(KcPhys)] + [P_] * 8),
    "kc_outlet_conserve": (I_, [C.POINTER(KcPhys), P_, P_]),
    "kc_assemble_pcorr": (I_, [C.POINTER(KcPhys)] + [P_] * 13),
    "kc_correct": (I_, [C.POINTER(KcPhys)] + [P_] * 10),
    "kc_mass_residual": (I_, [C.POINTER(KcPhys)] + [P_] * 7),
    "kc_karman_fill_u": (I_, [C.POINTER(KcKarman)] + [P_] * 9),
    "kc_karman_fill_v": (I_, [C.POINTER(KcKarman)] + [P_] * 9),
    "kc_karman_fill_p": (I_, [C.POINTER(KcKarman)] + [P_] * 9),
    "kc_karman_back": (I_, [C.POINTER(KcKarman), I_, P_, P_, P_]),
    "kc_karman_puv_correction": (I_, [C.POINTER(KcKarman)] + [P_] * 10),
    "kc_karman_correct_conserv": (I_, [C.POINTER(KcKarman), P_, P_, P_, P_]),
    "kc_copy": (I_, [P_, P_, S_, P_]),
    "kc_to_f32": (I_, [P_, P_, L_, P_]),
    "kc_unet_conv3x3": (I_, [P_, I_, I_, I_, P_, L_, P_, I_, I_, P_, P_, I_, P_]),
    "kc_unet_conv3x3_wgrad": (I_, [P_, P_, I_, I_, I_, I_, P_, P_, P_]),
    "kc_unet_flip_weights": (I_, [P_, I_, I_, I_, P_, P_]),
    "kc_unet_pool2": (I_, [P_, I_, I_, I_, P_, P_]),
    "kc_unet_pool2_bwd": (I_, [P_, I_, I_, I_, P_, I_, P_]),
    "kc_unet_up2_concat": (I_, [P_, I_, P_, I_, I_, I_, P_, P_]),
    "kc_unet_up2_concat_bwd": (I_, [P_, I_, I_, I_, I_, P_, P_, I_, P_]),
    "kc_unet_relu_bwd": (I_, [P_, P_, L_, P_]),
    "kc_unet_head": (I_, [P_, I_, L_, P_, P_, P_, P_]),
    "kc_unet_head_bwd": (I_, [P_, I_, L_, P_, P_, P_, P_, P_, P_]),
    "kc_unet_mse": (I_, [P_, P_, P_, L_, C.c_float, P_, P_, P_]),
    "kc_unet_adam": (I_, [P_, P_, P_, P_, L_, C.c_float, C.c_float, C.c_float, C.c_float, I_, P_, P_]),
    "kc_unet_to_bf16": (I_, [P_, P_, L_, P_]),
    "kc_channel_step": (I_, [C.POINTER(KcChannel), C.POINTER(KcChannelStats), P_]),
    "kc_channel_batch_step": (I_, [C.POINTER(C.POINTER(KcChannel)), I_, C.POINTER(P_), I_, I_,
                                   C.POINTER(KcChannelStats)]),
    "kc_channel_batch_fused_ws_bytes": (S_, [C.POINTER(C.POINTER(KcChannel)), I_]),
    "kc_channel_batch_fused": (I_, [C.POINTER(C.POINTER(KcChannel)), I_, I_, P_, S_, C.POINTER(KcChannelStats),
                                    C.POINTER(KcChannelStats), P_]),
    "kc_post_process_ws_bytes": (S_, []),
    "kc_post_process": (I_, [I_, I_, D_, D_, P_, P_, P_, P_, P_, P_, P_, P_, P_, P_, S_, P_]),
    "kc_unet_features_ws_bytes": (S_, [I_]),
    "kc_unet_features": (I_, [P_, P_, I_, I_, I_, I_, P_, P_, P_, P_, S_, P_]),
    "kc_unet_guess_up2": (I_, [P_, I_, I_, P_, I_, I_, P_, P_, P_]),
    "kc_unet_target_down2": (I_, [P_, P_, I_, I_, P_, I_, I_, P_, P_, P_]),
}

_lock = threading.Lock()
_lib = None


def lib_path() -> str:
    return LIB_PATH


def load() -> C.CDLL:
    """Load libkarman_gb300.so once; raises KcLibraryMissing if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise KcLibraryMissing(
                f"{LIB_PATH} is missing: build it with `python -m karman_taichi_gb300.build` "
                "(or __graft_entry__.build()); there is no CPU fallback")
        h = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(h, name)
            f.restype = res
            f.argtypes = args
        _lib = h
    return _lib


def last_error() -> str:
    return load().kc_last_error().decode(errors="replace")


def check(rc: int, what: str) -> int:
    """Raise KcError for argument/CUDA errors (rc < 0); return solver outcomes."""
    if rc < 0:
        raise KcError(rc, what, last_error())
    return rc


def status_name(rc: int) -> str:
    return STATUS_NAMES.get(rc, str(rc))
