"""ctypes bindings of the two native libraries.

``host()`` returns the structure-phase library (CPU only), ``gpu()`` the
numeric engine.  Both are built in-tree on first use.  The numeric engine has
no CPU fallback: every numeric call goes to ``libspk_gpu.so`` and raises when
the library or a CUDA device is unavailable.
"""
from __future__ import annotations

import ctypes
import threading

import numpy as np

from . import _build

i64 = ctypes.c_int64
P64 = ctypes.POINTER(ctypes.c_int64)
PD = ctypes.POINTER(ctypes.c_double)
VP = ctypes.c_void_p

HOST_SYMBOLS = {
    "spk_host_last_error": (ctypes.c_char_p, []),
    "spk_graph_is_symmetric": (ctypes.c_int, [i64, P64, P64]),
    "spk_graph_symmetrize": (ctypes.c_int, [i64, P64, P64, P64, P64, P64]),
    "spk_order_mmd": (ctypes.c_int, [i64, P64, P64, P64, P64]),
    "spk_order_nd_grid": (ctypes.c_int, [i64, i64, i64, i64, P64, P64, P64, P64]),
    "spk_order_nd_graph": (ctypes.c_int, [i64, P64, P64, i64, P64, P64]),
    "spk_symbolic_create": (ctypes.c_int, [i64, P64, P64, P64, P64, i64, ctypes.POINTER(VP)]),
    "spk_symbolic_sizes": (ctypes.c_int, [VP, P64, P64, P64, P64]),
    "spk_symbolic_get": (ctypes.c_int, [VP, P64, P64, P64, P64, P64, P64, P64, P64, P64, P64]),
    "spk_symbolic_destroy": (None, [VP]),
}

GPU_SYMBOLS = {
    "spk_create": (ctypes.c_int, [i64, i64, P64, P64, P64, P64, P64, P64, ctypes.c_int, ctypes.POINTER(VP)]),
    "spk_set_stream": (ctypes.c_int, [VP, VP]),
    "spk_set_pattern": (ctypes.c_int, [VP, i64, P64, P64, P64, P64, ctypes.c_int]),
    "spk_load_values": (ctypes.c_int, [VP, VP, ctypes.c_int, ctypes.c_int]),
    "spk_factor": (ctypes.c_int, [VP, ctypes.c_int, P64]),
    "spk_solve": (ctypes.c_int, [VP, VP, i64, i64, ctypes.c_int, ctypes.c_int]),
    "spk_solve_transpose": (ctypes.c_int, [VP, VP, i64, i64, ctypes.c_int, ctypes.c_int]),
    "spk_refine_transpose": (ctypes.c_int, [VP, VP, VP, i64, i64, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                            ctypes.c_int, ctypes.POINTER(ctypes.c_int), PD]),
    "spk_grad_pattern": (ctypes.c_int, [VP, VP, VP, i64, i64, ctypes.c_int, VP]),
    "spk_refine": (ctypes.c_int, [VP, VP, VP, i64, i64, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                  ctypes.c_int, ctypes.POINTER(ctypes.c_int), PD]),
    "spk_measure_peaks": (ctypes.c_int, [PD, PD, PD]),
    "spk_set_option": (ctypes.c_int, [VP, ctypes.c_int, i64]),
    "spk_get_option": (ctypes.c_int, [VP, ctypes.c_int, P64]),
    "spk_autotune": (ctypes.c_int, [VP, ctypes.c_int, ctypes.c_int, PD]),
    "spk_refine_ex": (ctypes.c_int, [VP, VP, VP, i64, i64, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), PD,
                                     ctypes.POINTER(ctypes.c_int)]),
    "spk_factor_refine": (ctypes.c_int, [VP, VP, VP, i64, i64, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), PD,
                                         ctypes.POINTER(ctypes.c_int), P64]),
    "spk_residual": (ctypes.c_int, [VP, VP, VP, i64, i64, ctypes.c_int, PD]),
    "spk_residual_noalloc": (ctypes.c_int, [VP, VP, VP, i64, i64, PD]),
    "spk_get_factors": (ctypes.c_int, [VP, ctypes.c_int, PD, PD, P64]),
    "spk_stats": (ctypes.c_int, [VP, P64, P64, P64, PD]),
    "spk_profile": (ctypes.c_int, [VP, ctypes.c_uint]),
    "spk_profile_reset": (ctypes.c_int, [VP]),
    "spk_profile_read": (ctypes.c_int, [VP, ctypes.c_int, PD, P64, PD, PD]),
    "spk_last_error": (ctypes.c_char_p, [VP]),
    "spk_destroy": (None, [VP]),
}

SPK_OK, SPK_EARG, SPK_ECUDA, SPK_ENOMEM, SPK_ESEQ, SPK_ESTRUCT, SPK_ESINGULAR, SPK_ENOCONV = 0, -1, -2, -3, -4, -5, -6, -7
SPK_ETIMEOUT = -8
# spk_set_option / spk_get_option
OPTIONS = {"leaf_queue": 0, "wait_budget": 1, "stall_test": 2, "tc_schur_m": 3, "tc_trail_rows": 4, "tc_wide": 5,
           "lu_pieces": 6, "solve_cluster_minb": 7, "panel_split": 8,
           "schur_split": 9, "schur_far_sms": 10, "solve_chunk": 11}
SPK_HOST, SPK_DEVICE = 0, 1
KERNEL_CLASSES = ["assemble", "getrf", "panel", "trail", "schur", "fwd", "bwd", "permute", "residual", "blockinv",
                  "tc_trail", "tc_schur"]
KERNEL_NAMES = {"assemble": "k_scatter_values",
                "getrf": "k_block_lu_pc+k_block_lu+k_block_lu_small+k_leaf_factor+k_leaf_queue",
                "panel": "k_block_panel",
                "trail": "k_block_trail", "schur": "k_schur",
                "fwd": "k_fwd+k_front_solve<fwd>+k_fwd_l21+k_solve_leaf<fwd>",
                "bwd": "k_bwd_u12+k_bwd+k_front_solve<bwd>+k_solve_leaf<bwd>", "permute": "k_permute+k_unpermute",
                "residual": "k_residual", "blockinv": "k_block_inv",
                "tc_trail": "k_tc_update<TC_TRAIL>", "tc_schur": "k_tc_update<TC_SCHUR>"}
# How each class's FP32 form computes: tensor cores (tcgen05, 3xTF32) or CUDA cores.
KERNEL_UNITS = {"tc_trail": "tcgen05 kind::tf32, 3xTF32 per term", "tc_schur": "tcgen05 kind::tf32, 3xTF32 per term",
                "trail": "FP32/FP64 FMA (fronts without a pack)", "schur": "FP32/FP64 FMA (fronts without a pack)",
                "getrf": "FP32 FMA, latency-bound (one CTA per front, sequential pivot columns; small fronts a warp each)",
                "panel": "FP32 FMA (register-line triangular sweeps)"}
SPK_FP64, SPK_FP32, SPK_BF16S = 0, 1, 2
SPK_SPD = 16   # or-ed with a precision: the symmetric (SPD, Cholesky) form
SPK_SOLVER_AUTO, SPK_SOLVER_IR, SPK_SOLVER_GMRES = 0, 1, 2
SOLVERS = {"auto": SPK_SOLVER_AUTO, "ir": SPK_SOLVER_IR, "gmres": SPK_SOLVER_GMRES}

_lock = threading.Lock()
_host = None
_gpu = None


def _bind(lib, table):
    for name, (res, args) in table.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def host():
    global _host
    with _lock:
        if _host is None:
            _build.build()
            _host = _bind(ctypes.CDLL(_build.HOST_SO), HOST_SYMBOLS)
    return _host


def gpu():
    global _gpu
    with _lock:
        if _gpu is None:
            _build.build()
            _gpu = _bind(ctypes.CDLL(_build.GPU_SO), GPU_SYMBOLS)
    return _gpu


def p64(a: np.ndarray):
    assert a.dtype == np.int64 and a.flags.c_contiguous
    return a.ctypes.data_as(P64)


def pd(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(PD)


def host_error() -> str:
    return host().spk_host_last_error().decode()
