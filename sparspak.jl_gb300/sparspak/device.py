"""Python face of the numeric engine (include/spk_gpu.h).

``NumericEngine`` owns one ``spk_handle``: the supernodal structure on the
device, the value map of one sparsity pattern, and the FP64 and/or FP32
factors.  Arrays may be numpy (host) or torch CUDA tensors (device); device
tensors are passed by pointer, so the data never leaves HBM.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N

PRECISIONS = {"fp64": N.SPK_FP64, "fp32": N.SPK_FP32, "bf16s": N.SPK_BF16S}


class ErrorException(Exception):
    """Mirror of Julia's ErrorException, raised where the reference throws one."""


class SingularException(ErrorException):
    """A diagonal block had an exactly zero pivot; ``supernode`` is 1-based."""

    def __init__(self, msg, supernode):
        super().__init__(msg)
        self.supernode = supernode


class DeviceTimeoutError(ErrorException):
    """A bounded device wait ran out (SPK_ETIMEOUT): the factors are invalid,
    the CUDA context is still usable and the next factor reassembles A."""


def _prec(p) -> int:
    """Precision code of 'fp64' / 'fp32' / 'bf16s', with '+spd' for the
    symmetric (Cholesky) form of SPD matrices, or an int code."""
    if isinstance(p, str):
        base, _, form = p.lower().partition("+")
        if base not in PRECISIONS or form not in ("", "spd"):
            raise ValueError(f"unknown precision {p!r}; use 'fp64', 'fp32' or 'bf16s', optionally with '+spd'")
        return PRECISIONS[base] | (N.SPK_SPD if form == "spd" else 0)
    return int(p)


def _is_device(a) -> bool:
    return hasattr(a, "is_cuda") and bool(a.is_cuda)


def _ptr(a):
    """(pointer, where) of a numpy array or a torch CUDA tensor of float64."""
    if _is_device(a):
        import torch

        if a.dtype != torch.float64 or not a.is_contiguous():
            raise ValueError("device arrays must be contiguous torch.float64 tensors")
        return ctypes.c_void_p(a.data_ptr()), N.SPK_DEVICE
    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.f_contiguous | a.flags.c_contiguous):
        raise ValueError("host arrays must be contiguous numpy float64 arrays")
    return ctypes.c_void_p(a.ctypes.data), N.SPK_HOST


def _shape(a):
    """(n, nrhs, ld) of a right-hand-side block.

    numpy: a vector, or an F-contiguous n x nrhs matrix.  torch (CUDA): a
    vector, or a contiguous (nrhs, n) tensor whose rows are the right-hand sides.
    """
    if _is_device(a):
        if a.dim() == 1:
            return a.shape[0], 1, a.shape[0]
        return a.shape[1], a.shape[0], a.shape[1]
    if a.ndim == 1:
        return a.shape[0], 1, a.shape[0]
    if a.flags.f_contiguous or a.shape[1] == 1:
        return a.shape[0], a.shape[1], a.shape[0]
    raise ValueError("a numpy right-hand-side matrix must be F-contiguous (n x nrhs)")


class NumericEngine:
    """One supernodal structure on the GPU (spk_create ... spk_destroy)."""

    def __init__(self, n, nsuper, xsuper, snode, xlindx, lindx, xlnz, xunz, index_base=1):
        self._lib = N.gpu()
        self.n = int(n)
        arrs = [np.ascontiguousarray(a, dtype=np.int64) for a in (xsuper, snode, xlindx, lindx, xlnz, xunz)]
        h = ctypes.c_void_p()
        rc = self._lib.spk_create(self.n, int(nsuper), *[N.p64(a) for a in arrs], int(index_base), ctypes.byref(h))
        if rc != N.SPK_OK:
            raise ErrorException(f"spk_create failed ({rc}): {self._lib.spk_last_error(None).decode()}")
        self._h = h
        self.nnz = 0

    # -- plumbing ---------------------------------------------------------
    def _check(self, rc, what):
        if rc == N.SPK_OK:
            return
        msg = self._lib.spk_last_error(self._h).decode()
        if rc == N.SPK_ESINGULAR:
            raise SingularException(msg, None)
        if rc == N.SPK_ETIMEOUT:
            raise DeviceTimeoutError(f"{what}: {msg}")
        raise ErrorException(f"{what}: {msg}")

    def close(self):
        if getattr(self, "_h", None):
            self._lib.spk_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr):
        self._check(self._lib.spk_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)), "spk_set_stream")

    # -- phases -------------------------------------------------------------
    def set_pattern(self, colptr, rowval, rperm, rinvp, index_base=0):
        colptr = np.ascontiguousarray(colptr, dtype=np.int64)
        rowval = np.ascontiguousarray(rowval, dtype=np.int64)
        rperm = np.ascontiguousarray(rperm, dtype=np.int64)
        rinvp = np.ascontiguousarray(rinvp, dtype=np.int64)
        rc = self._lib.spk_set_pattern(self._h, self.n, N.p64(colptr), N.p64(rowval), N.p64(rperm), N.p64(rinvp),
                                       int(index_base))
        self._check(rc, "spk_set_pattern")
        self.nnz = int(colptr[-1] - colptr[0])

    def load_values(self, nzval, precision="fp64"):
        if not _is_device(nzval):
            nzval = np.ascontiguousarray(nzval, dtype=np.float64)
        p, where = _ptr(nzval)
        self._check(self._lib.spk_load_values(self._h, p, where, _prec(precision)), "spk_load_values")

    def factor(self, precision="fp64"):
        first = ctypes.c_int64(0)
        rc = self._lib.spk_factor(self._h, _prec(precision), ctypes.byref(first))
        if rc == N.SPK_ESINGULAR:
            raise SingularException(self._lib.spk_last_error(self._h).decode(), int(first.value))
        self._check(rc, "spk_factor")

    def solve(self, b, precision="fp64", transpose=False):
        """Solve A x = b (A^T x = b with transpose) in place; b is a vector or
        n x nrhs column-major (numpy) / (nrhs, n) (torch)."""
        n, nrhs, ld = _shape(b)
        p, where = _ptr(b)
        fn = self._lib.spk_solve_transpose if transpose else self._lib.spk_solve
        self._check(fn(self._h, p, nrhs, ld, where, _prec(precision)), "spk_solve")
        return b

    def refine(self, b, x, precision="fp32", tol=1e-12, max_iter=20, raise_on_fail=True, transpose=False,
               solver=None):
        """FP64 refinement of x for A x = b (A^T x = b with `transpose`).  Returns
        (preconditioned solves after the first, relative residual); with
        `solver` ('auto', 'ir', 'gmres') the solver actually used is appended."""
        n, nrhs, ld = _shape(b)
        pb, wb = _ptr(b)
        px, wx = _ptr(x)
        if wb != wx:
            raise ValueError("b and x must both live on the host or both on the device")
        it = ctypes.c_int(0)
        rr = ctypes.c_double(0.0)
        used = ctypes.c_int(0)
        if transpose:
            rc = self._lib.spk_refine_transpose(self._h, pb, px, nrhs, ld, wb, _prec(precision), float(tol),
                                                int(max_iter), ctypes.byref(it), ctypes.byref(rr))
        else:
            rc = self._lib.spk_refine_ex(self._h, pb, px, nrhs, ld, wb, _prec(precision), float(tol), int(max_iter),
                                         N.SOLVERS[solver or "auto"], ctypes.byref(it), ctypes.byref(rr),
                                         ctypes.byref(used))
        if not (rc == N.SPK_ENOCONV and not raise_on_fail):
            self._check(rc, "spk_refine")
        if solver is None:
            return it.value, rr.value
        return it.value, rr.value, {N.SPK_SOLVER_IR: "ir", N.SPK_SOLVER_GMRES: "gmres"}.get(used.value, "ir")

    def factor_refine(self, b, x, precision="fp32", tol=1e-12, max_iter=20, raise_on_fail=True, solver=None):
        """Factor (values as loaded) and refine x for A x = b in one call, the
        first solve's lower levels overlapped with the factorisation.  Returns
        as refine."""
        n, nrhs, ld = _shape(b)
        pb, wb = _ptr(b)
        px, wx = _ptr(x)
        if wb != wx:
            raise ValueError("b and x must both live on the host or both on the device")
        it = ctypes.c_int(0)
        rr = ctypes.c_double(0.0)
        used = ctypes.c_int(0)
        first = ctypes.c_int64(0)
        rc = self._lib.spk_factor_refine(self._h, pb, px, nrhs, ld, wb, _prec(precision), float(tol), int(max_iter),
                                         N.SOLVERS[solver or "auto"], ctypes.byref(it), ctypes.byref(rr),
                                         ctypes.byref(used), ctypes.byref(first))
        if rc == N.SPK_ESINGULAR:
            raise SingularException(self._lib.spk_last_error(self._h).decode(), int(first.value))
        if not (rc == N.SPK_ENOCONV and not raise_on_fail):
            self._check(rc, "spk_factor_refine")
        if solver is None:
            return it.value, rr.value
        return it.value, rr.value, {N.SPK_SOLVER_IR: "ir", N.SPK_SOLVER_GMRES: "gmres"}.get(used.value, "ir")

    def grad_pattern(self, lam, x):
        """dA on A's pattern (CSC order) = -sum_r lam_r x_r^T: numpy in, numpy out (or torch CUDA in and out)."""
        n, nrhs, ld = _shape(lam)
        pl, wl = _ptr(lam)
        px, wx = _ptr(x)
        if wl != wx:
            raise ValueError("lam and x must both live on the host or both on the device")
        if wl == N.SPK_DEVICE:
            import torch

            out = torch.empty(self.nnz, dtype=torch.float64, device=lam.device)
            po = ctypes.c_void_p(out.data_ptr())
        else:
            out = np.empty(self.nnz, np.float64)
            po = ctypes.c_void_p(out.ctypes.data)
        self._check(self._lib.spk_grad_pattern(self._h, pl, px, nrhs, ld, wl, po), "spk_grad_pattern")
        return out

    def residual(self, b, x):
        n, nrhs, ld = _shape(b)
        pb, wb = _ptr(b)
        px, _ = _ptr(x)
        rr = ctypes.c_double(0.0)
        self._check(self._lib.spk_residual(self._h, pb, px, nrhs, ld, wb, ctypes.byref(rr)), "spk_residual")
        return rr.value

    def get_factors(self, nnzl, nnzu, precision="fp64"):
        lnz = np.zeros(nnzl, np.float64)
        unz = np.zeros(max(nnzu, 1), np.float64)
        ipiv = np.zeros(self.n, np.int64)
        self._check(self._lib.spk_get_factors(self._h, _prec(precision), N.pd(lnz), N.pd(unz), N.p64(ipiv)),
                    "spk_get_factors")
        return lnz, unz[:nnzu], ipiv

    def stats(self):
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        f = ctypes.c_double()
        self._check(self._lib.spk_stats(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(f)),
                    "spk_stats")
        return {"fronts": a.value, "levels": b.value, "factor_entries": c.value, "lu_flops": f.value}

    # -- options --------------------------------------------------------------
    def set_option(self, name, value):
        """Set a factorisation option (_native.OPTIONS: leaf_queue, wait_budget,
        stall_test, tc_schur_m, tc_trail_rows, tc_wide); takes effect at the next factor."""
        self._check(self._lib.spk_set_option(self._h, N.OPTIONS[name], int(value)), "spk_set_option")

    def get_option(self, name):
        v = ctypes.c_int64()
        self._check(self._lib.spk_get_option(self._h, N.OPTIONS[name], ctypes.byref(v)), "spk_get_option")
        return int(v.value)

    def autotune(self, precision="fp32", reps=3):
        """Time the option sets for the loaded values, keep the fastest and
        return ({option: value}, best factor ms); A stays assembled."""
        ms = ctypes.c_double()
        self._check(self._lib.spk_autotune(self._h, _prec(precision), int(reps), ctypes.byref(ms)), "spk_autotune")
        return {k: self.get_option(k) for k in ("leaf_queue", "tc_schur_m", "tc_trail_rows", "tc_wide")}, ms.value

    # -- launch accounting ----------------------------------------------------
    def profile(self, classes=()):
        """Time the listed kernel classes (names of _native.KERNEL_CLASSES) with CUDA events."""
        mask = 0
        for c in classes:
            mask |= 1 << N.KERNEL_CLASSES.index(c)
        self._check(self._lib.spk_profile(self._h, mask), "spk_profile")

    def profile_reset(self):
        self._check(self._lib.spk_profile_reset(self._h), "spk_profile_reset")

    def profile_read(self):
        """{class: {ms, launches, flops, bytes}} since the last reset."""
        out = {}
        for k, name in enumerate(N.KERNEL_CLASSES):
            ms, fl, by = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
            la = ctypes.c_int64()
            self._check(self._lib.spk_profile_read(self._h, k, ctypes.byref(ms), ctypes.byref(la), ctypes.byref(fl),
                                                   ctypes.byref(by)), "spk_profile_read")
            out[name] = {"ms": ms.value, "launches": la.value, "flops": fl.value, "bytes": by.value}
        return out
