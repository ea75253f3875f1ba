"""ctypes front end of the CPU checker (TEST INFRASTRUCTURE ONLY).

Loads oracle/_build/libpcdm_oracle.so (the C restatement of the reference's
PCDM hot path) and, when it was built, oracle/_ref/libacdc_ref.so (the
reference's own multicore engine compiled from its sources).  Only tests, the
smoke check and the CPU-baseline leg of bench.py use this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpcdm_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libacdc_ref.so")
# The reference checkout, for building its engine (test infrastructure only):
# taken from the environment; without it the engine is not built and the
# tests that run it are skipped (the committed fixtures still pin the oracle).
REF_ROOT_ENV = "ACDC_REFERENCE_ROOT"

_lib = None
_ref = None

f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
I64, U64, D, I = C.c_int64, C.c_uint64, C.c_double, C.c_int

EVAL_KEYS = ("primal", "dual", "gap", "rel_gap", "zero_one_accuracy", "reg_norm", "sq_norm",
             "max_abs_grad", "support")


def build(ref_root=None):
    """Compile the restatement (and the reference engine when its sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    root = ref_root or os.environ.get(REF_ROOT_ENV)
    if root and os.path.isdir(os.path.join(root, "cpp", "src")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF_ROOT=" + root], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_philox4x32_10.argtypes = [u32p, u32p, u32p]
        L.orc_sample.argtypes = [U64, U64, U64]
        L.orc_sample.restype = U64
        L.orc_lasso_lipschitz.argtypes = [I64, i64p, f64p, D, f64p]
        L.orc_lasso_residuals.argtypes = [I64, I64, i64p, i32p, f64p, f64p, f64p, f64p]
        L.orc_lasso_updates.argtypes = [I64, i64p, i32p, f64p, D, f64p, f64p, f64p, U64, U64, U64]
        L.orc_lasso_eval.argtypes = [I64, I64, i64p, i32p, f64p, f64p, D, f64p, f64p, I, f64p]
        L.orc_lasso_solve.argtypes = [I64, I64, i64p, i32p, f64p, f64p, D, D, U64, D, I, I64, I64,
                                      f64p, f64p, f64p]
        L.orc_lasso_solve.restype = I64
        L.orc_lasso_solve_shrink.argtypes = [I64, I64, i64p, i32p, f64p, f64p, D, D, U64, D, I,
                                             I64, I64, D, D, I64, D, f64p, f64p, f64p, f64p]
        L.orc_lasso_solve_shrink.restype = I64
        L.orc_lasso_solve_ws.argtypes = [I64, I64, i64p, i32p, f64p, f64p, D, D, I, I64, I64, D, I,
                                         I, f64p, f64p, f64p, C.POINTER(I64)]
        L.orc_lasso_solve_ws.restype = I64
        L.orc_svm_lipschitz.argtypes = [I64, i64p, f64p, D, f64p]
        L.orc_svm_residuals.argtypes = [I64, I64, i64p, i32p, f64p, f64p, D, f64p, f64p]
        L.orc_svm_updates.argtypes = [I64, i64p, i32p, f64p, f64p, D, f64p, f64p, f64p, U64, U64,
                                      U64]
        L.orc_svm_eval.argtypes = [I64, I64, i64p, i32p, f64p, f64p, D, f64p, f64p, I, f64p]
        L.orc_svm_solve.argtypes = [I64, I64, i64p, i32p, f64p, f64p, D, D, U64, D, I64, I64, f64p,
                                    f64p, f64p]
        L.orc_svm_solve.restype = I64
        L.orc_tau_nice.argtypes = [U64, C.POINTER(U64), I64, I64, i32p]
        L.orc_svm_minibatch.argtypes = [I64, i64p, i32p, f64p, f64p, D, f64p, f64p, f64p, U64,
                                        C.POINTER(U64), I64, I64]
        L.orc_svm_minibatch_solve.argtypes = [I64, I64, i64p, i32p, f64p, f64p, D, D, U64, I64, D,
                                              I64, I64, f64p, f64p, f64p]
        L.orc_svm_minibatch_solve.restype = I64
        L.orc_lasso_hogwild.argtypes = [I64, i64p, i32p, f64p, D, f64p, f64p, f64p, U64, U64, U64,
                                        I]
        L.orc_lasso_hogwild.restype = D
        L.orc_svm_hogwild.argtypes = [I64, i64p, i32p, f64p, f64p, D, f64p, f64p, f64p, U64, U64,
                                      U64, I]
        L.orc_svm_hogwild.restype = D
        L.orc_smooth_lipschitz.argtypes = [I, I64, i64p, f64p, D, D, D, f64p]
        L.orc_smooth_residuals.argtypes = [I, I64, I64, i64p, i32p, f64p, f64p, f64p, f64p]
        L.orc_smooth_updates.argtypes = [I, I64, i64p, i32p, f64p, f64p, D, f64p, f64p, f64p, U64,
                                         U64, U64]
        L.orc_smooth_eval.argtypes = [I, I64, I64, i64p, i32p, f64p, f64p, D, f64p, f64p, f64p]
        L.orc_smooth_solve.argtypes = [I, I64, I64, i64p, i32p, f64p, f64p, D, D, D, U64, D, I,
                                       I64, f64p, f64p, f64p]
        L.orc_smooth_solve.restype = I64
        L.orc_omega.argtypes = [I64, I64, i64p, i32p]
        L.orc_omega.restype = I64
        L.orc_eso_beta.argtypes = [D, D, D]
        L.orc_eso_beta.restype = D
        _lib = L
    return _lib


def ref_lib():
    """The reference's engine, or None when it was not built here."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        R = C.CDLL(REF_PATH)
        R.ref_lasso_run.argtypes = [I, I, i32p, i32p, f64p, f64p, D, I, U64, I, C.c_ulong, f64p,
                                    f64p, f64p]
        R.ref_svm_run.argtypes = [I, I, i32p, i32p, f64p, f64p, D, D, I, U64, I, C.c_ulong, f64p,
                                  f64p, f64p]
        R.ref_smooth_run.argtypes = [I, I, I, i32p, i32p, f64p, f64p, D, D, I, U64, I, C.c_ulong,
                                     f64p, f64p, f64p]
        _ref = R
    return _ref


def _eval_dict(out):
    return {k: float(v) for k, v in zip(EVAL_KEYS, out)}


def philox(ctr, key):
    out = np.zeros(4, np.uint32)
    lib().orc_philox4x32_10(np.asarray(ctr, np.uint32), np.asarray(key, np.uint32), out)
    return out


def sample(seed, k, n):
    return int(lib().orc_sample(seed, k, n))


def omega(m, n, col_ptr, row_idx):
    return int(lib().orc_omega(m, n, col_ptr, row_idx))


def eso_beta(omega_, tau, n):
    return float(lib().orc_eso_beta(omega_, tau, n))


RIDGE, LOGISTIC = 1, 3


class Smooth:
    """Serial FP64 restatement of MulticoreL2SquareRegSquareLoss (loss 1) or
    MulticoreL2SquareRegLogisticLoss (loss 3) driven by the sampler; A is CSC
    over the coordinates (loss 3: features; rows are samples, b the labels)."""

    def __init__(self, loss, m, n, col_ptr, row_idx, vals, b, lam, beta=1.0, sigma=1.0, x0=None):
        self.loss, self.m, self.n, self.lam = int(loss), int(m), int(n), float(lam)
        self.col_ptr = np.ascontiguousarray(col_ptr, np.int64)
        self.row_idx = np.ascontiguousarray(row_idx, np.int32)
        self.vals = np.ascontiguousarray(vals, np.float64)
        self.b = np.ascontiguousarray(b, np.float64)
        self.x = np.zeros(self.n) if x0 is None else np.array(x0, np.float64)
        self.r = np.zeros(self.m)
        self.Li = np.zeros(self.n)
        lib().orc_smooth_lipschitz(self.loss, self.n, self.col_ptr, self.vals, self.lam,
                                   float(beta), float(sigma), self.Li)
        self.refresh()
        self.k = 0

    def refresh(self):
        lib().orc_smooth_residuals(self.loss, self.m, self.n, self.col_ptr, self.row_idx,
                                   self.vals, self.b, self.x, self.r)

    def updates(self, count, seed):
        lib().orc_smooth_updates(self.loss, self.n, self.col_ptr, self.row_idx, self.vals, self.b,
                                 self.lam, self.Li, self.x, self.r, seed, self.k, int(count))
        self.k += int(count)

    def evaluate(self):
        out = np.zeros(9)
        lib().orc_smooth_eval(self.loss, self.m, self.n, self.col_ptr, self.row_idx, self.vals,
                              self.b, self.lam, self.x, self.r, out)
        return _eval_dict(out)


def smooth_solve(loss, m, n, col_ptr, row_idx, vals, b, lam, beta=1.0, sigma=1.0, seed=1,
                 target=1e-9, rel=True, max_epochs=100000, x0=None):
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    r = np.zeros(m)
    out = np.zeros(9)
    ep = lib().orc_smooth_solve(int(loss), m, n, np.ascontiguousarray(col_ptr, np.int64),
                                np.ascontiguousarray(row_idx, np.int32),
                                np.ascontiguousarray(vals, np.float64),
                                np.ascontiguousarray(b, np.float64), lam, beta, sigma, seed,
                                target, int(rel), max_epochs, x, r, out)
    return x, r, _eval_dict(out), int(ep)


def ref_smooth(loss, m, n, col_ptr, row_idx, vals, b, lam, sigma, seed, bulks, inner, threads=1):
    """The reference engine's x, residuals and objective after each bulk (loss 1 or 3)."""
    R = ref_lib()
    if R is None:
        return None
    x = np.zeros(n)
    r = np.zeros(m)
    obj = np.zeros(bulks + 1)
    rc = R.ref_smooth_run(int(loss), m, n, np.ascontiguousarray(col_ptr, np.int32),
                          np.ascontiguousarray(row_idx, np.int32),
                          np.ascontiguousarray(vals, np.float64), np.ascontiguousarray(b, np.float64),
                          lam, sigma, threads, seed, bulks, inner, x, r, obj)
    assert rc == 0
    return x, r, obj


class Lasso:
    """Serial FP64 restatement of MulticoreL1RegSquareLoss driven by the sampler."""

    def __init__(self, m, n, col_ptr, row_idx, vals, b, lam, beta=1.0, x0=None):
        self.m, self.n, self.lam = int(m), int(n), float(lam)
        self.col_ptr = np.ascontiguousarray(col_ptr, np.int64)
        self.row_idx = np.ascontiguousarray(row_idx, np.int32)
        self.vals = np.ascontiguousarray(vals, np.float64)
        self.b = np.ascontiguousarray(b, np.float64)
        self.x = np.zeros(self.n) if x0 is None else np.array(x0, np.float64)
        self.r = np.zeros(self.m)
        self.Li = np.zeros(self.n)
        lib().orc_lasso_lipschitz(self.n, self.col_ptr, self.vals, float(beta), self.Li)
        self.refresh()
        self.k = 0

    def refresh(self):
        lib().orc_lasso_residuals(self.m, self.n, self.col_ptr, self.row_idx, self.vals, self.b,
                                  self.x, self.r)

    def updates(self, count, seed):
        lib().orc_lasso_updates(self.n, self.col_ptr, self.row_idx, self.vals, self.lam, self.Li,
                                self.x, self.r, seed, self.k, int(count))
        self.k += int(count)

    def hogwild(self, count, seed, threads):
        t = lib().orc_lasso_hogwild(self.n, self.col_ptr, self.row_idx, self.vals, self.lam,
                                    self.Li, self.x, self.r, seed, self.k, int(count), threads)
        self.k += int(count)
        return t

    def evaluate(self, threads=0):
        out = np.zeros(9)
        lib().orc_lasso_eval(self.m, self.n, self.col_ptr, self.row_idx, self.vals, self.b,
                             self.lam, self.x, self.r, threads, out)
        return _eval_dict(out)


def lasso_solve(m, n, col_ptr, row_idx, vals, b, lam, beta=1.0, seed=1, target=1e-9, rel=False,
                max_epochs=100000, check_every=1, x0=None):
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    r = np.zeros(m)
    out = np.zeros(9)
    ep = lib().orc_lasso_solve(m, n, np.ascontiguousarray(col_ptr, np.int64),
                               np.ascontiguousarray(row_idx, np.int32),
                               np.ascontiguousarray(vals, np.float64),
                               np.ascontiguousarray(b, np.float64), lam, beta, seed, target,
                               int(rel), max_epochs, check_every, x, r, out)
    return x, r, _eval_dict(out), int(ep)


def lasso_solve_shrink(m, n, col_ptr, row_idx, vals, b, lam, beta=1.0, seed=1, target=1e-9,
                       rel=False, max_epochs=100000, check_every=1, q=0.9, eps=0.1,
                       start_epoch=2, step_scale=1.0, x0=None):
    """Serial FP64 q-shrinking solve (the build's shrinking rule; unpinned)."""
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    r = np.zeros(m)
    out = np.zeros(9)
    trace = np.zeros(max_epochs // max(1, check_every) + 2)
    ep = lib().orc_lasso_solve_shrink(m, n, np.ascontiguousarray(col_ptr, np.int64),
                                      np.ascontiguousarray(row_idx, np.int32),
                                      np.ascontiguousarray(vals, np.float64),
                                      np.ascontiguousarray(b, np.float64), lam, beta, seed, target,
                                      int(rel), max_epochs, check_every, q, eps, start_epoch,
                                      step_scale, x, r, out, trace)
    return x, r, _eval_dict(out), int(ep), trace[:max(0, int(ep) // max(1, check_every))]


def lasso_solve_ws(m, n, col_ptr, row_idx, vals, b, lam, target=1e-9, rel=True, max_checks=100000,
                   sweeps=50, eps=0.1, threads=0, anderson=5, x0=None):
    """Working-set FP64 solve to a certified gap (cyclic exact-step sweeps over
    the working set, Anderson-extrapolated every anderson + 1 sweeps when
    anderson > 1): the optimum for fixtures of large instances.  Returns x,
    r, the last evaluation, the sweeps and the checks made."""
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    r = np.zeros(m)
    out = np.zeros(9)
    checks = I64(0)
    sw = lib().orc_lasso_solve_ws(m, n, np.ascontiguousarray(col_ptr, np.int64),
                                  np.ascontiguousarray(row_idx, np.int32),
                                  np.ascontiguousarray(vals, np.float64),
                                  np.ascontiguousarray(b, np.float64), lam, target, int(rel),
                                  max_checks, sweeps, eps, threads, anderson, x, r, out,
                                  C.byref(checks))
    return x, r, _eval_dict(out), int(sw), int(checks.value)


class SVM:
    """Serial FP64 restatement of MulticoreSVMDualLoss driven by the sampler."""

    def __init__(self, d, n, row_ptr, col_idx, vals, y, lam, sigma=1.0, alpha0=None):
        self.m, self.n, self.lam = int(d), int(n), float(lam)
        self.row_ptr = np.ascontiguousarray(row_ptr, np.int64)
        self.col_idx = np.ascontiguousarray(col_idx, np.int32)
        self.vals = np.ascontiguousarray(vals, np.float64)
        self.y = np.ascontiguousarray(y, np.float64)
        self.x = np.zeros(self.n) if alpha0 is None else np.array(alpha0, np.float64)
        self.r = np.zeros(self.m)
        self.Li = np.zeros(self.n)
        lib().orc_svm_lipschitz(self.n, self.row_ptr, self.vals, float(sigma), self.Li)
        self.refresh()
        self.k = 0

    def refresh(self):
        lib().orc_svm_residuals(self.m, self.n, self.row_ptr, self.col_idx, self.vals, self.y,
                                self.lam, self.x, self.r)

    def updates(self, count, seed):
        lib().orc_svm_updates(self.n, self.row_ptr, self.col_idx, self.vals, self.y, self.lam,
                              self.Li, self.x, self.r, seed, self.k, int(count))
        self.k += int(count)

    def minibatch(self, steps, seed, tau):
        """Synchronous tau-nice mini-batch steps (counter self.k continues)."""
        k = U64(self.k)
        lib().orc_svm_minibatch(self.n, self.row_ptr, self.col_idx, self.vals, self.y, self.lam,
                                self.Li, self.x, self.r, seed, C.byref(k), int(tau), int(steps))
        self.k = int(k.value)

    def hogwild(self, count, seed, threads):
        t = lib().orc_svm_hogwild(self.n, self.row_ptr, self.col_idx, self.vals, self.y, self.lam,
                                  self.Li, self.x, self.r, seed, self.k, int(count), threads)
        self.k += int(count)
        return t

    def evaluate(self, threads=0):
        out = np.zeros(9)
        lib().orc_svm_eval(self.m, self.n, self.row_ptr, self.col_idx, self.vals, self.y,
                           self.lam, self.x, self.r, threads, out)
        return _eval_dict(out)


def svm_solve(d, n, row_ptr, col_idx, vals, y, lam, sigma=1.0, seed=1, target=1e-9,
              max_epochs=100000, check_every=1):
    a = np.zeros(n)
    w = np.zeros(d)
    out = np.zeros(9)
    ep = lib().orc_svm_solve(d, n, np.ascontiguousarray(row_ptr, np.int64),
                             np.ascontiguousarray(col_idx, np.int32),
                             np.ascontiguousarray(vals, np.float64),
                             np.ascontiguousarray(y, np.float64), lam, sigma, seed, target,
                             max_epochs, check_every, a, w, out)
    return a, w, _eval_dict(out), int(ep)


def tau_nice(seed, k, n, tau, steps=1):
    """The tau-nice draws of `steps` steps from counter k: (array steps x tau, new k)."""
    kk = U64(k)
    out = np.zeros((steps, tau), np.int32)
    for st in range(steps):
        row = np.zeros(tau, np.int32)
        lib().orc_tau_nice(seed, C.byref(kk), n, tau, row)
        out[st] = row
    return out, int(kk.value)


def svm_minibatch_solve(d, n, row_ptr, col_idx, vals, y, lam, tau, sigma=1.0, seed=1,
                        target=1e-9, max_epochs=100000, check_every=1):
    """Synchronous mini-batch SDCA solve (hinge dual, tau-nice steps)."""
    a = np.zeros(n)
    w = np.zeros(d)
    out = np.zeros(9)
    ep = lib().orc_svm_minibatch_solve(d, n, np.ascontiguousarray(row_ptr, np.int64),
                                       np.ascontiguousarray(col_idx, np.int32),
                                       np.ascontiguousarray(vals, np.float64),
                                       np.ascontiguousarray(y, np.float64), lam, sigma, seed,
                                       int(tau), target, max_epochs, check_every, a, w, out)
    return a, w, _eval_dict(out), int(ep)


def ref_lasso(m, n, col_ptr, row_idx, vals, b, lam, seed, bulks, inner, threads=1):
    """The reference engine's x, residuals and objective after each bulk."""
    R = ref_lib()
    if R is None:
        return None
    x = np.zeros(n)
    r = np.zeros(m)
    obj = np.zeros(bulks + 1)
    R.ref_lasso_run(m, n, np.ascontiguousarray(col_ptr, np.int32),
                    np.ascontiguousarray(row_idx, np.int32), np.ascontiguousarray(vals, np.float64),
                    np.ascontiguousarray(b, np.float64), lam, threads, seed, bulks, inner, x, r, obj)
    return x, r, obj


def ref_svm(d, n, row_ptr, col_idx, vals, y, lam, sigma, seed, bulks, inner, threads=1):
    """The reference engine's alpha, w and (gap, P, D, acc) after each bulk."""
    R = ref_lib()
    if R is None:
        return None
    a = np.zeros(n)
    w = np.zeros(d)
    ev = np.zeros(4 * (bulks + 1))
    R.ref_svm_run(d, n, np.ascontiguousarray(row_ptr, np.int32),
                  np.ascontiguousarray(col_idx, np.int32), np.ascontiguousarray(vals, np.float64),
                  np.ascontiguousarray(y, np.float64), lam, sigma, threads, seed, bulks, inner, a, w,
                  ev)
    return a, w, ev.reshape(bulks + 1, 4)
