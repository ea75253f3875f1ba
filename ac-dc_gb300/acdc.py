"""Python binding of the GB300 PCDM library over its C-ABI (ctypes).

This is a thin caller of lib/libacdc_gpu.so and lib/libacdc_host.so for tests
and benchmarks; it computes nothing itself.  Loading fails loudly when the
native libraries are missing: there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(PKG, "lib")
GPU_LIB = os.path.join(LIBDIR, "libacdc_gpu.so")
HOST_LIB = os.path.join(LIBDIR, "libacdc_host.so")

OK, EINVAL, ENOMEM, EUNSUPPORTED, ECUDA, ETIMEOUT, EDEVICE, EBUSY, ENOTFOUND, ENODEV = (
    0, -1, -2, -3, -4, -5, -6, -7, -8, -9)
ECANCELED = -10
LOSS_L1_SQUARE, LOSS_L2_SQUARE, LOSS_SVM_DUAL, LOSS_LOGISTIC = 0, 1, 2, 3
NNZ_FIXED, NNZ_ZIPF, NNZ_UNIFORM = 0, 1, 2
PREC_AUTO, PREC_FP32, PREC_FP64 = 0, 1, 2

I32, I64, U64, D = C.c_int32, C.c_int64, C.c_uint64, C.c_double
VP = C.c_void_p


class Settings(C.Structure):
    _fields_ = [("loss", I32), ("tau", I32), ("warps_per_block", I32), ("refresh_every", I32),
                ("seed", U64), ("sigma", D), ("gap_target", D), ("gap_relative", I32),
                ("max_epochs", I32), ("use_shrinking", I32), ("shrinking_starting_iter", I32),
                ("shrinking_probability", D), ("shrink_eps", D), ("precision", I32),
                ("tau_active", I32), ("polish_rel_gap", D), ("active_passes", I32),
                ("screened_eval", I32), ("polish_stall_epochs", I32), ("hot_polish_sweeps", I32),
                ("hot_threshold", D), ("polish_active_passes", I32), ("lanes_per_update", I32),
                ("minibatch", I32), ("reserved3", I32)]


class Eval(C.Structure):
    _fields_ = [("primal", D), ("dual", D), ("gap", D), ("rel_gap", D),
                ("zero_one_accuracy", D), ("reg_norm", D), ("sq_norm", D),
                ("max_abs_grad", D), ("support", I64), ("active", I64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Stats(C.Structure):
    _fields_ = [("updates", U64), ("nonzero_updates", U64), ("nnz_read", U64),
                ("nnz_scattered", U64), ("update_ms", D), ("eval_ms", D),
                ("update_launches", I64), ("eval_launches", I64), ("screened_evals", I64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SolveResult(C.Structure):
    _fields_ = [("eval", Eval), ("converged", I32), ("epochs", I32), ("seconds", D),
                ("stats", Stats), ("device_ms", D), ("fp64_epochs", I32), ("reserved", I32)]


class TraceRow(C.Structure):
    _fields_ = [("updates", U64), ("primal", D), ("gap", D), ("rel_gap", D), ("active", I64),
                ("hot", I64), ("omega_active", I64), ("omega_hot", I64), ("update_ms", C.c_float),
                ("eval_ms", C.c_float), ("shrink", I32), ("fp64", I32), ("screened", I32),
                ("reserved", I32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class ProblemInfo(C.Structure):
    _fields_ = [("m", I64), ("n", I64), ("nnz", I64), ("nnz_padded", I64), ("omega", I64),
                ("sigma", D), ("lambda_", D), ("device_bytes", I64), ("loss", I32), ("tau", I32),
                ("omega_active", I64), ("active_step_scale", D), ("long_columns", I64)]


class BatchOptions(C.Structure):
    _fields_ = [("path_len", I32), ("max_epochs", I32), ("gap_target", D), ("refresh_every", I32),
                ("autotune", I32), ("tau_override", I32), ("plain", I32), ("use_shrinking", I32),
                ("active_passes", I32), ("reserved", I32 * 6)]


class BatchResult(C.Structure):
    _fields_ = [("eval", Eval), ("lambda_", D), ("converged", I32), ("epochs", I32), ("tau", I32),
                ("reserved", I32)]


class ServerOptions(C.Structure):
    _fields_ = [("memory_budget_bytes", I64), ("max_slots", I32), ("quantum_epochs", I32),
                ("max_epochs", I32), ("use_shrinking", I32), ("reserved", I32 * 6)]


class ServerStats(C.Structure):
    _fields_ = [("steps", I64), ("builds", I64), ("rounds", I64), ("admitted", I64),
                ("retired", I64), ("admit_s", D), ("build_s", D), ("rounds_s", D),
                ("retire_s", D)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Request(C.Structure):
    _fields_ = [("loss", I32), ("reserved0", I32), ("m", I64), ("n", I64), ("col_ptr", VP),
                ("row_idx", VP), ("vals", VP), ("rhs", VP), ("lambda_", D), ("gap_target", D),
                ("seed", U64)]


class RequestResult(C.Structure):
    _fields_ = [("state", I32), ("converged", I32), ("epochs", I32), ("status", I32),
                ("eval", Eval), ("submit_time", D), ("start_time", D), ("finish_time", D)]


class LassoGen(C.Structure):
    _fields_ = [("m", I64), ("n", I64), ("nnz_mode", I32), ("nnz_per_col", I32), ("zipf_s", D),
                ("nnz_min", I32), ("nnz_max", I32), ("nnz_mean", D), ("n_star", I64),
                ("noise_sigma", D), ("lambda_frac", D), ("seed", U64),
                ("normalize_columns", I32), ("threads", I32)]


class SvmGen(C.Structure):
    _fields_ = [("n_samples", I64), ("d", I64), ("nnz_median", D), ("nnz_sigma", D),
                ("w_star_nnz", I64), ("flip_prob", D), ("seed", U64), ("threads", I32)]


class AcdcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("acdc error %d: %s" % (code, msg))
        self.code = code


_gpu = None
_host = None


def _ptr(a):
    return None if a is None else VP(a.ctypes.data)


def gpu_lib():
    """libacdc_gpu.so; raises if it was not built (no fallback)."""
    global _gpu
    if _gpu is None:
        if not os.path.exists(GPU_LIB):
            raise RuntimeError("libacdc_gpu.so is missing: run __graft_entry__.build() first")
        L = C.CDLL(GPU_LIB)
        L.acdc_last_error.restype = C.c_char_p
        L.acdc_last_error.argtypes = [VP]
        L.acdc_status_string.restype = C.c_char_p
        L.acdc_status_string.argtypes = [C.c_int]
        L.acdc_settings_default.argtypes = [C.POINTER(Settings)]
        L.acdc_settings_default.restype = None
        L.acdc_settings_check.argtypes = [C.POINTER(Settings)]
        L.acdc_ctx_create.argtypes = [C.c_int, C.POINTER(VP)]
        L.acdc_ctx_destroy.argtypes = [VP]
        L.acdc_ctx_memory.argtypes = [VP, C.POINTER(I64), C.POINTER(I64)]
        L.acdc_problem_create.argtypes = [VP, I32, I64, I64, VP, VP, VP, VP, D, C.POINTER(VP)]
        L.acdc_problem_create_i32.argtypes = [VP, I32, I64, I64, VP, VP, VP, VP, D, C.POINTER(VP)]
        L.acdc_problem_create_rows.argtypes = [VP, I32, I64, I64, VP, VP, VP, VP, D,
                                               C.POINTER(VP)]
        L.acdc_problem_destroy.argtypes = [VP]
        L.acdc_problem_info_get.argtypes = [VP, C.POINTER(ProblemInfo)]
        L.acdc_problem_set_settings.argtypes = [VP, C.POINTER(Settings)]
        L.acdc_problem_set_lambda.argtypes = [VP, D]
        L.acdc_run_updates.argtypes = [VP, U64]
        L.acdc_recompute_residuals.argtypes = [VP]
        L.acdc_evaluate.argtypes = [VP, C.POINTER(Eval)]
        L.acdc_solve.argtypes = [VP, C.POINTER(SolveResult)]
        L.acdc_checkpoint_size.argtypes = [VP]
        L.acdc_checkpoint_size.restype = I64
        L.acdc_checkpoint_save.argtypes = [VP, VP, I64]
        L.acdc_checkpoint_load.argtypes = [VP, VP, I64]
        L.acdc_solve_traced.argtypes = [VP, C.POINTER(SolveResult), VP, I64, C.POINTER(I64)]
        L.acdc_problem_reset.argtypes = [VP]
        L.acdc_get_x.argtypes = [VP, VP]
        L.acdc_set_x.argtypes = [VP, VP]
        L.acdc_get_residuals.argtypes = [VP, VP]
        L.acdc_get_stats.argtypes = [VP, C.POINTER(Stats)]
        L.acdc_reset_stats.argtypes = [VP]
        L.acdc_synchronize.argtypes = [VP]
        L.acdc_debug_sample.argtypes = [VP, U64, U64, U64, I64, VP]
        L.acdc_test_accuracy.argtypes = [VP, I64, VP, VP, VP, VP, C.POINTER(D)]
        L.acdc_debug_sample_noalloc.argtypes = [VP, U64, U64, U64, I64, VP]
        L.acdc_debug_tau_nice.argtypes = [VP, U64, U64, I64, I32, I32, VP, C.POINTER(U64)]
        L.acdc_server_get_stats.argtypes = [VP, C.c_void_p]
        L.acdc_server_cancel.argtypes = [VP, I64]
        L.acdc_batch_solve_path.argtypes = [VP, I32, VP, VP, C.POINTER(BatchOptions), VP, VP]
        L.acdc_server_create.argtypes = [VP, C.POINTER(ServerOptions), C.POINTER(VP)]
        L.acdc_server_submit.argtypes = [VP, C.POINTER(Request), C.POINTER(I64)]
        L.acdc_server_step.argtypes = [VP, C.POINTER(I32)]
        L.acdc_server_poll.argtypes = [VP, I64, C.POINTER(RequestResult), VP]
        L.acdc_server_release.argtypes = [VP, I64]
        L.acdc_server_destroy.argtypes = [VP]
        _gpu = L
    return _gpu


def host_lib():
    global _host
    if _host is None:
        if not os.path.exists(HOST_LIB):
            raise RuntimeError("libacdc_host.so is missing: run __graft_entry__.build() first")
        H = C.CDLL(HOST_LIB)
        H.acdc_gen_lasso_colptr.argtypes = [C.POINTER(LassoGen), VP]
        H.acdc_gen_lasso_fill.argtypes = [C.POINTER(LassoGen), VP, VP, VP, VP, VP, C.POINTER(D)]
        H.acdc_gen_svm_rowptr.argtypes = [C.POINTER(SvmGen), VP]
        H.acdc_gen_svm_fill.argtypes = [C.POINTER(SvmGen), VP, VP, VP, VP]
        H.acdc_gen_nesterov.argtypes = [I64, I64, I32, I64, D, D, U64, VP, VP, VP, VP, VP,
                                        C.POINTER(D)]
        H.acdc_gen_mix_sizes.argtypes = [U64, I64, I64, I64, I64, I64, C.POINTER(I64),
                                         C.POINTER(I64)]
        H.acdc_host_omega.argtypes = [I64, I64, VP, VP, C.POINTER(I64)]
        H.acdc_philox4x32_10_host.argtypes = [VP, VP, VP]
        H.acdc_philox4x32_10_host.restype = None
        H.acdc_sample_coordinate.argtypes = [U64, U64, U64]
        H.acdc_sample_coordinate.restype = U64
        H.acdc_load_csc_text_sizes.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(I64),
                                               C.POINTER(I64), C.POINTER(I64)]
        H.acdc_load_csc_text.argtypes = [C.c_char_p, C.c_char_p, VP, VP, VP, VP]
        H.acdc_load_csc_binary_sizes.argtypes = [C.c_char_p, C.c_char_p, C.c_int32, C.c_char_p,
                                                 I64, C.POINTER(I64), C.POINTER(I64),
                                                 C.POINTER(I64)]
        H.acdc_load_csc_binary.argtypes = [C.c_char_p, C.c_char_p, C.c_int32, C.c_char_p, I64,
                                           VP, VP, VP, VP]
        H.acdc_load_libsvm_sizes.argtypes = [C.c_char_p, C.POINTER(I64), C.POINTER(I64),
                                             C.POINTER(I64)]
        H.acdc_load_libsvm.argtypes = [C.c_char_p, VP, VP, VP, VP]
        H.acdc_host_threads.argtypes = [I32]
        H.acdc_save_csc_binary.argtypes = [C.c_char_p, C.c_char_p, C.c_int32, I64, VP, VP, VP]
        _host = H
    return _host


def _check_host(rc, what):
    if rc != OK:
        raise AcdcError(rc, what)


# ---------------------------------------------------------------- generators

class Instance:
    """Compressed-column problem data on the host (ProblemData layout)."""

    def __init__(self, loss, m, n, col_ptr, row_idx, vals, rhs, lam, x_star=None, f_star=None):
        self.loss, self.m, self.n = loss, int(m), int(n)
        self.col_ptr, self.row_idx, self.vals, self.rhs = col_ptr, row_idx, vals, rhs
        self.lam = float(lam)
        self.x_star, self.f_star = x_star, f_star

    @property
    def nnz(self):
        return int(self.col_ptr[-1])


def _empty(shape, dtype, pinned):
    if pinned:
        import torch
        t = torch.empty(shape, dtype={np.float64: torch.float64, np.int64: torch.int64,
                                      np.int32: torch.int32}[dtype], pin_memory=True)
        return t.numpy()
    return np.empty(shape, dtype)


def gen_lasso(m, n, nnz_mode=NNZ_FIXED, nnz_per_col=20, zipf_s=1.5, nnz_min=1, nnz_max=2000,
              nnz_mean=20.0, n_star=100, noise_sigma=0.01, lambda_frac=0.1, seed=1,
              normalize=True, threads=0, pinned=False):
    g = LassoGen(m, n, nnz_mode, nnz_per_col, zipf_s, nnz_min, nnz_max, nnz_mean, n_star,
                 noise_sigma, lambda_frac, seed, 1 if normalize else 0, threads)
    H = host_lib()
    col_ptr = _empty(n + 1, np.int64, pinned)
    _check_host(H.acdc_gen_lasso_colptr(C.byref(g), _ptr(col_ptr)), "gen_lasso_colptr")
    nnz = int(col_ptr[-1])
    row_idx = _empty(max(nnz, 1), np.int32, pinned)[:nnz]
    vals = _empty(max(nnz, 1), np.float64, pinned)[:nnz]
    b = _empty(m, np.float64, pinned)
    x_star = np.zeros(n)
    lam = D(0)
    _check_host(H.acdc_gen_lasso_fill(C.byref(g), _ptr(col_ptr), _ptr(row_idx), _ptr(vals),
                                      _ptr(b), _ptr(x_star), C.byref(lam)), "gen_lasso_fill")
    return Instance(LOSS_L1_SQUARE, m, n, col_ptr, row_idx, vals, b, lam.value, x_star=x_star)


def gen_svm(n_samples, d, nnz_median=450.0, nnz_sigma=0.8, w_star_nnz=5000, flip_prob=0.05,
            lam=1e-4, seed=1, threads=0, pinned=False):
    g = SvmGen(n_samples, d, nnz_median, nnz_sigma, w_star_nnz, flip_prob, seed, threads)
    H = host_lib()
    row_ptr = _empty(n_samples + 1, np.int64, pinned)
    _check_host(H.acdc_gen_svm_rowptr(C.byref(g), _ptr(row_ptr)), "gen_svm_rowptr")
    nnz = int(row_ptr[-1])
    col_idx = _empty(nnz, np.int32, pinned)
    vals = _empty(nnz, np.float64, pinned)
    y = _empty(n_samples, np.float64, pinned)
    _check_host(H.acdc_gen_svm_fill(C.byref(g), _ptr(row_ptr), _ptr(col_idx), _ptr(vals), _ptr(y)),
                "gen_svm_fill")
    return Instance(LOSS_SVM_DUAL, d, n_samples, row_ptr, col_idx, vals, y, lam)


def gen_nesterov(m, n, p, n_nonzero, lam=1.0, rho=1.0, seed=1):
    col_ptr = np.zeros(n + 1, np.int64)
    row_idx = np.zeros(n * p, np.int32)
    vals = np.zeros(n * p)
    b = np.zeros(m)
    x_star = np.zeros(n)
    f = D(0)
    _check_host(host_lib().acdc_gen_nesterov(m, n, p, n_nonzero, lam, rho, seed, _ptr(col_ptr),
                                             _ptr(row_idx), _ptr(vals), _ptr(b), _ptr(x_star),
                                             C.byref(f)), "gen_nesterov")
    return Instance(LOSS_L1_SQUARE, m, n, col_ptr, row_idx, vals, b, lam, x_star=x_star,
                    f_star=f.value)


def transpose_compressed(rows, cols, ptr, idx, vals):
    """Compressed rows (rows x cols) -> compressed columns of the same matrix:
    (col_ptr[cols + 1], row_idx, vals), entries of each column in row order."""
    ptr = np.asarray(ptr, np.int64)
    idx = np.asarray(idx, np.int64)
    row_of = np.repeat(np.arange(rows, dtype=np.int64), np.diff(ptr))
    order = np.lexsort((row_of, idx))
    col_ptr = np.zeros(cols + 1, np.int64)
    np.cumsum(np.bincount(idx, minlength=cols), out=col_ptr[1:])
    return col_ptr, row_of[order].astype(np.int32), np.asarray(vals, np.float64)[order]


def logistic_from_svm(sv, lam):
    """An L2-regularised logistic instance (loss 3) from an SVM-generator one:
    samples become the rows and features the coordinates (CSC over features),
    labels the right-hand side, as the reference's MultiCoreSolver.cpp:80-105
    arranges LIBSVM data for this loss."""
    cp, ri, va = transpose_compressed(sv.n, sv.m, sv.col_ptr, sv.row_idx, sv.vals)
    return Instance(LOSS_LOGISTIC, sv.n, sv.m, cp, ri, va, np.array(sv.rhs, np.float64), lam)


def mix_sizes(seed, index, m_lo=500, m_hi=50000, n_lo=1000, n_hi=200000):
    m, n = I64(0), I64(0)
    _check_host(host_lib().acdc_gen_mix_sizes(seed, index, m_lo, m_hi, n_lo, n_hi, C.byref(m),
                                              C.byref(n)), "gen_mix_sizes")
    return m.value, n.value


def host_omega(inst):
    w = I64(0)
    _check_host(host_lib().acdc_host_omega(inst.m, inst.n, _ptr(inst.col_ptr), _ptr(inst.row_idx),
                                           C.byref(w)), "host_omega")
    return max(1, w.value)


def load_csc_text(prefix, vector_file, lam):
    H = host_lib()
    m, n, nnz = I64(0), I64(0), I64(0)
    _check_host(H.acdc_load_csc_text_sizes(prefix.encode(), vector_file.encode(), C.byref(m),
                                           C.byref(n), C.byref(nnz)), "load_csc_text_sizes")
    col_ptr = np.zeros(n.value + 1, np.int64)
    row_idx = np.zeros(nnz.value, np.int32)
    vals = np.zeros(nnz.value)
    b = np.zeros(m.value)
    _check_host(H.acdc_load_csc_text(prefix.encode(), vector_file.encode(), _ptr(col_ptr),
                                     _ptr(row_idx), _ptr(vals), _ptr(b)), "load_csc_text")
    return Instance(LOSS_L1_SQUARE, m.value, n.value, col_ptr, row_idx, vals, b, lam)


def load_csc_binary(prefix, suffix, rank, vector_file, local_n, lam, loss=LOSS_L1_SQUARE):
    """The binary per-rank CSC format (loadANSCIAndBinaryData)."""
    H = host_lib()
    m, n, nnz = I64(0), I64(0), I64(0)
    args = (prefix.encode(), suffix.encode(), int(rank), vector_file.encode(), int(local_n))
    _check_host(H.acdc_load_csc_binary_sizes(*args, C.byref(m), C.byref(n), C.byref(nnz)),
                "load_csc_binary_sizes")
    col_ptr = np.zeros(n.value + 1, np.int64)
    row_idx = np.zeros(nnz.value, np.int32)
    vals = np.zeros(nnz.value)
    b = np.zeros(m.value)
    _check_host(H.acdc_load_csc_binary(*args, _ptr(col_ptr), _ptr(row_idx), _ptr(vals), _ptr(b)),
                "load_csc_binary")
    return Instance(loss, m.value, n.value, col_ptr, row_idx, vals, b, lam)


def save_csc_binary(inst, prefix, suffix="", rank=0):
    """acdc_save_csc_binary: the instance's matrix in the per-rank binary format
    that load_csc_binary reads (the vector file is written separately)."""
    cp = np.ascontiguousarray(inst.col_ptr, np.int64)
    ri = np.ascontiguousarray(inst.row_idx, np.int32)
    va = np.ascontiguousarray(inst.vals, np.float64)
    _check_host(host_lib().acdc_save_csc_binary(prefix.encode(), suffix.encode(), int(rank),
                                                inst.n, _ptr(cp), _ptr(ri) if ri.size else None,
                                                _ptr(va) if va.size else None),
                "save_csc_binary")


def host_threads(threads):
    """Threads of the text loaders (0: one per MiB of text, up to the hardware
    threads); returns the previous setting."""
    return host_lib().acdc_host_threads(int(threads))


def load_libsvm(path, lam):
    H = host_lib()
    n, d, nnz = I64(0), I64(0), I64(0)
    _check_host(H.acdc_load_libsvm_sizes(path.encode(), C.byref(n), C.byref(d), C.byref(nnz)),
                "load_libsvm_sizes")
    row_ptr = np.zeros(n.value + 1, np.int64)
    col_idx = np.zeros(nnz.value, np.int32)
    vals = np.zeros(nnz.value)
    y = np.zeros(n.value)
    _check_host(H.acdc_load_libsvm(path.encode(), _ptr(row_ptr), _ptr(col_idx), _ptr(vals),
                                   _ptr(y)), "load_libsvm")
    return Instance(LOSS_SVM_DUAL, d.value, n.value, row_ptr, col_idx, vals, y, lam)


# ---------------------------------------------------------------- GPU engine

class Context:
    def __init__(self, device=0):
        self.L = gpu_lib()
        h = VP()
        rc = self.L.acdc_ctx_create(device, C.byref(h))
        if rc != OK:
            raise AcdcError(rc, self.L.acdc_status_string(rc).decode())
        self.h = h

    def check(self, rc):
        if rc != OK:
            raise AcdcError(rc, self.L.acdc_last_error(self.h).decode())
        return rc

    def close(self):
        """Destroys the context once no problem created on it is alive."""
        if self.h and self.L.acdc_ctx_destroy(self.h) == OK:
            self.h = None

    def memory(self):
        """(reserved, used) bytes of the context's device memory pool."""
        r, u = I64(0), I64(0)
        self.check(self.L.acdc_ctx_memory(self.h, C.byref(r), C.byref(u)))
        return int(r.value), int(u.value)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def philox_host(ctr, key):
    c = np.ascontiguousarray(ctr, np.uint32)
    k = np.ascontiguousarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    host_lib().acdc_philox4x32_10_host(_ptr(c), _ptr(k), _ptr(out))
    return out


def sample_coordinate(seed, k, n):
    return int(host_lib().acdc_sample_coordinate(seed, k, n))


def debug_sample(ctx, seed, k0, count, n):
    out = np.zeros(count, np.int64)
    ctx.check(ctx.L.acdc_debug_sample(ctx.h, seed, k0, count, n, _ptr(out)))
    return out


def debug_tau_nice(ctx, seed, k0, n, tau, steps):
    """acdc_debug_tau_nice: the mini-batch draws (steps x tau) and the next counter."""
    out = np.zeros((max(steps, 1), tau), np.int32)[:steps]
    k = U64(0)
    ctx.check(ctx.L.acdc_debug_tau_nice(ctx.h, seed, k0, n, tau, steps, _ptr(out), C.byref(k)))
    return out, int(k.value)


NOALLOC_MAX_SAMPLES = 65536  # ACDC_NOALLOC_MAX_SAMPLES


def debug_sample_noalloc(ctx, seed, k0, count, n):
    """acdc_debug_sample_noalloc: the same draws through a fixed device array."""
    out = np.zeros(max(count, 1), np.int64)[:count]
    ctx.check(ctx.L.acdc_debug_sample_noalloc(ctx.h, seed, k0, count, n, _ptr(out)))
    return out


def default_settings(loss=LOSS_L1_SQUARE, **kw):
    s = Settings()
    gpu_lib().acdc_settings_default(C.byref(s))
    s.loss = loss
    if loss == LOSS_SVM_DUAL:
        s.gap_relative = 0
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def settings_ok(s):
    """acdc_settings_check: True when every field of s lies in its range."""
    return gpu_lib().acdc_settings_check(C.byref(s)) == OK


class Problem:
    """One problem resident on the device (x, residual and sampler state).

    With rows=True, inst holds A by rows: col_ptr is the row pointer (m + 1
    entries) and row_idx the column indices (acdc_problem_create_rows)."""

    def __init__(self, ctx, inst, settings=None, rows=False, **kw):
        self.ctx, self.L = ctx, ctx.L
        self.m, self.n, self.loss = inst.m, inst.n, inst.loss
        h = VP()
        cp = inst.col_ptr
        if rows:
            cp = np.ascontiguousarray(cp, np.int64)
            fn = self.L.acdc_problem_create_rows
        elif cp.dtype == np.int32:
            fn = self.L.acdc_problem_create_i32
        else:
            cp = np.ascontiguousarray(cp, np.int64)
            fn = self.L.acdc_problem_create
        ri = np.ascontiguousarray(inst.row_idx, np.int32)
        va = np.ascontiguousarray(inst.vals, np.float64)
        rh = np.ascontiguousarray(inst.rhs, np.float64)
        ctx.check(fn(ctx.h, inst.loss, inst.m, inst.n, _ptr(cp), _ptr(ri) if ri.size else None,
                     _ptr(va) if va.size else None, _ptr(rh), inst.lam, C.byref(h)))
        self.h = h
        if settings is not None or kw:
            self.set_settings(settings or default_settings(inst.loss), **kw)

    def set_settings(self, s=None, **kw):
        s = s or default_settings(self.loss)
        for k, v in kw.items():
            setattr(s, k, v)
        self.ctx.check(self.L.acdc_problem_set_settings(self.h, C.byref(s)))
        self.settings = s

    def set_lambda(self, lam):
        self.ctx.check(self.L.acdc_problem_set_lambda(self.h, lam))

    def info(self):
        i = ProblemInfo()
        self.ctx.check(self.L.acdc_problem_info_get(self.h, C.byref(i)))
        return i

    def run_updates(self, count):
        self.ctx.check(self.L.acdc_run_updates(self.h, int(count)))

    def recompute_residuals(self):
        self.ctx.check(self.L.acdc_recompute_residuals(self.h))

    def evaluate(self):
        e = Eval()
        self.ctx.check(self.L.acdc_evaluate(self.h, C.byref(e)))
        return e.as_dict()

    def solve(self):
        r = SolveResult()
        self.ctx.check(self.L.acdc_solve(self.h, C.byref(r)))
        return r

    def solve_traced(self, cap=100000):
        """acdc_solve_traced: (result, list of per-evaluation row dicts)."""
        r = SolveResult()
        rows = (TraceRow * cap)()
        n = I64(0)
        self.ctx.check(self.L.acdc_solve_traced(self.h, C.byref(r), rows, cap, C.byref(n)))
        return r, [rows[i].as_dict() for i in range(min(n.value, cap))]

    def reset(self):
        self.ctx.check(self.L.acdc_problem_reset(self.h))

    def checkpoint(self):
        """acdc_checkpoint_save: the solver state as bytes."""
        size = self.L.acdc_checkpoint_size(self.h)
        buf = C.create_string_buffer(size)
        self.ctx.check(self.L.acdc_checkpoint_save(self.h, buf, size))
        return buf.raw

    def restore(self, data):
        """acdc_checkpoint_load from bytes made by checkpoint()."""
        buf = C.create_string_buffer(bytes(data), len(data))
        self.ctx.check(self.L.acdc_checkpoint_load(self.h, buf, len(data)))

    def get_x(self):
        x = np.zeros(self.n)
        self.ctx.check(self.L.acdc_get_x(self.h, _ptr(x)))
        return x

    def set_x(self, x):
        x = np.ascontiguousarray(x, np.float64)
        self.ctx.check(self.L.acdc_set_x(self.h, _ptr(x)))

    def get_residuals(self):
        r = np.zeros(self.m)
        self.ctx.check(self.L.acdc_get_residuals(self.h, _ptr(r)))
        return r

    def test_accuracy(self, row_ptr, col_idx, vals, labels):
        """0-1 accuracy on held-out samples (CSR over the features)."""
        rp = np.ascontiguousarray(row_ptr, np.int64)
        ci = np.ascontiguousarray(col_idx, np.int32)
        va = np.ascontiguousarray(vals, np.float64)
        lb = np.ascontiguousarray(labels, np.float64)
        acc = D(0)
        self.ctx.check(self.L.acdc_test_accuracy(self.h, len(rp) - 1, _ptr(rp),
                                                 _ptr(ci) if ci.size else None,
                                                 _ptr(va) if va.size else None, _ptr(lb),
                                                 C.byref(acc)))
        return acc.value

    def stats(self):
        s = Stats()
        self.ctx.check(self.L.acdc_get_stats(self.h, C.byref(s)))
        return s.as_dict()

    def reset_stats(self):
        self.ctx.check(self.L.acdc_reset_stats(self.h))

    def synchronize(self):
        self.ctx.check(self.L.acdc_synchronize(self.h))

    def close(self):
        if self.h:
            self.L.acdc_problem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous batching of solve requests on one context (acdc_server_*)."""

    STATES = ("queued", "running", "done", "failed")

    def __init__(self, ctx, memory_budget_bytes=120 << 30, max_slots=256, quantum_rounds=4,
                 max_epochs=2000, use_shrinking=0):
        self.ctx, self.L = ctx, ctx.L
        opt = ServerOptions(int(memory_budget_bytes), max_slots, quantum_rounds, max_epochs,
                            use_shrinking)
        h = VP()
        ctx.check(self.L.acdc_server_create(ctx.h, C.byref(opt), C.byref(h)))
        self.h = h
        self.n_of = {}

    def submit(self, inst, lam=None, gap_target=1e-6, seed=1):
        cp = np.ascontiguousarray(inst.col_ptr, np.int64)
        ri = np.ascontiguousarray(inst.row_idx, np.int32)
        va = np.ascontiguousarray(inst.vals, np.float64)
        rh = np.ascontiguousarray(inst.rhs, np.float64)
        req = Request(inst.loss, 0, inst.m, inst.n, cp.ctypes.data, ri.ctypes.data if ri.size else None,
                      va.ctypes.data if va.size else None, rh.ctypes.data,
                      float(inst.lam if lam is None else lam), gap_target, seed)
        t = I64()
        self.ctx.check(self.L.acdc_server_submit(self.h, C.byref(req), C.byref(t)))
        self.n_of[t.value] = inst.n
        return t.value

    def step(self):
        pend = I32()
        self.ctx.check(self.L.acdc_server_step(self.h, C.byref(pend)))
        return pend.value

    def stats(self):
        st = ServerStats()
        self.ctx.check(self.L.acdc_server_get_stats(self.h, C.byref(st)))
        return st.as_dict()

    def poll(self, ticket, want_x=False):
        res = RequestResult()
        x = np.zeros(self.n_of[ticket]) if want_x else None
        self.ctx.check(self.L.acdc_server_poll(self.h, ticket, C.byref(res), _ptr(x)))
        return res, x

    def release(self, ticket):
        self.ctx.check(self.L.acdc_server_release(self.h, ticket))

    def cancel(self, ticket):
        self.ctx.check(self.L.acdc_server_cancel(self.h, ticket))

    def close(self):
        if self.h:
            self.L.acdc_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_solve_path(ctx, problems, lambdas, gap_target=1e-6, max_epochs=1000, refresh_every=5,
                     autotune=1, tau_override=0, plain=0, want_x=False, use_shrinking=0,
                     active_passes=0):
    """Solve every problem along its lambda row; returns (results[count][path], xs)."""
    count = len(problems)
    lam = np.ascontiguousarray(lambdas, np.float64).reshape(count, -1)
    path = lam.shape[1]
    opt = BatchOptions(path, max_epochs, gap_target, refresh_every, autotune, tau_override, plain,
                       use_shrinking, active_passes)
    res = (BatchResult * (count * path))()
    handles = (VP * count)(*[p.h for p in problems])
    xs = [np.zeros(p.n) for p in problems] if want_x else None
    xptrs = (VP * count)(*[x.ctypes.data for x in xs]) if want_x else None
    ctx.check(ctx.L.acdc_batch_solve_path(ctx.h, count, handles, _ptr(lam), C.byref(opt), res,
                                          xptrs))
    out = [[res[i * path + k] for k in range(path)] for i in range(count)]
    return out, xs
