"""acdc_problem_create_rows: the matrix given by rows, turned into the column
layout on the device (a stable radix sort by column index, one to three 8-bit
passes).  The problem it builds must be the one acdc_problem_create builds
from the same matrix in column form: same sizes and padding, the same
evaluations (to the order of the FP64 refresh's atomics) and, with one warp,
the same trajectory (FP32 updates: to FP32 rounding)."""
import numpy as np
import pytest

import acdc

pytestmark = pytest.mark.gpu


def as_rows(inst):
    """The instance's A (m x n) in compressed-row form, rows in order."""
    rp, ci, va = acdc.transpose_compressed(inst.n, inst.m, inst.col_ptr, inst.row_idx, inst.vals)
    return acdc.Instance(inst.loss, inst.m, inst.n, rp, ci, va, inst.rhs, inst.lam)


def lasso(seed, m=700, n=3000):
    return acdc.gen_lasso(m, n, nnz_per_col=9, n_star=30, lambda_frac=0.1, seed=seed)


def same_problem(ctx, cols, rows, x):
    p = acdc.Problem(ctx, cols, tau=1, warps_per_block=1, precision=acdc.PREC_FP64, seed=3)
    q = acdc.Problem(ctx, rows, rows=True, tau=1, warps_per_block=1, precision=acdc.PREC_FP64,
                     seed=3)
    ip, iq = p.info(), q.info()
    assert (ip.m, ip.n, ip.nnz, ip.nnz_padded, ip.omega) == (iq.m, iq.n, iq.nnz, iq.nnz_padded,
                                                             iq.omega)
    p.set_x(x)
    q.set_x(x)
    ep, eq = p.evaluate(), q.evaluate()
    for k in ep:  # the FP64 refresh adds with atomics: equal up to their order
        assert eq[k] == pytest.approx(ep[k], rel=1e-12, abs=1e-12), k
    p.run_updates(3 * cols.n)
    q.run_updates(3 * cols.n)
    np.testing.assert_allclose(q.get_x(), p.get_x(), rtol=1e-5, atol=1e-7)
    p.close()
    q.close()


@pytest.mark.parametrize("n", [3000, 70000])  # two and three radix passes
def test_rows_give_the_column_layout_lasso(ctx, n):
    inst = lasso(11, n=n)
    x = np.zeros(inst.n)
    x[:: max(1, inst.n // 50)] = 0.5
    same_problem(ctx, inst, as_rows(inst), x)


def test_rows_give_the_column_layout_logistic(ctx):
    """LIBSVM-shaped rows (samples x features, labels as rhs) go in as read, the
    arrangement MultiCoreSolver.cpp:80-105 makes on the host for loss 3."""
    sv = acdc.gen_svm(1500, 3000, nnz_median=25, nnz_sigma=0.6, w_star_nnz=150, lam=1e-3, seed=5)
    cols = acdc.logistic_from_svm(sv, 1e-2)
    rows = acdc.Instance(acdc.LOSS_LOGISTIC, sv.n, sv.m, sv.col_ptr, sv.row_idx, sv.vals,
                         np.array(sv.rhs, np.float64), 1e-2)
    x = np.linspace(-0.5, 0.5, cols.n)
    same_problem(ctx, cols, rows, x)


def test_rows_edge_cases(ctx):
    # one row, one column; empty rows; a matrix without entries
    one = acdc.Instance(acdc.LOSS_L1_SQUARE, 1, 1, np.array([0, 1]), np.array([0], np.int32),
                        np.array([2.0]), np.array([1.0]), 0.1)
    q = acdc.Problem(ctx, one, rows=True)
    assert q.info().nnz == 1
    q.close()
    rp = np.array([0, 0, 2, 2, 3], np.int64)  # rows 0 and 2 empty
    ci = np.array([1, 3, 0], np.int32)
    va = np.array([1.0, -2.0, 0.5])
    rows = acdc.Instance(acdc.LOSS_L1_SQUARE, 4, 4, rp, ci, va, np.ones(4), 0.1)
    cp, ri, vv = acdc.transpose_compressed(4, 4, rp, ci, va)
    cols = acdc.Instance(acdc.LOSS_L1_SQUARE, 4, 4, cp, ri, vv, np.ones(4), 0.1)
    same_problem(ctx, cols, rows, np.array([0.0, 1.0, 0.0, -1.0]))
    empty = acdc.Instance(acdc.LOSS_L1_SQUARE, 3, 5, np.zeros(4, np.int64), np.zeros(0, np.int32),
                          np.zeros(0), np.ones(3), 0.1)
    q = acdc.Problem(ctx, empty, rows=True)
    assert q.info().nnz == 0 and q.evaluate()["primal"] == pytest.approx(1.5)
    q.close()


def test_rows_are_checked(ctx):
    inst = as_rows(lasso(12, m=50, n=80))
    bad = acdc.Instance(inst.loss, inst.m, inst.n, inst.col_ptr, inst.row_idx.copy(), inst.vals,
                        inst.rhs, inst.lam)
    bad.row_idx[17] = inst.n  # column out of range: flagged on the device, nothing read outside
    with pytest.raises(acdc.AcdcError) as e:
        acdc.Problem(ctx, bad, rows=True)
    assert e.value.code == acdc.EDEVICE
    rp = inst.col_ptr.copy()
    rp[3], rp[4] = rp[4], rp[3] - 1  # decreasing row pointers: refused on the host
    with pytest.raises(acdc.AcdcError) as e:
        acdc.Problem(ctx, acdc.Instance(inst.loss, inst.m, inst.n, rp, inst.row_idx, inst.vals,
                                        inst.rhs, inst.lam), rows=True)
    assert e.value.code == acdc.EINVAL
    # the context stays usable
    q = acdc.Problem(ctx, inst, rows=True)
    q.close()
