"""Batched lambda paths: many instances solved by one launch sequence must give
the same answers as solving each instance alone (the plain one-instance path)
and as the FP64 oracle, within the tolerance of the FP32 engine: objective within
1e-6 relative per lambda, identical support at the end of the path."""
import numpy as np
import pytest

import acdc
import oracle

pytestmark = pytest.mark.gpu

PATH = 4


def make_instances(seed0, count):
    insts = []
    for i in range(count):
        m, n = acdc.mix_sizes(seed0, i, m_lo=300, m_hi=3000, n_lo=600, n_hi=6000)
        inst = acdc.gen_lasso(m, n, nnz_mode=acdc.NNZ_UNIFORM, nnz_min=5, nnz_max=20,
                              n_star=min(20, n // 10), noise_sigma=0.01, lambda_frac=1.0,
                              seed=seed0 * 1000 + i)
        insts.append(inst)
    return insts


def path_for(inst):
    # inst.lam was generated with lambda_frac = 1: lambda_max = ||A^T b||_inf
    return np.array([inst.lam * 0.5 ** k for k in range(1, PATH + 1)])


def solve_batch(ctx, insts, plain, use_shrinking=0):
    probs = [acdc.Problem(ctx, inst) for inst in insts]
    lams = np.stack([path_for(inst) for inst in insts])
    res, xs = acdc.batch_solve_path(ctx, probs, lams, gap_target=1e-6, max_epochs=3000,
                                    refresh_every=2, autotune=1, plain=plain, want_x=True,
                                    use_shrinking=use_shrinking)
    for p in probs:
        p.close()
    return res, xs


def test_batched_equals_plain_per_lambda(ctx):
    insts = make_instances(7, 12)
    rb, xb = solve_batch(ctx, insts, plain=0)
    rp, xp = solve_batch(ctx, insts, plain=1)
    for i in range(len(insts)):
        for k in range(PATH):
            b, p = rb[i][k], rp[i][k]
            assert b.converged and p.converged, (i, k, b.eval.rel_gap, p.eval.rel_gap)
            assert abs(b.lambda_ - p.lambda_) == 0
            assert abs(b.eval.primal - p.eval.primal) <= 1e-6 * abs(p.eval.primal), (i, k)
            assert b.tau == p.tau
        assert set(np.nonzero(xb[i])[0]) == set(np.nonzero(xp[i])[0]), i


@pytest.mark.parametrize("use_shrinking", [0, 1])
def test_batched_path_matches_oracle_warm_started_path(ctx, use_shrinking):
    insts = make_instances(11, 4)
    rb, xb = solve_batch(ctx, insts, plain=0, use_shrinking=use_shrinking)
    for i, inst in enumerate(insts):
        x = None
        for k, lam in enumerate(path_for(inst)):
            x, r, ev, ep = oracle.lasso_solve(inst.m, inst.n, inst.col_ptr, inst.row_idx,
                                              inst.vals, inst.rhs, lam, seed=1, target=1e-10,
                                              x0=x)
            assert rb[i][k].converged, (i, k, rb[i][k].eval.rel_gap)
            assert abs(rb[i][k].eval.primal - ev["primal"]) <= 1e-6 * abs(ev["primal"]), (i, k)
        assert set(np.nonzero(xb[i])[0]) == set(np.nonzero(x)[0]), i


def test_shrinking_batched_equals_shrinking_plain(ctx):
    insts = make_instances(17, 6)
    rb, xb = solve_batch(ctx, insts, plain=0, use_shrinking=1)
    rp, xp = solve_batch(ctx, insts, plain=1, use_shrinking=1)
    for i in range(len(insts)):
        for k in range(PATH):
            b, p = rb[i][k], rp[i][k]
            assert b.converged and p.converged, (i, k, b.eval.rel_gap, p.eval.rel_gap)
            assert abs(b.eval.primal - p.eval.primal) <= 1e-6 * abs(p.eval.primal), (i, k)
        assert set(np.nonzero(xb[i])[0]) == set(np.nonzero(xp[i])[0]), i


def test_batch_mixes_losses_and_sizes(ctx):
    lasso = make_instances(13, 3)
    svm = acdc.gen_svm(800, 6000, nnz_median=60, w_star_nnz=300, lam=1e-3, seed=14)
    insts = lasso + [svm]
    probs = [acdc.Problem(ctx, inst) for inst in insts]
    lams = np.stack([path_for(inst) for inst in lasso] +
                    [np.array([4e-3, 2e-3, 1e-3, 5e-4])])
    res, xs = acdc.batch_solve_path(ctx, probs, lams, gap_target=1e-6, max_epochs=3000,
                                    refresh_every=2, autotune=1, plain=0, want_x=True)
    for p in probs:
        p.close()
    for i in range(len(insts)):
        assert all(r.converged for r in res[i]), [r.eval.rel_gap for r in res[i]]
    # the SVM slot against the oracle at its last lambda (gap 1e-6 relative)
    a, w, ev, ep = oracle.svm_solve(svm.m, svm.n, svm.col_ptr, svm.row_idx, svm.vals, svm.rhs,
                                    5e-4, seed=1, target=1e-10)
    assert abs(res[3][3].eval.primal - ev["primal"]) <= 1e-5 * abs(ev["primal"])
    assert np.all((xs[3] >= 0) & (xs[3] <= 1))


def test_batched_path_at_mix_sizes_matches_oracle(ctx):
    """Three instances of the 512-instance distribution itself (unscaled: 9,292,
    85,384 and 63,997 columns, 5..50 entries per column), the first four lambdas
    of the path, against the oracle's warm-started FP64 path (working-set
    solver to relative gap 1e-10): objective within 1e-6 relative per lambda,
    identical support at the end."""
    sizes = [acdc.mix_sizes(0xACDC0003, i) for i in (0, 2, 4)]
    insts = [acdc.gen_lasso(m, n, nnz_mode=acdc.NNZ_UNIFORM, nnz_min=5, nnz_max=50,
                            n_star=max(1, n // 100), lambda_frac=1.0, seed=0xACDC0003 + i)
             for (m, n), i in zip(sizes, (0, 2, 4))]
    rb, xb = solve_batch(ctx, insts, plain=0, use_shrinking=1)
    for i, inst in enumerate(insts):
        x = None
        for k, lam in enumerate(path_for(inst)):
            x, r, ev, sw, ch = oracle.lasso_solve_ws(inst.m, inst.n, inst.col_ptr, inst.row_idx,
                                                     inst.vals, inst.rhs, lam, target=1e-10,
                                                     rel=True, x0=x)
            assert rb[i][k].converged, (i, k, rb[i][k].eval.rel_gap)
            assert abs(rb[i][k].eval.primal - ev["primal"]) <= 1e-6 * abs(ev["primal"]), (i, k)
        assert set(np.nonzero(xb[i])[0]) == set(np.nonzero(x)[0]), i
