"""Losses 1 (L2-regularised square, MulticoreL2SquareRegSquareLoss) and 3
(L2-regularised logistic, MulticoreL2SquareRegLogisticLoss) on the GPU against
the oracle, which is pinned bit for bit to the reference engine.

Tolerances (FP32 device state against the FP64 oracle), as for losses 0 and 2:
  * FP64 evaluation of a given x: 1e-10 relative against the oracle run on the
    FP32-rounded values the device stores;
  * one-warp (tau = 1) trajectory: the device visits the oracle's coordinate
    sequence, so after a few epochs the objectives agree to 1e-4 relative;
  * solves reach the oracle's optimum (gap 1e-10) within 1e-6 relative."""
import numpy as np
import pytest

import acdc
import oracle

pytestmark = pytest.mark.gpu


def ridge_instance(seed):
    g = acdc.gen_lasso(600, 2000, nnz_per_col=8, n_star=40, lambda_frac=0.1, seed=seed)
    return acdc.Instance(acdc.LOSS_L2_SQUARE, g.m, g.n, g.col_ptr, g.row_idx, g.vals, g.rhs, 0.3)


def logistic_instance(seed, lam=1e-2):
    sv = acdc.gen_svm(1500, 3000, nnz_median=25, nnz_sigma=0.6, w_star_nnz=150, lam=1e-3,
                      seed=seed)
    return acdc.logistic_from_svm(sv, lam)


def oracle_of(inst, vals=None, sigma=1.0, x0=None):
    return oracle.Smooth(inst.loss, inst.m, inst.n, inst.col_ptr, inst.row_idx,
                         inst.vals if vals is None else vals, inst.rhs, inst.lam, sigma=sigma,
                         x0=x0)


@pytest.mark.parametrize("make", [ridge_instance, logistic_instance])
def test_evaluate_matches_oracle_fp64(ctx, make):
    inst = make(101)
    rng = np.random.default_rng(2)
    x = np.zeros(inst.n)
    pick = rng.choice(inst.n, inst.n // 4, replace=False)
    x[pick] = rng.normal(scale=0.5, size=pick.size).astype(np.float32)
    p = acdc.Problem(ctx, inst)
    p.set_x(x)
    ev = p.evaluate()
    want = oracle_of(inst, vals=inst.vals.astype(np.float32).astype(np.float64), x0=x).evaluate()
    for k in ("primal", "dual", "gap", "reg_norm", "sq_norm", "zero_one_accuracy"):
        assert abs(ev[k] - want[k]) <= 1e-10 * max(1.0, abs(want[k])), (k, ev[k], want[k])
    assert ev["support"] == pick.size
    p.close()


@pytest.mark.parametrize("make", [ridge_instance, logistic_instance])
def test_one_warp_trajectory_tracks_serial_oracle(ctx, make):
    inst = make(102)
    p = acdc.Problem(ctx, inst, tau=1, warps_per_block=1, seed=77, sigma=1.0)
    O = oracle_of(inst)
    for _ in range(3):
        p.run_updates(inst.n)
        O.updates(inst.n, 77)
        ev = p.evaluate()
        O.refresh()
        want = O.evaluate()
        assert abs(ev["primal"] - want["primal"]) <= 1e-4 * abs(want["primal"])
    x = p.get_x()
    assert np.abs(x - O.x).max() <= 1e-3 * max(1.0, np.abs(O.x).max())
    p.close()


@pytest.mark.parametrize("make,tau", [(ridge_instance, 64), (logistic_instance, 64),
                                      (logistic_instance, 1)])
def test_solution_parity(ctx, make, tau):
    inst = make(103)
    x_o, r_o, ev_o, ep = oracle.smooth_solve(inst.loss, inst.m, inst.n, inst.col_ptr, inst.row_idx,
                                             inst.vals, inst.rhs, inst.lam, target=1e-10,
                                             max_epochs=50000)
    assert ev_o["rel_gap"] <= 1e-10
    p = acdc.Problem(ctx, inst, tau=tau, warps_per_block=min(8, tau), gap_target=1e-8,
                     gap_relative=1, refresh_every=2, max_epochs=20000, seed=5)
    r = p.solve()
    assert r.converged, (r.eval.rel_gap, r.epochs, r.fp64_epochs)
    assert abs(r.eval.primal - ev_o["primal"]) <= 1e-6 * abs(ev_o["primal"])
    assert r.eval.gap >= -1e-9 * abs(r.eval.primal)
    if inst.loss == acdc.LOSS_LOGISTIC:
        assert abs(r.eval.zero_one_accuracy - ev_o["zero_one_accuracy"]) <= 2.0 / inst.m
    np.testing.assert_allclose(p.get_x(), x_o, atol=1e-3 * max(1.0, np.abs(x_o).max()))
    p.close()


def test_lambda_change_recomputes_the_step_sizes(ctx):
    """Losses 1 and 3 keep lambda in Li: a new lambda must give the oracle's
    optimum for that lambda, warm-started."""
    inst = ridge_instance(104)
    p = acdc.Problem(ctx, inst, tau=32, warps_per_block=8, gap_target=1e-9, gap_relative=1,
                     refresh_every=2, max_epochs=20000, seed=6)
    assert p.solve().converged
    p.set_lambda(0.05)
    r = p.solve()
    assert r.converged
    x_o, r_o, ev_o, ep = oracle.smooth_solve(inst.loss, inst.m, inst.n, inst.col_ptr, inst.row_idx,
                                             inst.vals, inst.rhs, 0.05, target=1e-11,
                                             max_epochs=50000)
    assert abs(r.eval.primal - ev_o["primal"]) <= 1e-6 * abs(ev_o["primal"])
    p.close()


def split_rows(sv, n_train):
    """First n_train samples of an SVM-generator instance, and the rest as CSR."""
    cp = sv.col_ptr
    train = acdc.Instance(acdc.LOSS_SVM_DUAL, sv.m, n_train, cp[:n_train + 1].copy(),
                          sv.row_idx[:cp[n_train]].copy(), sv.vals[:cp[n_train]].copy(),
                          sv.rhs[:n_train].copy(), sv.lam)
    s = cp[n_train]
    test = (cp[n_train:] - s, sv.row_idx[s:], sv.vals[s:], sv.rhs[n_train:])
    return train, test


def margins_accuracy(test, w):
    rp, ci, va, y = test
    s = np.array([va[rp[i]:rp[i + 1]] @ w[ci[rp[i]:rp[i + 1]]] for i in range(len(rp) - 1)])
    return np.mean(y * s > 0)


def test_test_set_accuracy_svm_and_logistic(ctx):
    """acdc_test_accuracy: the SVM's w (from the FP64 refresh of alpha) or the
    logistic model's x applied to held-out samples, against numpy margins on the
    same model (FP32-rounded training values, as the device stores them)."""
    # 800 features, 2400 training samples: the oracle's exact solutions reach
    # 0.78 held-out accuracy on both losses (4000 features only reach 0.6)
    sv = acdc.gen_svm(3000, 800, nnz_median=60, nnz_sigma=0.6, w_star_nnz=80, lam=1e-3, seed=105)
    train, test = split_rows(sv, 2400)
    p = acdc.Problem(ctx, train, tau=64, warps_per_block=8, gap_target=1e-6, gap_relative=0,
                     max_epochs=2000, seed=4)
    assert p.solve().converged
    a = p.get_x()
    v32 = train.vals.astype(np.float32).astype(np.float64)
    w = np.zeros(train.m)
    for i in range(train.n):
        s, e = train.col_ptr[i], train.col_ptr[i + 1]
        w[train.row_idx[s:e]] += a[i] * train.rhs[i] * v32[s:e] / (train.lam * train.n)
    acc = p.test_accuracy(*test)
    want = margins_accuracy(test, w)
    assert abs(acc - want) <= 1.0 / (len(test[0]) - 1)
    assert acc > 0.7  # labels of a sparse w* with 5% flips: well above chance
    p.close()

    lg = acdc.logistic_from_svm(train, 1e-2)
    q = acdc.Problem(ctx, lg, tau=32, warps_per_block=8, gap_target=1e-7, gap_relative=1,
                     max_epochs=20000, seed=4)
    assert q.solve().converged
    acc = q.test_accuracy(*test)
    assert abs(acc - margins_accuracy(test, q.get_x())) <= 1.0 / (len(test[0]) - 1)
    assert acc > 0.7
    with pytest.raises(acdc.AcdcError) as e:
        acdc.Problem(ctx, ridge_instance(106)).test_accuracy(*test)
    assert e.value.code == acdc.EUNSUPPORTED
    q.close()
