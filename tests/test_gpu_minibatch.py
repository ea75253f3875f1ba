"""Synchronous mini-batch SDCA (settings.minibatch = 1, hinge-loss dual) through
the C-ABI against the oracle's restatement of the reference's mini-batch loop
(cpp/src/experiments/mSDCA.cpp:60-105: tau distinct draws per step, every delta
from the same w, then all applied).

Tolerances:
  * the device's tau-nice draws equal the oracle's exactly (integer work);
  * FP64 mode against the oracle run on the FP32-rounded values and step
    constants the device stores: alpha within 1e-9 after two epochs (the steps
    are synchronous, so only the order of the FP64 additions into w differs);
  * FP32 mode: alpha within 1e-4 after two epochs;
  * a solve to an absolute gap of 1e-6 reaches the oracle's optimum objective
    within 1e-5 relative.
"""
import numpy as np
import pytest

import acdc
import oracle

pytestmark = pytest.mark.gpu


def small_svm(seed=71):
    return acdc.gen_svm(1500, 12000, nnz_median=60, nnz_sigma=0.8, w_star_nnz=300, lam=1e-3,
                        seed=seed)


@pytest.mark.parametrize("n,tau,steps,k0", [(50, 20, 7, 0), (50, 50, 3, 11), (1000, 1, 5, 3),
                                            (20000, 1024, 4, 123456), (3, 2, 40, 0),
                                            (1 << 22, 4096, 2, 7)])
def test_tau_nice_draws_equal_the_oracle(ctx, n, tau, steps, k0):
    got, k_dev = acdc.debug_tau_nice(ctx, 0xACDC0002, k0, n, tau, steps)
    want, k_orc = oracle.tau_nice(0xACDC0002, k0, n, tau, steps)
    np.testing.assert_array_equal(got, want)
    assert k_dev == k_orc
    for row in got:
        assert len(set(row.tolist())) == tau and row.min() >= 0 and row.max() < n


def oracle_like_device(sv, beta):
    """The oracle on the values and step constants the device holds: FP32
    values, Li = 1/(beta ||x_i||^2) (the norm of the FP64 input) rounded to FP32."""
    v32 = sv.vals.astype(np.float32).astype(np.float64)
    O = oracle.SVM(sv.m, sv.n, sv.col_ptr, sv.row_idx, v32, sv.rhs, sv.lam)
    sq = np.add.reduceat(sv.vals * sv.vals, sv.col_ptr[:-1]) * (np.diff(sv.col_ptr) > 0)
    with np.errstate(divide="ignore"):
        li = np.where(sq > 0, 1.0 / (beta * sq), 0.0)
    O.Li[:] = li.astype(np.float32).astype(np.float64)
    return O


@pytest.mark.parametrize("precision,tol", [(acdc.PREC_FP64, 1e-9), (acdc.PREC_FP32, 1e-4)])
def test_minibatch_trajectory_matches_the_oracle(ctx, precision, tol):
    sv = small_svm()
    tau, seed = 64, 5
    p = acdc.Problem(ctx, sv, tau=tau, minibatch=1, precision=precision, gap_target=0.0,
                     gap_relative=0, refresh_every=1, max_epochs=2, seed=seed)
    beta = p.info().sigma
    r = p.solve()
    assert r.epochs == 2
    O = oracle_like_device(sv, beta)
    O.minibatch(2 * ((sv.n + tau - 1) // tau), seed, tau)
    np.testing.assert_allclose(p.get_x(), O.x, rtol=0, atol=tol)
    O.refresh()
    want = O.evaluate()
    assert abs(r.eval.primal - want["primal"]) <= 10 * tol * abs(want["primal"])
    p.close()


def test_minibatch_solve_reaches_the_oracle_optimum(ctx):
    sv = small_svm(72)
    a_o, w_o, ev_o, _ = oracle.svm_solve(sv.m, sv.n, sv.col_ptr, sv.row_idx, sv.vals, sv.rhs,
                                         sv.lam, seed=1, target=1e-10)
    p = acdc.Problem(ctx, sv, tau=256, minibatch=1, gap_target=1e-6, gap_relative=0,
                     refresh_every=1, max_epochs=3000, seed=9)
    r = p.solve()
    assert r.converged, r.eval.gap
    assert abs(r.eval.primal - ev_o["primal"]) <= 1e-5 * abs(ev_o["primal"])
    a = p.get_x()
    assert np.all((a >= 0) & (a <= 1))
    p.close()


def test_minibatch_checkpoint_continues_the_same_draws(ctx):
    sv = small_svm(73)
    kw = dict(tau=32, minibatch=1, precision=acdc.PREC_FP64, gap_target=0.0, gap_relative=0,
              refresh_every=1, seed=3)
    p = acdc.Problem(ctx, sv, max_epochs=2, **kw)
    p.solve()
    ck = p.checkpoint()
    p.set_settings(acdc.default_settings(acdc.LOSS_SVM_DUAL, max_epochs=1, **kw))
    p.solve()
    a1 = p.get_x()
    q = acdc.Problem(ctx, sv, max_epochs=1, **kw)
    q.restore(ck)
    q.solve()
    np.testing.assert_allclose(q.get_x(), a1, rtol=0, atol=1e-12)
    p.close()
    q.close()
