"""The update kernels against each other and against the oracle.

settings.lanes_per_update picks the kernel: -1 the ring kernel, 1 the lean
kernel, 0 (default) the lean kernel for the q-shrinking launches only, 8/16/32
the grouped kernel.  All perform the reference's updates
(MulticoreL1RegSquareLoss.h:41-63, MulticoreSVMDualLoss.h:119-141,
MulticoreL2SquareRegSquareLoss.h:56-78, MulticoreL2SquareRegLogisticLoss.h:88-115)
on the same draws, so:
  * at one update in flight (tau = 1) the ring and lean kernels give identical
    iterates, bit for bit, for every loss, and track the oracle's trajectory;
  * at tau > 1 every kernel solves to the oracle's optimum: objective within
    1e-6 relative, identical support."""
import numpy as np
import pytest

import acdc
import oracle

pytestmark = pytest.mark.gpu


def lasso_instance(seed):
    return acdc.gen_lasso(400, 1500, nnz_per_col=8, n_star=30, seed=seed)


def zipf_lasso_instance(seed, nnz_min=1):
    """About 80% of the columns have at most 4 entries, the tail up to about
    130: both the one-lane and the multi-lane sums of the lean kernel.  With
    nnz_min = 1 many one-entry columns share a row (exact duplicates up to sign,
    so the optimum's support is not unique); from 2 entries there are none."""
    return acdc.gen_lasso(2000, 12000, nnz_mode=acdc.NNZ_ZIPF, zipf_s=1.5, nnz_min=nnz_min,
                          nnz_max=300, nnz_mean=6.0, n_star=60, lambda_frac=0.1, seed=seed)


def svm_instance(seed):
    return acdc.gen_svm(300, 2000, nnz_median=50, w_star_nnz=100, lam=2e-3, seed=seed)


def ridge_instance(seed):
    g = acdc.gen_lasso(600, 2000, nnz_per_col=8, n_star=40, lambda_frac=0.1, seed=seed)
    return acdc.Instance(acdc.LOSS_L2_SQUARE, g.m, g.n, g.col_ptr, g.row_idx, g.vals, g.rhs, 0.3)


def logistic_instance(seed):
    sv = acdc.gen_svm(1500, 3000, nnz_median=25, nnz_sigma=0.6, w_star_nnz=150, lam=1e-3,
                      seed=seed)
    return acdc.logistic_from_svm(sv, 1e-2)


def one_warp_x(ctx, inst, lanes, epochs=3):
    p = acdc.Problem(ctx, inst, tau=1, warps_per_block=1, seed=77, sigma=1.0,
                     lanes_per_update=lanes)
    for _ in range(epochs):
        p.run_updates(inst.n)
    x = p.get_x()
    ev = p.evaluate()
    p.close()
    return x, ev


@pytest.mark.parametrize("make", [lasso_instance, zipf_lasso_instance, svm_instance,
                                  ridge_instance, logistic_instance])
def test_lean_and_ring_kernels_give_identical_iterates_at_one_update_in_flight(ctx, make):
    inst = make(201)
    x_ring, ev_ring = one_warp_x(ctx, inst, -1)
    x_lean, ev_lean = one_warp_x(ctx, inst, 1)
    np.testing.assert_array_equal(x_lean, x_ring)
    assert ev_lean["primal"] == ev_ring["primal"]


def test_lean_kernel_trajectory_tracks_serial_oracle(ctx):
    inst = zipf_lasso_instance(202)
    O = oracle.Lasso(inst.m, inst.n, inst.col_ptr, inst.row_idx, inst.vals, inst.rhs, inst.lam)
    p = acdc.Problem(ctx, inst, tau=1, warps_per_block=1, seed=77, lanes_per_update=1)
    for _ in range(3):
        p.run_updates(inst.n)
        O.updates(inst.n, 77)
        ev = p.evaluate()
        O.refresh()
        want = O.evaluate()
        assert abs(ev["primal"] - want["primal"]) <= 1e-4 * abs(want["primal"])
    assert np.abs(p.get_x() - O.x).max() <= 1e-3 * max(1.0, np.abs(O.x).max())
    assert p.stats()["updates"] == 3 * inst.n
    p.close()


def long_and_empty_instance():
    """Columns of 0, 1, 3, 129, 700 and 2999 entries (longer than one 128-entry
    chunk, and empty) and a dense row."""
    m, n = 3000, 400
    rng = np.random.default_rng(5)
    cols = []
    for j in range(n):
        k = [0, 1, 3, 129, 700, 2999][j % 6] if j % 7 else 0
        rows = np.sort(rng.choice(m, size=k, replace=False))
        v = rng.normal(size=k)
        if k:
            v /= np.linalg.norm(v)
        cols.append((rows, v))
    cp = np.concatenate([[0], np.cumsum([len(c[0]) for c in cols])]).astype(np.int64)
    ri = np.concatenate([c[0] for c in cols]).astype(np.int32)
    va = np.concatenate([c[1] for c in cols])
    b = rng.normal(size=m)
    lam = 0.3 * max(abs(va[cp[j]:cp[j + 1]] @ b[ri[cp[j]:cp[j + 1]]]) for j in range(n))
    return acdc.Instance(acdc.LOSS_L1_SQUARE, m, n, cp, ri, va, b, lam)


def test_lean_kernel_long_and_empty_columns(ctx):
    inst = long_and_empty_instance()
    x_ring, _ = one_warp_x(ctx, inst, -1, epochs=5)
    x_lean, _ = one_warp_x(ctx, inst, 1, epochs=5)
    np.testing.assert_array_equal(x_lean, x_ring)
    x_o, r, ev_o, ep = oracle.lasso_solve(inst.m, inst.n, inst.col_ptr, inst.row_idx, inst.vals,
                                          inst.rhs, inst.lam, seed=1, target=1e-9)
    p = acdc.Problem(ctx, inst, tau=16, warps_per_block=8, gap_target=1e-8, gap_relative=1,
                     refresh_every=5, max_epochs=20000, seed=2, lanes_per_update=1)
    res = p.solve()
    assert res.converged, (res.eval.rel_gap, res.epochs)
    assert abs(res.eval.primal - ev_o["primal"]) <= 1e-6 * abs(ev_o["primal"])
    x = p.get_x()
    assert set(np.nonzero(x)[0]) == set(np.nonzero(x_o)[0])
    assert np.all(x[np.diff(inst.col_ptr) == 0] == 0)
    p.close()


@pytest.mark.parametrize("lanes", [-1, 0, 1, 8, 16, 32])
def test_every_kernel_solves_a_shrinking_lasso_to_the_oracle_optimum(ctx, lanes):
    inst = zipf_lasso_instance(203, nnz_min=2)
    x_o, r, ev_o, ep = oracle.lasso_solve(inst.m, inst.n, inst.col_ptr, inst.row_idx, inst.vals,
                                          inst.rhs, inst.lam, seed=1, target=1e-10)
    p = acdc.Problem(ctx, inst, tau=128, tau_active=64, warps_per_block=8, gap_target=1e-7,
                     gap_relative=1, refresh_every=2, max_epochs=5000, use_shrinking=1,
                     shrinking_probability=0.9, shrinking_starting_iter=2, seed=4,
                     lanes_per_update=lanes)
    res = p.solve()
    assert res.converged, (lanes, res.eval.rel_gap, res.epochs)
    assert res.eval.active > 0
    assert abs(res.eval.primal - ev_o["primal"]) <= 1e-6 * abs(ev_o["primal"])
    assert set(np.nonzero(p.get_x())[0]) == set(np.nonzero(x_o)[0])
    p.close()


@pytest.mark.parametrize("lanes", [1, 8, 32])
def test_every_kernel_solves_the_svm_dual_to_the_oracle_optimum(ctx, lanes):
    inst = acdc.gen_svm(800, 6000, nnz_median=60, w_star_nnz=300, lam=1e-3, seed=204)
    a_o, w_o, ev_o, ep = oracle.svm_solve(inst.m, inst.n, inst.col_ptr, inst.row_idx, inst.vals,
                                          inst.rhs, inst.lam, seed=1, target=1e-10)
    p = acdc.Problem(ctx, inst, tau=64, warps_per_block=8, gap_target=1e-6, gap_relative=1,
                     refresh_every=2, max_epochs=5000, seed=5, lanes_per_update=lanes)
    res = p.solve()
    assert res.converged, (lanes, res.eval.rel_gap, res.epochs)
    assert abs(res.eval.primal - ev_o["primal"]) <= 1e-5 * abs(ev_o["primal"])
    a = p.get_x()
    assert np.all((a >= 0) & (a <= 1))
    p.close()
