"""GPU parity: the CUDA path through the C-ABI against the CPU oracle (which is
itself pinned bit-for-bit to the reference's engine).

Tolerances (FP32 device state against the FP64 oracle):
  * final objective within 1e-6 relative of the oracle's FP64 optimum (gap 1e-9),
    identical support set;
  * one-warp (tau = 1) trajectories: the device visits the oracle's coordinate
    sequence, so after a few epochs objectives agree to 1e-4 relative;
  * FP64 evaluation of a given x: 1e-10 relative against the oracle run on the
    FP32-rounded matrix values the device stores.
"""
import json
import os

import numpy as np
import pytest

import acdc
import oracle

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def oracle_optimum(inst, target=1e-9):
    if inst.loss == acdc.LOSS_L1_SQUARE:
        x, r, ev, ep = oracle.lasso_solve(inst.m, inst.n, inst.col_ptr, inst.row_idx, inst.vals,
                                          inst.rhs, inst.lam, seed=1, target=target)
    else:
        x, r, ev, ep = oracle.svm_solve(inst.m, inst.n, inst.col_ptr, inst.row_idx, inst.vals,
                                        inst.rhs, inst.lam, seed=1, target=target)
    return x, ev


def f32_values(inst):
    return inst.vals.astype(np.float32).astype(np.float64)


def test_device_sampler_draws_the_oracle_sequence(ctx):
    for seed, n in ((0, 10), (0xACDC0001, 10**7), (12345, 2**33 + 7)):
        got = acdc.debug_sample(ctx, seed, 1000, 4096, n)
        want = [oracle.sample(seed, 1000 + k, n) for k in range(4096)]
        assert got.tolist() == want


def test_evaluate_matches_oracle_fp64(ctx):
    inst = acdc.gen_lasso(700, 2500, nnz_per_col=9, n_star=40, seed=31)
    x = np.zeros(inst.n)
    rng = np.random.default_rng(0)
    x[rng.choice(inst.n, 200, replace=False)] = rng.normal(size=200).astype(np.float32)
    p = acdc.Problem(ctx, inst)
    p.set_x(x)
    ev = p.evaluate()
    L = oracle.Lasso(inst.m, inst.n, inst.col_ptr, inst.row_idx, f32_values(inst), inst.rhs,
                     inst.lam, x0=x)
    want = L.evaluate()
    for k in ("primal", "dual", "gap", "max_abs_grad", "reg_norm", "sq_norm"):
        assert abs(ev[k] - want[k]) <= 1e-10 * max(1.0, abs(want[k])), k
    assert ev["support"] == 200
    np.testing.assert_allclose(p.get_residuals(), L.r, rtol=1e-6, atol=1e-6)
    np.testing.assert_array_equal(p.get_x(), x)


def test_svm_evaluate_matches_oracle_fp64(ctx):
    sv = acdc.gen_svm(400, 3000, nnz_median=40, w_star_nnz=150, lam=1e-3, seed=32)
    rng = np.random.default_rng(1)
    a = rng.uniform(0, 1, sv.n).astype(np.float32).astype(np.float64)
    a[rng.choice(sv.n, 100, replace=False)] = 0
    p = acdc.Problem(ctx, sv)
    p.set_x(a)
    ev = p.evaluate()
    S = oracle.SVM(sv.m, sv.n, sv.col_ptr, sv.row_idx, f32_values(sv), sv.rhs, sv.lam, alpha0=a)
    want = S.evaluate()
    for k in ("primal", "dual", "gap", "zero_one_accuracy", "reg_norm", "sq_norm"):
        assert abs(ev[k] - want[k]) <= 1e-10 * max(1.0, abs(want[k])), k


@pytest.mark.parametrize("loss", [acdc.LOSS_L1_SQUARE, acdc.LOSS_SVM_DUAL])
def test_one_warp_trajectory_tracks_serial_oracle(ctx, loss):
    if loss == acdc.LOSS_L1_SQUARE:
        inst = acdc.gen_lasso(400, 1500, nnz_per_col=8, n_star=30, seed=41)
        O = oracle.Lasso(inst.m, inst.n, inst.col_ptr, inst.row_idx, inst.vals, inst.rhs, inst.lam)
    else:
        inst = acdc.gen_svm(300, 2000, nnz_median=50, w_star_nnz=100, lam=2e-3, seed=42)
        O = oracle.SVM(inst.m, inst.n, inst.col_ptr, inst.row_idx, inst.vals, inst.rhs, inst.lam)
    p = acdc.Problem(ctx, inst, tau=1, warps_per_block=1, seed=77)
    for epoch in range(3):
        p.run_updates(inst.n)
        O.updates(inst.n, 77)
        ev = p.evaluate()
        O.refresh()
        want = O.evaluate()
        assert abs(ev["primal"] - want["primal"]) <= 1e-4 * abs(want["primal"])
    x = p.get_x()
    assert np.abs(x - O.x).max() <= 1e-3 * max(1.0, np.abs(O.x).max())
    st = p.stats()
    assert st["updates"] == 3 * inst.n


@pytest.mark.parametrize("tau", [1, 32, 256])
def test_config0_solution_parity(ctx, tau):
    """Config 0 (2,000 x 10,000, 20 per column): objective within 1e-6 relative
    of the FP64 oracle's optimum and of the reference engine's solution, same
    support."""
    rec = json.load(open(os.path.join(GOLDEN, "lasso_config0.json")))
    g = rec["generator"]
    inst = acdc.gen_lasso(g["m"], g["n"], nnz_per_col=g["nnz_per_col"], n_star=g["n_star"],
                          noise_sigma=g["noise_sigma"], lambda_frac=g["lambda_frac"], seed=g["seed"])
    x_o, ev_o = oracle_optimum(inst)
    p = acdc.Problem(ctx, inst, tau=tau, warps_per_block=min(8, tau), gap_target=1e-7,
                     gap_relative=1, refresh_every=2, max_epochs=3000, seed=5)
    r = p.solve()
    assert r.converged, (r.eval.rel_gap, r.epochs)
    assert abs(r.eval.primal - ev_o["primal"]) <= 1e-6 * abs(ev_o["primal"])
    x = p.get_x()
    assert set(np.nonzero(x)[0]) == set(np.nonzero(x_o)[0])
    # against the reference's own serial solver (fixture written from its engine)
    assert abs(r.eval.primal - rec["objective"]) <= 1e-6 * abs(rec["objective"])
    assert sorted(np.nonzero(x)[0].tolist()) == rec["support"]


def test_nesterov_known_optimum_on_gpu(ctx):
    inst = acdc.gen_nesterov(2000, 6000, 10, 300, lam=1.0, rho=1.0, seed=51)
    p = acdc.Problem(ctx, inst, tau=64, warps_per_block=8, gap_target=1e-8, gap_relative=1,
                     refresh_every=2, max_epochs=4000, seed=3)
    r = p.solve()
    assert r.converged, (r.eval.rel_gap, r.epochs, r.fp64_epochs)
    assert abs(r.eval.primal - inst.f_star) <= 1e-6 * inst.f_star
    x = p.get_x()
    assert set(np.nonzero(x)[0]) == set(np.nonzero(inst.x_star)[0])


def test_svm_solution_parity(ctx):
    sv = acdc.gen_svm(2000, 40000, nnz_median=120, nnz_sigma=0.8, w_star_nnz=800, lam=1e-3, seed=61)
    a_o, ev_o = oracle_optimum(sv, target=1e-9)
    p = acdc.Problem(ctx, sv, tau=64, warps_per_block=8, gap_target=1e-6, gap_relative=0,
                     refresh_every=2, max_epochs=2000, seed=8)
    r = p.solve()
    assert r.converged, r.eval.gap
    assert abs(r.eval.primal - ev_o["primal"]) <= 1e-5 * abs(ev_o["primal"])
    assert abs(r.eval.dual - ev_o["dual"]) <= 1e-5 * abs(ev_o["dual"])
    a = p.get_x()
    assert np.all((a >= 0) & (a <= 1))


def test_long_and_empty_columns(ctx):
    """Columns longer than one 128-entry chunk, empty columns and a dense row."""
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
    inst = acdc.Instance(acdc.LOSS_L1_SQUARE, m, n, cp, ri, va, b, lam)
    x_o, ev_o = oracle_optimum(inst)
    p = acdc.Problem(ctx, inst, tau=16, warps_per_block=8, gap_target=1e-8, gap_relative=1,
                     refresh_every=5, max_epochs=20000, seed=2)
    r = p.solve()
    assert r.converged, (r.eval.rel_gap, r.epochs, r.fp64_epochs)
    assert abs(r.eval.primal - ev_o["primal"]) <= 1e-6 * abs(ev_o["primal"])
    x = p.get_x()
    assert set(np.nonzero(x)[0]) == set(np.nonzero(x_o)[0])
    assert np.all(x[np.diff(cp) == 0] == 0)
    info = p.info()
    assert info.nnz == cp[-1] and info.nnz_padded % 4 == 0
    assert info.omega == oracle.omega(m, n, cp, ri)


def test_int32_column_pointers_and_warm_start(ctx):
    inst = acdc.gen_lasso(800, 3000, nnz_per_col=10, n_star=40, seed=71)
    x_o, ev_o = oracle_optimum(inst)
    i32 = acdc.Instance(inst.loss, inst.m, inst.n, inst.col_ptr.astype(np.int32), inst.row_idx,
                        inst.vals, inst.rhs, inst.lam)
    p = acdc.Problem(ctx, i32, tau=32, warps_per_block=8, gap_target=1e-6, refresh_every=2,
                     max_epochs=3000)
    p.set_x(x_o)  # warm start at the optimum: converged before any update
    r = p.solve()
    assert r.converged and r.epochs <= 2


def test_shrinking_keeps_the_solution(ctx):
    inst = acdc.gen_lasso(3000, 30000, nnz_per_col=15, n_star=150, lambda_frac=0.1, seed=81)
    x_o, ev_o = oracle_optimum(inst)
    p = acdc.Problem(ctx, inst, tau=256, warps_per_block=8, gap_target=1e-7, refresh_every=2,
                     max_epochs=3000, use_shrinking=1, shrinking_probability=0.9,
                     shrinking_starting_iter=2, seed=4)
    r = p.solve()
    assert r.converged, (r.eval.rel_gap, r.epochs, r.fp64_epochs)
    assert r.eval.active > 0
    assert abs(r.eval.primal - ev_o["primal"]) <= 1e-6 * abs(ev_o["primal"])
    assert set(np.nonzero(p.get_x())[0]) == set(np.nonzero(x_o)[0])


@pytest.mark.parametrize("precision", [acdc.PREC_AUTO, acdc.PREC_FP64])
def test_screened_evaluations_certify_the_gap(ctx, precision):
    """Evaluations that read only the active columns report a duality gap no
    smaller than the full pass's on the same iterate, and the solve they stop
    reaches the oracle's optimum and support."""
    inst = acdc.gen_lasso(4000, 40000, nnz_mode=acdc.NNZ_ZIPF, zipf_s=1.5, nnz_min=3,
                          nnz_max=400, nnz_mean=12.0, n_star=60, lambda_frac=0.1, seed=83)
    x_o, ev_o = oracle_optimum(inst, target=1e-10)
    kw = dict(tau=256, warps_per_block=8, gap_target=1e-7, refresh_every=2, max_epochs=5000,
              use_shrinking=1, shrinking_probability=0.9, shrinking_starting_iter=2, seed=5,
              tau_active=64, active_passes=10, precision=precision)
    p = acdc.Problem(ctx, inst, screened_eval=1, **kw)
    r = p.solve()
    assert r.converged, (r.eval.rel_gap, r.epochs)
    assert r.stats.screened_evals > 0
    full = p.evaluate()
    assert full["primal"] == pytest.approx(r.eval.primal, rel=1e-12)
    assert full["rel_gap"] <= r.eval.rel_gap * (1 + 1e-9) + 1e-15
    assert abs(r.eval.primal - ev_o["primal"]) <= 1e-6 * abs(ev_o["primal"])
    x = p.get_x()
    assert set(np.nonzero(x)[0]) == set(np.nonzero(x_o)[0])
    # the same solve with full evaluations only
    q = acdc.Problem(ctx, inst, screened_eval=0, **kw)
    rq = q.solve()
    assert rq.converged and rq.stats.screened_evals == 0
    assert abs(rq.eval.primal - ev_o["primal"]) <= 1e-6 * abs(ev_o["primal"])
    q.close()
    p.close()


def test_hot_polish_certifies_the_fp64_iterate(ctx):
    """FP32 bulks with the FP64 polish of the hot columns (hot_polish_sweeps):
    on this instance the FP32 iterate alone stalls near a 1.2e-6 gap, while the
    polish certifies 1e-7.  The certificate is that of the iterate the solve
    leaves (x in FP64), which the full evaluation afterwards reproduces, and the
    solution is the oracle's."""
    inst = acdc.gen_lasso(4000, 40000, nnz_mode=acdc.NNZ_ZIPF, zipf_s=1.5, nnz_min=3,
                          nnz_max=400, nnz_mean=12.0, n_star=60, lambda_frac=0.1, seed=83)
    x_o, ev_o = oracle_optimum(inst, target=1e-10)
    kw = dict(tau=256, warps_per_block=8, gap_target=1e-7, refresh_every=2, max_epochs=5000,
              use_shrinking=1, shrinking_probability=0.9, shrinking_starting_iter=2, seed=5,
              tau_active=64, active_passes=10, precision=acdc.PREC_FP32, polish_rel_gap=1e-5)
    p = acdc.Problem(ctx, inst, hot_polish_sweeps=16, **kw)
    r, rows = p.solve_traced()
    assert r.converged, (r.eval.rel_gap, r.epochs)
    assert r.stats.updates == rows[-1]["updates"]
    full = p.evaluate()
    assert full["primal"] == pytest.approx(r.eval.primal, rel=1e-12)
    assert full["rel_gap"] <= r.eval.rel_gap * (1 + 1e-9) + 1e-15
    assert abs(r.eval.primal - ev_o["primal"]) <= 1e-6 * abs(ev_o["primal"])
    x = p.get_x()
    assert set(np.nonzero(x)[0]) == set(np.nonzero(x_o)[0])
    assert not np.array_equal(x, x.astype(np.float32).astype(np.float64))  # the FP64 iterate
    p.close()
    # the same FP32 bulks without the polish, for as many epochs: no certificate
    q = acdc.Problem(ctx, inst, hot_polish_sweeps=0, **dict(kw, max_epochs=r.epochs))
    rq = q.solve()
    assert not rq.converged and rq.eval.rel_gap > 1e-7
    x = q.get_x()
    assert np.array_equal(x, x.astype(np.float32).astype(np.float64))  # FP32 throughout
    q.close()


def test_solve_trace_records_every_evaluation(ctx):
    """acdc_solve_traced: one row per evaluation (row 0 before any update), the
    last row the solve's final certificate, work counters increasing; the same
    solve without a trace ends at the same state (the trace only reads)."""
    inst = acdc.gen_lasso(4000, 40000, nnz_mode=acdc.NNZ_ZIPF, zipf_s=1.5, nnz_min=3,
                          nnz_max=400, nnz_mean=12.0, n_star=60, lambda_frac=0.1, seed=83)
    kw = dict(tau=256, warps_per_block=8, gap_target=1e-7, refresh_every=2, max_epochs=5000,
              use_shrinking=1, shrinking_probability=0.9, shrinking_starting_iter=2, seed=5,
              tau_active=64, active_passes=10, precision=acdc.PREC_FP64)
    p = acdc.Problem(ctx, inst, **kw)
    r, rows = p.solve_traced()
    assert r.converged and len(rows) >= 3
    assert rows[0]["updates"] == 0 and rows[0]["update_ms"] == 0
    assert all(b["updates"] > a["updates"] for a, b in zip(rows, rows[1:]))
    assert rows[-1]["rel_gap"] == r.eval.rel_gap and rows[-1]["primal"] == r.eval.primal
    assert rows[-1]["updates"] == r.stats.updates
    assert any(t["shrink"] for t in rows) and any(t["screened"] for t in rows)
    assert any(t["hot"] > 0 and t["omega_hot"] >= 1 for t in rows)
    assert sum(t["update_ms"] for t in rows) > 0
    _, few = p.solve_traced(cap=1)  # converged already: one evaluation, no bulk
    assert len(few) == 1 and few[0]["updates"] == 0
    p.close()


def test_checkpoint_resumes_the_same_draws(ctx):
    """acdc_checkpoint_save / _load: a problem restored from a checkpoint into a
    fresh one continues with the same sampler counter, so one warp reproduces the
    original continuation (to FP32 rounding of the recomputed residual); a
    checkpoint of another shape or size is refused."""
    inst = acdc.gen_lasso(600, 2500, nnz_per_col=8, n_star=30, lambda_frac=0.1, seed=21)
    kw = dict(tau=1, warps_per_block=1, seed=9)
    p = acdc.Problem(ctx, inst, **kw)
    p.run_updates(3 * inst.n)
    ck = p.checkpoint()
    p.run_updates(2 * inst.n)
    x1 = p.get_x()
    q = acdc.Problem(ctx, inst, **kw)
    q.restore(ck)
    q.run_updates(2 * inst.n)
    np.testing.assert_allclose(q.get_x(), x1, rtol=1e-5, atol=1e-7)
    q.reset()
    q.run_updates(2 * inst.n)
    assert not np.allclose(q.get_x(), x1, atol=1e-7)
    other = acdc.Problem(ctx, acdc.gen_lasso(600, 2400, nnz_per_col=8, n_star=30, seed=22))
    for bad, target in ((ck, other), (ck[:-8], q), (b"X" + ck[1:], q)):
        with pytest.raises(acdc.AcdcError) as e:
            target.restore(bad)
        assert e.value.code == acdc.EINVAL
    for x in (p, q, other):
        x.close()


def test_invalid_inputs_are_rejected(ctx):
    inst = acdc.gen_lasso(50, 80, nnz_per_col=3, n_star=5, seed=1)
    bad = acdc.Instance(inst.loss, inst.m, inst.n, inst.col_ptr, inst.row_idx.copy(), inst.vals,
                        inst.rhs, inst.lam)
    bad.row_idx[7] = 50  # out of range: the layout kernel flags it, nothing is read out of bounds
    with pytest.raises(acdc.AcdcError) as e:
        acdc.Problem(ctx, bad)
    assert e.value.code == acdc.EDEVICE
    # losses 1 and 3 solve one problem at a time; the batched paths take 0 and 2
    ridge = acdc.Problem(ctx, acdc.Instance(acdc.LOSS_L2_SQUARE, inst.m, inst.n, inst.col_ptr,
                                            inst.row_idx, inst.vals, inst.rhs, inst.lam))
    with pytest.raises(acdc.AcdcError) as e:
        acdc.batch_solve_path(ctx, [ridge], np.array([[inst.lam]]))
    assert e.value.code == acdc.EUNSUPPORTED
    ridge.close()
    with pytest.raises(acdc.AcdcError) as e:
        acdc.Problem(ctx, acdc.Instance(4, inst.m, inst.n, inst.col_ptr, inst.row_idx, inst.vals,
                                        inst.rhs, inst.lam))
    assert e.value.code == acdc.EINVAL
    cp = inst.col_ptr.copy()
    cp[0] = 1
    with pytest.raises(acdc.AcdcError) as e:
        acdc.Problem(ctx, acdc.Instance(inst.loss, inst.m, inst.n, cp, inst.row_idx, inst.vals,
                                        inst.rhs, inst.lam))
    assert e.value.code == acdc.EINVAL
    p = acdc.Problem(ctx, inst)
    with pytest.raises(acdc.AcdcError):
        p.set_settings(acdc.default_settings(inst.loss), tau=0)
    with pytest.raises(acdc.AcdcError):
        p.set_lambda(-1.0)
    # the context is still usable after the errors
    p.set_settings(acdc.default_settings(inst.loss), tau=8, warps_per_block=8, max_epochs=400,
                   gap_target=1e-6)
    assert p.solve().converged
