"""Writes the golden fixtures of tests/golden from the reference's own engine.

Run where the reference sources are available (they are compiled into
oracle/_ref by `make -C oracle ref`):

    python tests/golden/make_golden.py [reference_root]

Fixtures (all inputs are stored, so no generator has to reproduce them):
  lasso_traj.npz   small Lasso: inputs + the reference engine's x, residuals and
                   objective after each of 6 bulks (one thread, seeded sampler)
  svm_traj.npz     small SVM dual: inputs + alpha, w and (gap, P, D, 0-1) per bulk
  ridge_traj.npz   small L2-regularised square loss (lossFunction 1): inputs + x,
                   residuals and objective per bulk
  logistic_traj.npz
                   small L2-regularised logistic loss (lossFunction 3), samples as
                   rows and features as coordinates: inputs + x, residuals and
                   objective per bulk
  lasso_config0.json
                   the 2,000 x 10,000 config-0 instance, identified by the SHA-256
                   of its generated arrays, with the reference engine's solution
                   after enough epochs for an FP64 duality gap <= 1e-9: objective,
                   support and the values on the support
  philox_kat.json  published Philox4x32-10 known-answer vectors (Random123)
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "ac-dc_gb300"))

import acdc  # noqa: E402
import oracle  # noqa: E402

CONFIG0 = dict(m=2000, n=10000, nnz_per_col=20, n_star=100, noise_sigma=0.01, lambda_frac=0.1,
               seed=0xACDC0000)


def instance_hash(inst):
    h = hashlib.sha256()
    for a in (inst.col_ptr, inst.row_idx, inst.vals, inst.rhs):
        h.update(np.ascontiguousarray(a).tobytes())
    h.update(np.float64(inst.lam).tobytes())
    return h.hexdigest()


def main(ref_root=None):
    oracle.build(ref_root)
    if oracle.ref_lib() is None:
        raise SystemExit("reference engine not built (reference sources missing)")

    # small Lasso trajectory
    inst = acdc.gen_lasso(300, 1200, nnz_per_col=6, n_star=20, noise_sigma=0.01, lambda_frac=0.1,
                          seed=11)
    seed, bulks, inner = 12345, 6, 700
    x, r, obj = oracle.ref_lasso(inst.m, inst.n, inst.col_ptr.astype(np.int32), inst.row_idx,
                                 inst.vals, inst.rhs, inst.lam, seed, bulks, inner)
    np.savez_compressed(os.path.join(HERE, "lasso_traj.npz"), m=inst.m, n=inst.n,
                        col_ptr=inst.col_ptr, row_idx=inst.row_idx, vals=inst.vals, b=inst.rhs,
                        lam=inst.lam, seed=seed, bulks=bulks, inner=inner, x=x, r=r, obj=obj)

    # small SVM trajectory
    sv = acdc.gen_svm(150, 900, nnz_median=30, nnz_sigma=0.7, w_star_nnz=100, lam=1e-3, seed=13)
    seed, bulks, inner, sigma = 777, 5, 300, 1.0
    a, w, ev = oracle.ref_svm(sv.m, sv.n, sv.col_ptr.astype(np.int32), sv.row_idx, sv.vals, sv.rhs,
                              sv.lam, sigma, seed, bulks, inner)
    np.savez_compressed(os.path.join(HERE, "svm_traj.npz"), d=sv.m, n=sv.n, row_ptr=sv.col_ptr,
                        col_idx=sv.row_idx, vals=sv.vals, y=sv.rhs, lam=sv.lam, sigma=sigma,
                        seed=seed, bulks=bulks, inner=inner, alpha=a, w=w, evals=ev)

    # small L2-regularised square loss (lossFunction 1) trajectory
    rd = acdc.gen_lasso(250, 900, nnz_per_col=7, n_star=25, noise_sigma=0.01, lambda_frac=0.1,
                        seed=15)
    seed, bulks, inner, lam = 4242, 5, 600, 0.3
    x, r, obj = oracle.ref_smooth(1, rd.m, rd.n, rd.col_ptr.astype(np.int32), rd.row_idx, rd.vals,
                                  rd.rhs, lam, 1.0, seed, bulks, inner)
    np.savez_compressed(os.path.join(HERE, "ridge_traj.npz"), m=rd.m, n=rd.n, col_ptr=rd.col_ptr,
                        row_idx=rd.row_idx, vals=rd.vals, b=rd.rhs, lam=lam, seed=seed,
                        bulks=bulks, inner=inner, x=x, r=r, obj=obj)

    # small L2-regularised logistic loss (lossFunction 3) trajectory: samples of the
    # SVM generator as rows, features as coordinates (CSC over features), the
    # engine's sigma taken above 1
    lg = acdc.gen_svm(350, 800, nnz_median=18, nnz_sigma=0.6, w_star_nnz=60, lam=1e-3, seed=17)
    import scipy.sparse as sp
    X = sp.csr_matrix((lg.vals, lg.row_idx, lg.col_ptr), shape=(lg.n, lg.m)).tocsc()
    X.sort_indices()
    cp = X.indptr.astype(np.int64)
    ri = X.indices.astype(np.int32)
    va = X.data.astype(np.float64)
    seed, bulks, inner, lam, sigma = 9191, 5, 800, 1e-2, 1.5
    x, r, obj = oracle.ref_smooth(3, X.shape[0], X.shape[1], cp.astype(np.int32), ri, va, lg.rhs,
                                  lam, sigma, seed, bulks, inner)
    np.savez_compressed(os.path.join(HERE, "logistic_traj.npz"), m=X.shape[0], n=X.shape[1],
                        col_ptr=cp, row_idx=ri, vals=va, b=lg.rhs, lam=lam, sigma=sigma, seed=seed,
                        bulks=bulks, inner=inner, x=x, r=r, obj=obj)

    # config 0: the reference engine run epoch by epoch until the FP64 gap <= 1e-9
    c0 = acdc.gen_lasso(CONFIG0["m"], CONFIG0["n"], nnz_per_col=CONFIG0["nnz_per_col"],
                        n_star=CONFIG0["n_star"], noise_sigma=CONFIG0["noise_sigma"],
                        lambda_frac=CONFIG0["lambda_frac"], seed=CONFIG0["seed"])
    seed = 1
    epochs = 0
    ev = None
    cp32 = c0.col_ptr.astype(np.int32)
    L = oracle.Lasso(c0.m, c0.n, c0.col_ptr, c0.row_idx, c0.vals, c0.rhs, c0.lam)
    for epochs in range(10, 400, 10):
        x, r, obj = oracle.ref_lasso(c0.m, c0.n, cp32, c0.row_idx, c0.vals, c0.rhs, c0.lam, seed,
                                     epochs, c0.n)
        L.x[:] = x
        L.refresh()
        ev = L.evaluate()
        if ev["gap"] <= 1e-9:
            break
    support = np.nonzero(x)[0]
    rec = dict(generator=CONFIG0, input_sha256=instance_hash(c0), lam=c0.lam, sampler_seed=seed,
               epochs=epochs, objective=ev["primal"], dual=ev["dual"], gap=ev["gap"],
               support=support.tolist(), x_support=x[support].tolist(),
               reference_last_objective=float(obj[-1]))
    with open(os.path.join(HERE, "lasso_config0.json"), "w") as f:
        json.dump(rec, f, indent=1)

    kat = {"source": "Random123 kat_vectors, philox4x32_10",
           "cases": [
               {"ctr": [0, 0, 0, 0], "key": [0, 0],
                "out": [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]},
               {"ctr": [0xffffffff] * 4, "key": [0xffffffff] * 2,
                "out": [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]},
               {"ctr": [0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                "key": [0xa4093822, 0x299f31d0],
                "out": [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]}]}
    with open(os.path.join(HERE, "philox_kat.json"), "w") as f:
        json.dump(kat, f, indent=1)
    print("wrote fixtures; config0 epochs", epochs, "gap", ev["gap"], "support", len(support))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
