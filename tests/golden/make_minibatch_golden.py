"""Writes svm_minibatch_traj.npz: a small hinge-loss SVM dual (inputs stored)
and the oracle's synchronous mini-batch SDCA trajectory on it (alpha and w
after each of 4 epochs of tau-nice steps), the fixture that pins the oracle's
restatement of the reference's mini-batch loop (cpp/src/experiments/
mSDCA.cpp:60-105) against later changes.  TEST INFRASTRUCTURE: runs the
oracle on the CPU.

    python tests/golden/make_minibatch_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "ac-dc_gb300"))

import acdc  # noqa: E402
import oracle  # noqa: E402


def main():
    oracle.build()
    sv = acdc.gen_svm(300, 2000, nnz_median=25, nnz_sigma=0.6, w_star_nnz=100, lam=2e-3,
                      seed=0xACDC0005)
    tau, seed, epochs = 48, 17, 4
    omega = oracle.omega(sv.m, sv.n, sv.col_ptr, sv.row_idx)
    beta = oracle.eso_beta(omega, tau, sv.n)
    S = oracle.SVM(sv.m, sv.n, sv.col_ptr, sv.row_idx, sv.vals, sv.rhs, sv.lam, sigma=beta)
    steps = (sv.n + tau - 1) // tau
    alphas, ws, ks = [], [], []
    for _ in range(epochs):
        S.minibatch(steps, seed, tau)
        alphas.append(S.x.copy())
        ws.append(S.r.copy())
        ks.append(S.k)
    np.savez_compressed(os.path.join(HERE, "svm_minibatch_traj.npz"), m=sv.m, n=sv.n,
                        row_ptr=sv.col_ptr, col_idx=sv.row_idx, vals=sv.vals, y=sv.rhs,
                        lam=sv.lam, tau=tau, seed=seed, beta=beta, steps_per_epoch=steps,
                        alpha=np.array(alphas), w=np.array(ws), counter=np.array(ks))


if __name__ == "__main__":
    main()
