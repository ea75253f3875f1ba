"""Writes the FP64 optima of the two large benchmark workloads (TEST
INFRASTRUCTURE: the oracle, run on the CPU; nothing here runs on a GPU).

    python tests/golden/make_config_optima.py [lasso] [svm] [--resume x.npy]

lasso_m1e6_n1e7_optimum.npz
    The 1,000,000 x 10,000,000 Zipf Lasso (about 2.0e8 nonzeros), generated by
    the library's seeded generator exactly as bench.py generates it, solved by
    the oracle's working-set FP64 solver (oracle.lasso_solve_ws: cyclic sweeps
    of the reference's exact-step update, MulticoreL1RegSquareLoss.h:41-63, over
    the working set, with an exact residual refresh and a full duality-gap
    evaluation at every check) to a relative duality gap <= 1e-9.
svm_n2e4_d1355191_optimum.npz
    The 20,000-sample hinge-loss SVM dual (1,355,191 features), solved by the
    oracle's serial SDCA (the reference's update, MulticoreSVMDualLoss.h:119-141,
    with the counter-based sampler) to an absolute duality gap <= 1e-9.

Each file holds the SHA-256 of the generated arrays and lambda (so a run that
generated different data can tell), the objective, dual, gap, the support (the
indices of the nonzero coordinates) and the coordinates' values there, and for
the SVM the full alpha.  bench.py compares its last timed solve with them.
"""
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "ac-dc_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

import bench  # noqa: E402  (the workload table and generator calls)
import oracle  # noqa: E402

LASSO_WORKLOAD = "lasso_m1e6_n1e7_zipf"
SVM_WORKLOAD = "svm_n2e4_d1355191"
LASSO_FILE = os.path.join(HERE, "lasso_m1e6_n1e7_optimum.npz")
SVM_FILE = os.path.join(HERE, "svm_n2e4_d1355191_optimum.npz")


def instance_hash(inst):
    h = hashlib.sha256()
    for a in (inst.col_ptr, inst.row_idx, inst.vals, inst.rhs):
        h.update(np.ascontiguousarray(a).tobytes())
    h.update(np.float64(inst.lam).tobytes())
    return h.hexdigest()


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def lasso(target=1e-9, sweeps=500, eps=0.05, anderson=5, resume=None):
    """resume: a .npy file where x is saved after every block of checks; an
    existing one (for the same input) is the start point, so an interrupted
    run continues instead of starting over."""
    w = dict(bench.WORKLOADS[LASSO_WORKLOAD])
    t0 = time.time()
    inst = bench.generate(w, pinned=False)
    digest = instance_hash(inst)
    log("generated", inst.m, inst.n, inst.nnz, "lambda", inst.lam, digest, "%.1fs" % (time.time() - t0))
    x = None
    if resume and os.path.exists(resume):
        x = np.load(resume)
        log("resuming from", resume)
    total_sweeps = checks = 0
    t1 = time.time()
    while True:
        x, r, ev, sw, ch = oracle.lasso_solve_ws(inst.m, inst.n, inst.col_ptr, inst.row_idx,
                                                 inst.vals, inst.rhs, inst.lam, target=target,
                                                 rel=True, max_checks=10, sweeps=sweeps, eps=eps,
                                                 anderson=anderson, x0=x)
        total_sweeps += sw
        checks += ch
        log("sweeps %d checks %d rel_gap %.3e support %d  %.0fs" %
            (total_sweeps, checks, ev["rel_gap"], ev["support"], time.time() - t1))
        if resume:
            np.save(resume + ".tmp.npy", x)
            os.replace(resume + ".tmp.npy", resume)
        if ev["rel_gap"] <= target:
            break
    sup = np.nonzero(x)[0].astype(np.int64)
    np.savez_compressed(LASSO_FILE, workload=LASSO_WORKLOAD, sha256=digest, m=inst.m, n=inst.n,
                        nnz=inst.nnz, lam=inst.lam, primal=ev["primal"], dual=ev["dual"],
                        gap=ev["gap"], rel_gap=ev["rel_gap"], support=sup, x_support=x[sup],
                        sweeps=total_sweeps, checks=checks, seconds=time.time() - t1)
    log("wrote", LASSO_FILE)


def svm(target=1e-9):
    w = dict(bench.WORKLOADS[SVM_WORKLOAD])
    t0 = time.time()
    inst = bench.generate(w, pinned=False)
    digest = instance_hash(inst)
    log("generated", inst.m, inst.n, inst.nnz, "lambda", inst.lam, digest, "%.1fs" % (time.time() - t0))
    t1 = time.time()
    a, wv, ev, ep = oracle.svm_solve(inst.m, inst.n, inst.col_ptr, inst.row_idx, inst.vals,
                                     inst.rhs, inst.lam, seed=1, target=target, max_epochs=1000000,
                                     check_every=5)
    log("epochs %d gap %.3e support %d %.0fs" % (ep, ev["gap"], ev["support"], time.time() - t1))
    sup = np.nonzero(a)[0].astype(np.int64)
    np.savez_compressed(SVM_FILE, workload=SVM_WORKLOAD, sha256=digest, m=inst.m, n=inst.n,
                        nnz=inst.nnz, lam=inst.lam, primal=ev["primal"], dual=ev["dual"],
                        gap=ev["gap"], rel_gap=ev["rel_gap"], support=sup, alpha=a, epochs=ep,
                        seconds=time.time() - t1)
    log("wrote", SVM_FILE)


def main(argv):
    resume = None
    if "--resume" in argv:
        i = argv.index("--resume")
        resume = argv[i + 1]
        argv = argv[:i] + argv[i + 2:]
    which = argv or ["lasso", "svm"]
    oracle.build()
    if "svm" in which:
        svm()
    if "lasso" in which:
        lasso(resume=resume)


if __name__ == "__main__":
    main(sys.argv[1:])
