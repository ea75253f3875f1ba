"""The two benchmark workloads at full size against their committed FP64
optima (tests/golden/make_config_optima.py: the oracle run to a relative gap of
1.65e-10 for the Lasso and an absolute gap of 9e-11 for the SVM dual).

Bars:
  * the generated data equal the data the optima were computed on (SHA-256);
  * SVM dual, 20,000 x 1,355,191, synchronous mini-batch of 1024: solved to the
    absolute gap that bounds the objective error by 1e-6 relative, the FP64
    objective of alpha on the host within 1e-6 relative of the optimum and the
    same support (every alpha_i nonzero in both);
  * Lasso, 1e6 x 1e7 (2e8 nonzeros), the benchmark's settings: relative gap
    1e-6, the FP64 objective of x on the host within 1e-6 relative of the
    optimum, and the support equal to the optimum's up to exact-duplicate
    columns except for at most 0.1% of the classes (near-duplicate pairs whose
    split a gap of 1e-6 does not settle).
"""
import os
import sys

import pytest

import acdc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
import bench  # noqa: E402  (workload table, generator calls, oracle comparison)

pytestmark = pytest.mark.gpu


def test_svm_workload_reaches_the_fp64_optimum(ctx):
    name = "svm_n2e4_d1355191"
    w = dict(bench.WORKLOADS[name], name=name)
    inst = bench.generate(w, pinned=False)
    import numpy as np
    f = np.load(bench.OPTIMA[name])
    assert bench.instance_digest(inst) == str(f["sha256"])
    w["gap"] = 1e-6 * abs(float(f["primal"]))
    p = acdc.Problem(ctx, inst, bench.settings_for(w))
    r = p.solve()
    assert r.converged
    o = bench.oracle_error(name, inst, p.get_x(), r.eval.primal)
    assert o["oracle_rel_err"] <= 1e-6, o
    assert o["support_match"], o
    p.close()


def test_lasso_workload_reaches_the_fp64_optimum(ctx):
    name = "lasso_m1e6_n1e7_zipf"
    w = dict(bench.WORKLOADS[name], name=name)
    inst = bench.generate(w, pinned=False)
    import numpy as np
    f = np.load(bench.OPTIMA[name])
    assert bench.instance_digest(inst) == str(f["sha256"])
    p = acdc.Problem(ctx, inst, bench.settings_for(w))
    r = p.solve()
    assert r.converged and r.eval.rel_gap <= 1e-6
    o = bench.oracle_error(name, inst, p.get_x(), r.eval.primal)
    assert o["oracle_rel_err"] <= 1e-6, o
    assert o["class_symmetric_difference"] <= 1e-3 * o["oracle_class_support"], o
    p.close()
