"""The C++ boundary: CudaEngineExecutor plugs into the reference's engine
interface.  CPU: the header compiles against the reference's own headers (when
the reference sources are present) and against the mirrors shipped here.  GPU:
the drop-in console solver reads the reference's text CSC format and reaches the
oracle's optimum; its bulk mode prints the reference's log rows."""
import os
import subprocess

import numpy as np
import pytest

import acdc
import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# the reference checkout's sources (ACDC_REFERENCE_ROOT); the check is skipped without it
REF = os.path.join(os.environ.get("ACDC_REFERENCE_ROOT", ""), "cpp", "src")
CPP = os.path.join(ROOT, "ac-dc_gb300", "cpp")
SOLVER = os.path.join(ROOT, "ac-dc_gb300", "lib", "acdc_solver")

PROBE = r"""
#include "helpers/utils.h"
#include "solver/structures.h"
#include "solver/settingsAndStatistics.h"
#include "solver/AbstractEngineExecutor.h"
#include "solver/Solver.h"
#include "CudaEngineExecutor.h"
int probe(ProblemData<int, double>& inst, OptimizationSettings* s) {
  CudaEngineExecutor<int, double> engine(inst, s);
  Solver<int, double> solver(engine);
  solver.runSolver();
  return (int)engine.getObjectiveValue();
}
"""


@pytest.mark.skipif(not os.environ.get("ACDC_REFERENCE_ROOT") or not os.path.isdir(REF),
                    reason="reference sources not present (set ACDC_REFERENCE_ROOT)")
def test_engine_header_compiles_against_reference_headers(tmp_path):
    src = tmp_path / "probe.cpp"
    src.write_text(PROBE)
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-w", "-fopenmp",
           "-include", os.path.join(ROOT, "oracle", "ref_pre.h"),
           "-I" + REF, "-I" + os.path.join(ROOT, "oracle", "gsl_shim"),
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(CPP, "solver"), str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_console_solver_built_against_mirror_headers():
    assert os.access(SOLVER, os.X_OK)
    r = subprocess.run([SOLVER, "-h"], capture_output=True, text=True)
    assert r.returncode == 0 and "usage" in r.stdout


def write_csc(tmp_path, inst):
    pre = str(tmp_path / "A")
    np.savetxt(pre + "_values.txt", inst.vals, fmt="%.17g")
    np.savetxt(pre + "_colPtr.txt", inst.col_ptr, fmt="%d")
    np.savetxt(pre + "_rowIdx.txt", inst.row_idx, fmt="%d")
    np.savetxt(str(tmp_path / "b.txt"), inst.rhs, fmt="%.17g")
    return pre, str(tmp_path / "b.txt")


def test_console_solver_refuses_bad_settings_before_device_work(tmp_path):
    """A shrinking probability above 1 is refused by the engine's settings check,
    which runs before a context is made (so this needs no GPU)."""
    inst = acdc.gen_lasso(60, 90, nnz_per_col=4, n_star=5, seed=3)
    pre, bfile = write_csc(tmp_path, inst)
    out = subprocess.run([SOLVER, "-A", pre, "-b", bfile, "-l", "0.1", "-f", "0", "-S", "1.5"],
                         capture_output=True, text=True, timeout=60)
    assert out.returncode == 1 and "out of range" in out.stderr, out.stderr


@pytest.mark.gpu
def test_console_solver_reaches_the_oracle_optimum(tmp_path):
    inst = acdc.gen_lasso(800, 3000, nnz_per_col=10, n_star=40, lambda_frac=0.1, seed=91)
    pre, bfile = write_csc(tmp_path, inst)
    x, r, ev, ep = oracle.lasso_solve(inst.m, inst.n, inst.col_ptr, inst.row_idx, inst.vals,
                                      inst.rhs, inst.lam, seed=1, target=1e-10)
    out = subprocess.run([SOLVER, "-A", pre, "-b", bfile, "-l", repr(inst.lam), "-t", "32",
                          "-f", "0", "-G", "1e-7"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    line = [l for l in out.stdout.splitlines() if l.startswith("converged,")][-1].split(",")
    fields = dict(zip(line[0::2], line[1::2]))
    assert fields["converged"] == "1"
    assert abs(float(fields["primal"]) - ev["primal"]) <= 1e-6 * ev["primal"]


@pytest.mark.gpu
def test_console_solver_bulk_mode_prints_reference_rows(tmp_path):
    inst = acdc.gen_lasso(500, 2000, nnz_per_col=8, n_star=20, lambda_frac=0.1, seed=92)
    pre, bfile = write_csc(tmp_path, inst)
    out = subprocess.run([SOLVER, "-A", pre, "-b", bfile, "-l", repr(inst.lam), "-t", "16",
                          "-f", "0", "-I", "20000", "-B", "6", "-i", "1"],
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    rows = [l.split(",") for l in out.stdout.splitlines()
            if l.count(",") == 3 and l.split(",")[0].isdigit()]
    assert [int(r[0]) for r in rows] == [0, 1, 2, 3, 4, 5, 6]
    objs = [float(r[1]) for r in rows]
    assert objs[-1] < objs[0] and all(b <= a * (1 + 1e-6) for a, b in zip(objs, objs[1:]))
    assert "Last objective value" in out.stdout


def write_libsvm(path, sv):
    """LIBSVM text of an SVM-generator instance (samples as lines, 1-based features)."""
    with open(path, "w") as f:
        for i in range(sv.n):
            s, e = sv.col_ptr[i], sv.col_ptr[i + 1]
            feats = " ".join("%d:%.17g" % (int(c) + 1, v)
                             for c, v in zip(sv.row_idx[s:e], sv.vals[s:e]))
            f.write("%d %s\n" % (int(sv.rhs[i]), feats))


@pytest.mark.gpu
def test_console_solver_ridge_and_logistic(tmp_path):
    """-f 1 reads the CSC text format like -f 0; -f 3 reads LIBSVM samples and
    turns them into rows over feature columns (MultiCoreSolver.cpp:80-105).
    Both solve to the oracle's optimum."""
    rd = acdc.gen_lasso(500, 1500, nnz_per_col=6, n_star=20, lambda_frac=0.1, seed=93)
    pre, bfile = write_csc(tmp_path, rd)
    lam = 0.2
    x, r, ev, ep = oracle.smooth_solve(oracle.RIDGE, rd.m, rd.n, rd.col_ptr, rd.row_idx, rd.vals,
                                       rd.rhs, lam, target=1e-11)
    out = subprocess.run([SOLVER, "-A", pre, "-b", bfile, "-l", repr(lam), "-t", "32", "-f", "1",
                          "-G", "1e-9"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    line = [l for l in out.stdout.splitlines() if l.startswith("converged,")][-1].split(",")
    fields = dict(zip(line[0::2], line[1::2]))
    assert fields["converged"] == "1"
    assert abs(float(fields["primal"]) - ev["primal"]) <= 1e-6 * ev["primal"]

    sv = acdc.gen_svm(600, 1200, nnz_median=15, nnz_sigma=0.5, w_star_nnz=60, lam=1e-3, seed=94)
    path = str(tmp_path / "train.libsvm")
    write_libsvm(path, sv)
    lg = acdc.logistic_from_svm(sv, 0.02)
    x, r, ev, ep = oracle.smooth_solve(oracle.LOGISTIC, lg.m, lg.n, lg.col_ptr, lg.row_idx,
                                       lg.vals, lg.rhs, 0.02, target=1e-11, max_epochs=50000)
    out = subprocess.run([SOLVER, "-A", path, "-l", "0.02", "-t", "16", "-f", "3", "-G", "1e-9"],
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    line = [l for l in out.stdout.splitlines() if l.startswith("converged,")][-1].split(",")
    fields = dict(zip(line[0::2], line[1::2]))
    assert fields["converged"] == "1"
    assert abs(float(fields["primal"]) - ev["primal"]) <= 1e-6 * ev["primal"]
