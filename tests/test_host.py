"""Host-side logic without a GPU: generators, loaders, the C-ABI export list
and argument checking that happens before any device work."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import acdc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(acdc_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.mark.parametrize("header,lib", [("acdc_gpu.h", acdc.GPU_LIB), ("acdc_host.h", acdc.HOST_LIB)])
def test_library_exports_every_declared_symbol(header, lib):
    names = declared_functions(header)
    assert len(names) > 5
    L = C.CDLL(lib)
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


STRUCTS = [("acdc_settings", "Settings"), ("acdc_eval", "Eval"), ("acdc_stats", "Stats"),
           ("acdc_solve_result", "SolveResult"), ("acdc_trace_row", "TraceRow"),
           ("acdc_problem_info", "ProblemInfo"), ("acdc_batch_options", "BatchOptions"),
           ("acdc_batch_result", "BatchResult"), ("acdc_server_options", "ServerOptions"),
           ("acdc_server_stats", "ServerStats"), ("acdc_request", "Request"),
           ("acdc_request_result", "RequestResult"), ("acdc_lasso_gen", "LassoGen"),
           ("acdc_svm_gen", "SvmGen")]


def test_ctypes_structs_match_the_c_headers(tmp_path):
    """Every struct of the C-ABI has the same size and field offsets in the
    ctypes binding as the C compiler gives it from include/*.h."""
    import subprocess
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "acdc_gpu.h"',
             '#include "acdc_host.h"', 'int main(void) {']
    for c_name, py_name in STRUCTS:
        lines.append('  printf("%s size %%zu\\n", sizeof(%s));' % (c_name, c_name))
        for field, _ in getattr(acdc, py_name)._fields_:
            c_field = {"lambda_": "lambda"}.get(field, field)
            lines.append('  printf("%s.%s %%zu\\n", offsetof(%s, %s));'
                         % (c_name, field, c_name, c_field))
    lines += ['  return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = dict(line.rsplit(" ", 1) for line in out if line)
    for c_name, py_name in STRUCTS:
        cls = getattr(acdc, py_name)
        assert int(got["%s size" % c_name]) == C.sizeof(cls), c_name
        for field, _ in cls._fields_:
            assert int(got["%s.%s" % (c_name, field)]) == getattr(cls, field).offset, (c_name, field)


def test_gpu_library_loads_and_reports_no_device_cleanly():
    L = acdc.gpu_lib()
    s = acdc.default_settings()
    assert s.tau == 4096 and s.refresh_every == 5 and s.gap_relative == 1
    assert L.acdc_status_string(acdc.EUNSUPPORTED) == b"unsupported loss"
    assert L.acdc_status_string(acdc.ECANCELED) == b"request cancelled"
    assert L.acdc_checkpoint_size(None) == 0
    h = acdc.VP()
    rc = L.acdc_ctx_create(0, C.byref(h))
    import torch
    if not torch.cuda.is_available():
        assert rc == acdc.ENODEV


def test_settings_check_refuses_every_out_of_range_field():
    """acdc_settings_check (the check acdc_problem_set_settings makes) needs no
    device: defaults of every loss pass, and each field outside its range,
    NaN and infinities included, is refused on its own (an infinite gap target
    would end a solve at its first evaluation)."""
    nan, inf = float("nan"), float("inf")
    for loss in range(4):
        assert acdc.settings_ok(acdc.default_settings(loss))
    assert acdc.gpu_lib().acdc_settings_check(None) == acdc.EINVAL
    good = [("sigma", -1.0), ("sigma", 0.0), ("sigma", 1.7), ("shrinking_probability", 0.0),
            ("shrinking_probability", 1.0), ("shrink_eps", 0.0), ("gap_target", 0.0),
            ("gap_target", 1e300), ("tau_active", 0), ("max_epochs", 0), ("warps_per_block", 8),
            ("precision", acdc.PREC_FP64), ("hot_threshold", 0.0), ("polish_stall_epochs", 0),
            ("hot_polish_sweeps", 0), ("polish_active_passes", 0), ("active_passes", -3),
            ("shrinking_starting_iter", -1), ("lanes_per_update", -1), ("lanes_per_update", 1),
            ("lanes_per_update", 8), ("lanes_per_update", 16), ("lanes_per_update", 32)]
    bad = [("lanes_per_update", 2), ("lanes_per_update", 4), ("lanes_per_update", 64),
           ("lanes_per_update", -2), ("loss", -1), ("loss", 4), ("tau", 0), ("tau_active", -1), ("warps_per_block", 0),
           ("warps_per_block", 9), ("refresh_every", 0), ("max_epochs", -1), ("sigma", nan),
           ("sigma", inf), ("sigma", -inf), ("gap_target", -1e-9), ("gap_target", nan),
           ("shrinking_probability", -0.1), ("shrinking_probability", 1.01),
           ("shrinking_probability", nan), ("shrink_eps", -0.1), ("shrink_eps", 1.0),
           ("shrink_eps", nan), ("precision", -1), ("precision", 3), ("polish_rel_gap", -1.0),
           ("polish_rel_gap", nan), ("hot_threshold", -0.5), ("hot_threshold", nan),
           ("gap_target", inf), ("polish_rel_gap", inf), ("hot_threshold", inf),
           ("polish_stall_epochs", -1), ("hot_polish_sweeps", -1), ("polish_active_passes", -1)]
    for field, value in good:
        assert acdc.settings_ok(acdc.default_settings(**{field: value})), (field, value)
    for field, value in bad:
        assert not acdc.settings_ok(acdc.default_settings(**{field: value})), (field, value)


def test_minibatch_is_for_the_svm_dual_only():
    assert not acdc.settings_ok(acdc.default_settings(acdc.LOSS_L1_SQUARE, minibatch=1))
    assert not acdc.settings_ok(acdc.default_settings(acdc.LOSS_SVM_DUAL, minibatch=2))
    assert acdc.settings_ok(acdc.default_settings(acdc.LOSS_SVM_DUAL, minibatch=1))


def test_generator_is_deterministic_and_thread_independent():
    a = acdc.gen_lasso(500, 2000, nnz_per_col=7, n_star=30, seed=42, threads=1)
    b = acdc.gen_lasso(500, 2000, nnz_per_col=7, n_star=30, seed=42, threads=4)
    for f in ("col_ptr", "row_idx", "vals", "rhs"):
        assert np.array_equal(getattr(a, f), getattr(b, f))
    assert a.lam == b.lam
    c = acdc.gen_lasso(500, 2000, nnz_per_col=7, n_star=30, seed=43)
    assert not np.array_equal(a.vals, c.vals)


def test_lasso_generator_properties():
    m, n = 1000, 3000
    inst = acdc.gen_lasso(m, n, nnz_per_col=20, n_star=100, noise_sigma=0.01, lambda_frac=0.1, seed=7)
    cp, ri, va = inst.col_ptr, inst.row_idx, inst.vals
    assert cp[0] == 0 and cp[-1] == 20 * n
    for j in range(0, n, 97):
        rows = ri[cp[j]:cp[j + 1]]
        assert np.all(np.diff(rows) > 0) and rows.min() >= 0 and rows.max() < m
        assert abs(np.linalg.norm(va[cp[j]:cp[j + 1]]) - 1) < 1e-12
    assert np.count_nonzero(inst.x_star) == 100
    assert set(np.unique(inst.x_star[inst.x_star != 0])) <= {-1.0, 1.0}
    # lambda = 0.1 ||A^T b||_inf
    g = np.zeros(n)
    for j in range(n):
        g[j] = va[cp[j]:cp[j + 1]] @ inst.rhs[ri[cp[j]:cp[j + 1]]]
    assert abs(inst.lam - 0.1 * np.abs(g).max()) < 1e-12


def test_zipf_column_lengths_have_requested_mean_and_range():
    inst = acdc.gen_lasso(100000, 200000, nnz_mode=acdc.NNZ_ZIPF, zipf_s=1.5, nnz_min=1,
                          nnz_max=2000, nnz_mean=20.0, n_star=10, seed=9)
    lens = np.diff(inst.col_ptr)
    assert lens.min() >= 1 and lens.max() <= 2000
    assert abs(lens.mean() - 20.0) < 1.0
    assert (lens == 1).mean() > 0.2  # heavy head of single-entry columns


def test_svm_generator_properties():
    inst = acdc.gen_svm(300, 5000, nnz_median=60, nnz_sigma=0.8, w_star_nnz=200, flip_prob=0.05,
                        lam=1e-3, seed=3)
    rp, ci, va = inst.col_ptr, inst.row_idx, inst.vals
    assert set(np.unique(inst.rhs)) <= {-1.0, 1.0}
    for i in range(0, 300, 31):
        v = va[rp[i]:rp[i + 1]]
        assert np.all(v > 0) and abs(np.linalg.norm(v) - 1) < 1e-12
        assert np.all(np.diff(ci[rp[i]:rp[i + 1]]) > 0)
    med = np.median(np.diff(rp))
    assert 40 < med < 90


def test_nesterov_generator_support_and_optimality():
    inst = acdc.gen_nesterov(200, 500, 5, 25, lam=1.0, rho=1.0, seed=2)
    cp, ri, va = inst.col_ptr, inst.row_idx, inst.vals
    r = -inst.rhs.copy()
    for j in range(inst.n):
        r[ri[cp[j]:cp[j + 1]]] += va[cp[j]:cp[j + 1]] * inst.x_star[j]
    g = np.array([va[cp[j]:cp[j + 1]] @ r[ri[cp[j]:cp[j + 1]]] for j in range(inst.n)])
    sup = inst.x_star != 0
    assert sup.sum() == 25
    # optimality: a_j^T r = -lambda sign(x_j) on the support, |a_j^T r| <= 0.9 lambda off it
    np.testing.assert_allclose(g[sup], -np.sign(inst.x_star[sup]), atol=1e-12)
    assert np.abs(g[~sup]).max() <= 0.9 + 1e-12
    f = 0.5 * r @ r + np.abs(inst.x_star).sum()
    assert abs(f - inst.f_star) < 1e-10


def test_mix_sizes_are_log_uniform_in_range():
    ms, ns = zip(*[acdc.mix_sizes(77, i) for i in range(400)])
    assert min(ms) >= 500 and max(ms) <= 50000 and min(ns) >= 1000 and max(ns) <= 200000
    assert 0.3 < np.mean(np.log(ms) < np.log(5000)) < 0.7


def test_csc_text_loader_roundtrip(tmp_path):
    inst = acdc.gen_lasso(40, 60, nnz_per_col=3, n_star=5, seed=1)
    pre = str(tmp_path / "A")
    np.savetxt(pre + "_values.txt", inst.vals, fmt="%.17g")
    np.savetxt(pre + "_colPtr.txt", inst.col_ptr, fmt="%d")
    np.savetxt(pre + "_rowIdx.txt", inst.row_idx, fmt="%d")
    np.savetxt(str(tmp_path / "b.txt"), inst.rhs, fmt="%.17g")
    got = acdc.load_csc_text(pre, str(tmp_path / "b.txt"), 0.5)
    assert np.array_equal(got.col_ptr, inst.col_ptr)
    assert np.array_equal(got.row_idx, inst.row_idx)
    assert np.array_equal(got.vals, inst.vals) and np.array_equal(got.rhs, inst.rhs)
    # a final value without a trailing newline is kept
    with open(pre + "_values.txt", "w") as f:
        f.write(" ".join("%.17g" % v for v in inst.vals))
    assert np.array_equal(acdc.load_csc_text(pre, str(tmp_path / "b.txt"), 0.5).vals, inst.vals)


def decimal_tokens(count, seed):
    """Decimal strings of many shapes: signs, leading and trailing zeros, points at
    either end, exponents with and without signs, 1 to 24 significant digits."""
    rng = np.random.default_rng(seed)
    out = ["0", "-0", "+0.0", "0.1", "0.2", "0.3", "1e22", "1e23", "-1E-22", "9007199254740992",
           "9007199254740993", "123456789012345678", "1.7976931348623157e308", "2.2250738585072014e-308",
           "5.", ".5", "-.5e+3", "00012.5000", "1234567890123456789", "12345678901234567890", "7e0",
           "3.14159265358979323846264338327950288", "1e-0022", "0.000000000000000000000001"]
    for _ in range(count):
        nd = int(rng.integers(1, 25))
        digits = "".join(str(d) for d in rng.integers(0, 10, nd))
        if rng.random() < 0.3:
            digits = "0" * int(rng.integers(1, 4)) + digits
        point = int(rng.integers(0, len(digits) + 1))
        t = digits[:point] + ("." if rng.random() < 0.8 else "") + digits[point:]
        if rng.random() < 0.5:
            t += rng.choice(["e", "E"]) + rng.choice(["", "+", "-"]) + str(int(rng.integers(0, 40)))
        t = rng.choice(["", "-", "+"]) + t
        out.append(t)
    return out


def test_text_numbers_are_read_as_correctly_rounded_doubles(tmp_path):
    """The loaders' decimal conversion (a fast path for short decimals, strtod for
    the rest) gives the correctly rounded double of every token, as Python's
    float() does: bit for bit, signed zeros included."""
    toks = decimal_tokens(20000, 7)
    want = np.array([float(t) for t in toks])
    pre = str(tmp_path / "A")
    with open(pre + "_values.txt", "w") as f:
        f.write("\n".join(toks) + "\n")
    np.savetxt(pre + "_colPtr.txt", np.arange(len(toks) + 1), fmt="%d")
    np.savetxt(pre + "_rowIdx.txt", np.zeros(len(toks), np.int64), fmt="%d")
    np.savetxt(str(tmp_path / "b.txt"), [1.0])
    got = acdc.load_csc_text(pre, str(tmp_path / "b.txt"), 0.5).vals
    assert np.array_equal(got.view(np.int64), want.view(np.int64))
    path = str(tmp_path / "s.svm")
    with open(path, "w") as f:
        for i, t in enumerate(toks):
            f.write("%s %d:%s\n" % (t if i % 2 else "+1", i % 97 + 1, t))
    sv = acdc.load_libsvm(path, 1e-3)
    assert np.array_equal(np.asarray(sv.vals).view(np.int64), want.view(np.int64))
    labels = np.array([float(t) if i % 2 else 1.0 for i, t in enumerate(toks)])
    labels[labels == 0] = -1.0
    assert np.array_equal(np.asarray(sv.rhs), labels)


def test_csc_text_loader_rejects_bad_input(tmp_path):
    pre = str(tmp_path / "A")
    open(pre + "_values.txt", "w").write("1 2 3\n")
    open(pre + "_colPtr.txt", "w").write("0 2 3\n")
    open(pre + "_rowIdx.txt", "w").write("0 5 1\n")  # row 5 out of range for m = 2
    open(str(tmp_path / "b.txt"), "w").write("1 1\n")
    with pytest.raises(acdc.AcdcError):
        acdc.load_csc_text(pre, str(tmp_path / "b.txt"), 1.0)
    with pytest.raises(acdc.AcdcError):
        acdc.load_csc_text(str(tmp_path / "missing"), str(tmp_path / "b.txt"), 1.0)


def write_csc_binary(pre, suffix, rank, inst, b_path):
    np.savetxt("%s_colptr_%d%s" % (pre, rank, suffix), inst.col_ptr, fmt="%d")
    inst.row_idx.astype(np.int32).tofile("%s_rowid_%d%s" % (pre, rank, suffix))
    inst.vals.astype(np.float64).tofile("%s_values_%d%s" % (pre, rank, suffix))
    np.savetxt(b_path, inst.rhs, fmt="%.17g")


def test_csc_binary_loader_roundtrip(tmp_path):
    """loadANSCIAndBinaryData's per-rank format: text offsets, raw int32 rows,
    raw doubles (file_reader.h:50-106)."""
    inst = acdc.gen_lasso(50, 80, nnz_per_col=4, n_star=5, seed=2)
    pre, b_path = str(tmp_path / "A"), str(tmp_path / "b.txt")
    write_csc_binary(pre, ".dat", 3, inst, b_path)
    got = acdc.load_csc_binary(pre, ".dat", 3, b_path, inst.n, 0.5)
    assert (got.m, got.n) == (inst.m, inst.n)
    assert np.array_equal(got.col_ptr, inst.col_ptr)
    assert np.array_equal(got.row_idx, inst.row_idx)
    assert np.array_equal(got.vals, inst.vals) and np.array_equal(got.rhs, inst.rhs)
    # fewer columns than the offsets file holds: the first local_n are read
    part = acdc.load_csc_binary(pre, ".dat", 3, b_path, 10, 0.5)
    assert part.n == 10 and np.array_equal(part.col_ptr, inst.col_ptr[:11])
    assert np.array_equal(part.vals, inst.vals[:inst.col_ptr[10]])


def test_csc_binary_writer_roundtrip(tmp_path):
    """acdc_save_csc_binary writes what acdc_load_csc_binary reads: a text
    instance converted once loads back bit for bit."""
    inst = acdc.gen_lasso(70, 120, nnz_per_col=5, n_star=6, seed=4)
    pre, b_path = str(tmp_path / "A"), str(tmp_path / "b.txt")
    acdc.save_csc_binary(inst, pre, ".bin", 2)
    np.savetxt(b_path, inst.rhs, fmt="%.17g")
    got = acdc.load_csc_binary(pre, ".bin", 2, b_path, inst.n, 0.5)
    assert np.array_equal(got.col_ptr, inst.col_ptr) and np.array_equal(got.row_idx, inst.row_idx)
    assert np.array_equal(got.vals, inst.vals) and np.array_equal(got.rhs, inst.rhs)
    bad = acdc.Instance(inst.loss, inst.m, inst.n, inst.col_ptr.copy(), inst.row_idx, inst.vals,
                        inst.rhs, inst.lam)
    bad.col_ptr[3] = bad.col_ptr[4] + 1  # decreasing
    with pytest.raises(acdc.AcdcError):
        acdc.save_csc_binary(bad, pre, ".bin", 3)


def test_csc_binary_loader_rejects_bad_input(tmp_path):
    inst = acdc.gen_lasso(30, 40, nnz_per_col=3, n_star=4, seed=3)
    pre, b_path = str(tmp_path / "A"), str(tmp_path / "b.txt")
    write_csc_binary(pre, "", 0, inst, b_path)
    with pytest.raises(acdc.AcdcError):  # more columns than offsets
        acdc.load_csc_binary(pre, "", 0, b_path, inst.n + 1, 1.0)
    with pytest.raises(acdc.AcdcError):  # missing rank
        acdc.load_csc_binary(pre, "", 1, b_path, inst.n, 1.0)
    rows = inst.row_idx.astype(np.int32).copy()
    rows[5] = inst.m  # out of range
    rows.tofile(pre + "_rowid_0")
    with pytest.raises(acdc.AcdcError):
        acdc.load_csc_binary(pre, "", 0, b_path, inst.n, 1.0)
    inst.row_idx.astype(np.int32)[:-2].tofile(pre + "_rowid_0")  # truncated
    with pytest.raises(acdc.AcdcError):
        acdc.load_csc_binary(pre, "", 0, b_path, inst.n, 1.0)


def test_libsvm_loader(tmp_path):
    p = tmp_path / "d.svm"
    p.write_text("+1 1:0.5 3:1.5\n-1 2:2\n\n0 1:1 4:-1\n")
    inst = acdc.load_libsvm(str(p), 0.1)
    assert inst.n == 3 and inst.m == 4 and inst.nnz == 5
    assert inst.col_ptr.tolist() == [0, 2, 3, 5]
    assert inst.row_idx.tolist() == [0, 2, 1, 0, 3]
    assert inst.vals.tolist() == [0.5, 1.5, 2.0, 1.0, -1.0]
    assert inst.rhs.tolist() == [1.0, -1.0, -1.0]
    p.write_text("+1 0:1\n")  # indices are 1-based
    with pytest.raises(acdc.AcdcError):
        acdc.load_libsvm(str(p), 0.1)


def libsvm_reference_parse(text):
    """LIBSVM parsed line by line in Python: (row_ptr, col_idx, vals, y, d)."""
    rp, ci, va, y, d = [0], [], [], [], 0
    for line in text.split("\n"):
        t = line.strip(" \t\r")
        if not t or t.startswith("#"):
            continue
        toks = t.split()
        y.append(-1.0 if float(toks[0]) == 0 else float(toks[0]))
        for tok in toks[1:]:
            i, v = tok.split(":")
            ci.append(int(i) - 1)
            va.append(float(v))
            d = max(d, int(i))
        rp.append(len(ci))
    return np.array(rp), np.array(ci), np.array(va), np.array(y), d


@pytest.mark.parametrize("threads", [1, 2, 3, 7, 64])
def test_loaders_do_not_depend_on_threads(tmp_path, threads):
    """Every text loader cuts its file into pieces at separators and parses them
    on separate threads: the arrays match a line-by-line Python parse and the
    one-thread result for any number of pieces, including more pieces than lines
    and files without a final newline."""
    rng = np.random.default_rng(threads)
    lines = []
    for i in range(300):
        k = int(rng.integers(0, 12))
        feats = np.sort(rng.choice(5000, size=k, replace=False)) + 1
        lab = ["+1", "-1", "0"][i % 3]
        body = " ".join("%d:%.17g" % (f, rng.normal()) for f in feats)
        lines.append(("%s %s" % (lab, body)).rstrip() + (" \r" if i % 17 == 0 else ""))
        if i % 41 == 0:
            lines.append("")  # blank line
        if i % 53 == 0:
            lines.append("# comment 1:2")
    text = "\n".join(lines)  # no final newline
    p = tmp_path / "d.svm"
    p.write_text(text)
    want = libsvm_reference_parse(text)
    old = acdc.host_threads(threads)
    try:
        got = acdc.load_libsvm(str(p), 0.1)
        assert np.array_equal(got.col_ptr, want[0]) and np.array_equal(got.row_idx, want[1])
        assert np.array_equal(got.vals, want[2]) and np.array_equal(got.rhs, want[3])
        assert got.m == want[4]
        inst = acdc.gen_lasso(70, 90, nnz_per_col=4, n_star=5, seed=threads)
        pre = str(tmp_path / "A")
        with open(pre + "_values.txt", "w") as f:  # mixed separators, no final newline
            f.write("\t".join("%.17g" % v for v in inst.vals[:50]) + "\n\n  ")
            f.write("  ".join("%.17g" % v for v in inst.vals[50:]))
        np.savetxt(pre + "_colPtr.txt", inst.col_ptr, fmt="%d")
        np.savetxt(pre + "_rowIdx.txt", inst.row_idx, fmt="%d")
        np.savetxt(str(tmp_path / "b.txt"), inst.rhs, fmt="%.17g")
        c = acdc.load_csc_text(pre, str(tmp_path / "b.txt"), 0.5)
        assert np.array_equal(c.col_ptr, inst.col_ptr) and np.array_equal(c.row_idx, inst.row_idx)
        assert np.array_equal(c.vals, inst.vals) and np.array_equal(c.rhs, inst.rhs)
    finally:
        acdc.host_threads(old)


def test_loaders_refuse_non_finite_values(tmp_path):
    inst = acdc.gen_lasso(30, 40, nnz_per_col=3, n_star=4, seed=5)
    pre, b_path = str(tmp_path / "A"), str(tmp_path / "b.txt")
    np.savetxt(pre + "_colPtr.txt", inst.col_ptr, fmt="%d")
    np.savetxt(pre + "_rowIdx.txt", inst.row_idx, fmt="%d")
    for bad in ("nan", "inf", "-inf", "1e999"):
        v = [("%.17g" % x) for x in inst.vals]
        v[7] = bad
        open(pre + "_values.txt", "w").write(" ".join(v) + "\n")
        np.savetxt(b_path, inst.rhs, fmt="%.17g")
        with pytest.raises(acdc.AcdcError):
            acdc.load_csc_text(pre, b_path, 0.5)
    np.savetxt(pre + "_values.txt", inst.vals, fmt="%.17g")
    open(b_path, "w").write(" ".join(["1"] * (inst.m - 1) + ["nan"]) + "\n")
    with pytest.raises(acdc.AcdcError):
        acdc.load_csc_text(pre, b_path, 0.5)
    # binary values
    np.savetxt(b_path, inst.rhs, fmt="%.17g")
    vals = inst.vals.copy()
    vals[3] = np.nan
    acdc.save_csc_binary(acdc.Instance(inst.loss, inst.m, inst.n, inst.col_ptr, inst.row_idx,
                                       vals, inst.rhs, inst.lam), pre, "", 0)
    with pytest.raises(acdc.AcdcError):
        acdc.load_csc_binary(pre, "", 0, b_path, inst.n, 0.5)
    # LIBSVM value and label
    p = tmp_path / "d.svm"
    for text in ("+1 1:nan\n", "inf 1:0.5\n", "+1 2:1e400\n"):
        p.write_text(text)
        with pytest.raises(acdc.AcdcError):
            acdc.load_libsvm(str(p), 0.1)


def test_libsvm_value_must_follow_the_colon(tmp_path):
    p = tmp_path / "d.svm"
    p.write_text("+1 1:0.5 3:\n-1 2:2\n")  # a value may not come from the next line
    with pytest.raises(acdc.AcdcError):
        acdc.load_libsvm(str(p), 0.1)
    p.write_text("+1 1: 0.5\n")
    with pytest.raises(acdc.AcdcError):
        acdc.load_libsvm(str(p), 0.1)


def test_host_omega_matches_oracle():
    import oracle
    inst = acdc.gen_lasso(300, 900, nnz_per_col=9, n_star=5, seed=12)
    assert acdc.host_omega(inst) == oracle.omega(inst.m, inst.n, inst.col_ptr, inst.row_idx)
    assert abs(oracle.eso_beta(10, 1, 900) - 1.0) < 1e-15
    assert abs(oracle.eso_beta(10, 4096, 1e7) - (1 + 9 * 4095 / (1e7 - 1))) < 1e-15
