"""bench.py's bookkeeping on CPU: the split of a solve's update bulks into
uniform and q-shrinking kinds from its trace rows, and the names of the update
kernels a setting launches."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "ac-dc_gb300"))

import acdc  # noqa: E402
import bench  # noqa: E402


def row(updates, shrink, fp64, ms):
    return {"updates": updates, "shrink": shrink, "fp64": fp64, "update_ms": ms}


def test_bulk_phases_split_the_trace_by_kind():
    s = acdc.default_settings(tau=4096, tau_active=1024, use_shrinking=1)
    # trace rows hold the cumulative updates after each bulk; row 0 is the
    # evaluation before the first bulk
    trace = [row(0, 0, 0, 0.0), row(5_000_000, 0, 0, 2.0), row(7_000_000, 1, 0, 1.5),
             row(8_000_000, 1, 1, 1.0)]
    out = bench.bulk_phases([trace, trace], s)
    assert set(out) == {"uniform", "active", "active_fp64"}
    u, a, f = out["uniform"], out["active"], out["active_fp64"]
    assert (u["bulks"], u["updates"], u["ms"], u["in_flight"]) == (2, 10_000_000, 4.0, 4096)
    assert (a["bulks"], a["updates"], a["ms"], a["in_flight"]) == (2, 4_000_000, 3.0, 1024)
    assert (f["bulks"], f["updates"], f["in_flight"]) == (2, 2_000_000, 1024)
    assert abs(u["updates_per_s"] - 2.5e9) < 1
    # in flight x time / updates: 4096 x 4 ms / 1e7 = 1.6384 us
    assert abs(u["us_per_update_in_flight"] - 1.6384) < 1e-12
    assert abs(a["us_per_update_in_flight"] - 0.768) < 1e-12


def test_bulk_phases_without_tau_active_use_tau():
    s = acdc.default_settings(tau=256, tau_active=0, use_shrinking=1)
    out = bench.bulk_phases([[row(0, 0, 0, 0.0), row(1000, 1, 0, 1.0)]], s)
    assert out["active"]["in_flight"] == 256


def test_update_kernel_label_names_the_launched_kernels():
    lasso = {"loss": "lasso"}
    svm = {"loss": "svm"}
    shrink = acdc.default_settings(use_shrinking=1)
    assert "k_pcdm_update_lean" in bench.update_kernel_label(shrink, lasso)
    assert "k_pcdm_update " in bench.update_kernel_label(shrink, lasso)
    ring = acdc.default_settings(use_shrinking=1, lanes_per_update=-1)
    assert bench.update_kernel_label(ring, lasso) == "k_pcdm_update"
    assert bench.update_kernel_label(acdc.default_settings(lanes_per_update=1), lasso) == \
        "k_pcdm_update_lean"
    assert bench.update_kernel_label(acdc.default_settings(lanes_per_update=16), lasso) == \
        "k_pcdm_update_grouped<16>"
    mb = acdc.default_settings(acdc.LOSS_SVM_DUAL, minibatch=1)
    assert bench.update_kernel_label(mb, svm).startswith("k_sdca_phase1")
