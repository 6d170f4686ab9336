"""bench.py's roofline and convergence fields on the CPU, from synthetic profile counters: the
achieved rate is the algorithmic bytes per launch over the CUDA-event time per launch (bytes per
contact-sweep, contact-evaluation and lift as the module states them), the fraction is against the
peak bench.py reads, the kernel named is the one the counters say ran (the FP64 probe alone; the
probe with the float-float one-level and two-level continuation; the two-level FP32 sweeps; the
plain FP64 solver), and a window with one step at the cap is reported unconverged."""
import os
import sys
import types

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def prof(**over):
    p = {"gs_ms": 10.0, "gs_launches": 4, "contact_sweeps": 4_000_000, "contact_sweeps32": 0,
         "contact_evals": 2_000_000, "contact_lifts": 0, "body_lifts": 0, "two_level_solves": 0,
         "fp64_start_solves": 4, "steps": 4, "stage_ms": [0.4, 0.8, 0.8, 1.2, 0.3, 10.0, 0.3, 0.2]}
    p.update(over)
    return p


def args(precision=1):
    return types.SimpleNamespace(precision=precision)


def test_achieved_rate_and_fraction():
    p = prof()
    roof, stages = bench.headline_roofline(p, total_ms=14.0, args=args(), sweeps=[2, 4, 6, 8])
    hbm, _ = bench.peaks()
    per_launch = (4_000_000 * bench.BYTES_PER_CONTACT_SWEEP + 2_000_000 * bench.BYTES_PER_CONTACT_EVAL) / 4
    assert abs(roof["bytes_per_launch"] - per_launch) < 1e-6 * per_launch
    assert abs(roof["achieved"] - per_launch / (10.0 / 4 / 1e3) / 1e9) < 1e-9 * roof["achieved"]
    assert abs(roof["frac"] - roof["achieved"] / hbm) < 1e-12 and roof["peak"] == hbm
    assert roof["unit"] == "GB/s" and roof["bound"] == "hbm"
    assert abs(roof["gs_share_of_step"] - 10.0 / 14.0) < 1e-12
    assert stages["gauss_seidel"] == 2.5 and list(stages) == bench.STAGES


def test_kernel_named_as_run():
    r, _ = bench.headline_roofline(prof(), 14.0, args(), [2, 4, 6, 8])
    assert r["kernel"].startswith("k_gs (the FP64 probe") and "every solve converged" in r["kernel"]
    r, _ = bench.headline_roofline(prof(two_level_solves=1), 14.0, args(), [2, 11, 6, 747])
    assert "k_gs_ff1" in r["kernel"] and "k_gs_patch_ff" in r["kernel"] and "2 of 4 solves" in r["kernel"]
    r, _ = bench.headline_roofline(prof(fp64_start_solves=0, two_level_solves=4, contact_sweeps32=10**8), 14.0,
                                   args(), [400, 400, 400, 400])
    assert r["kernel"].startswith("k_gs_patch (two-level FP32 sweeps")
    r, _ = bench.headline_roofline(prof(fp64_start_solves=0), 14.0, args(precision=0), [5, 5, 5, 5])
    assert r["kernel"].startswith("k_gs (cooperative coloured block Gauss-Seidel, FP64)")


def test_unconverged_step_is_reported():
    recs = [{"converged": True, "residual": 9e-7, "sweeps": 15}, {"converged": False, "residual": 1.036e-6,
                                                                  "sweeps": 5000}]
    c = bench.convergence_record(recs)
    assert c["steps"] == 2 and c["steps_converged"] == 1 and c["all_converged"] is False
    assert c["sweeps"] == [15, 5000] and c["max_residual"] == 1.036e-6
