"""bench.py's CPU legs on the host (no GPU): the oracle's full solve of a
small workload, and the bounded sample used above 1M cells -- seconds per
outer iteration from a capped run, iterations to 1e-8 from the device
solve's count when given, else extrapolated from the residual reduction."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_full_and_bounded_cpu_solves():
    sys.path.insert(0, ROOT)
    import bench
    from sayakaamr_gb300 import workloads
    p = workloads.config1()
    full = bench.cpu_solve(p)
    assert full["status"] == 0 and not full["sampled"] and full["iterations"] > 0
    assert full["value"] > 0
    s = bench.cpu_solve(p, budget_s=0.2, n_iters=full["iterations"])
    assert s["sampled"] and s["sample_iterations"] >= 3
    if s["sample_iterations"] < full["iterations"]:
        assert s["iterations"] == full["iterations"]
    assert s["status"] == 0 and s["value"] > 0 and s["per_iteration"] > 0
    # the sampled rate agrees with the full solve's to within a factor 3
    assert full["value"] / 3 < s["value"] < full["value"] * 3
