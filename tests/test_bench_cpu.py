"""bench.py's CPU legs on the host (no GPU): the oracle's full solve of a
small workload, and the bounded sample used above 1M cells -- seconds per
outer iteration from a capped run, iterations to 1e-8 from the device
solve's count when given, else extrapolated from the residual reduction.
The reference's outer iterations get dearer as the solve proceeds (config1:
0.02 s each early on, 0.25 s on average), so a sample of the first ones
overstates the CPU's rate: a baseline that favours the CPU."""
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
    # the sample times the first outer iterations, the cheapest ones of the
    # reference's algorithm (its bottom BiCGSTAB works harder as the outer
    # residual falls): the sampled rate is not below the full solve's by
    # more than timing noise, so the bounded baseline favours the CPU
    assert s["value"] > full["value"] / 3
