"""bench.py's host-side logic on the CPU: the graph plan that covers exactly
the requested steps, the workload recipes and their CPU samples."""
import numpy as np


def test_graph_plan_covers_exactly_the_steps():
    import bench
    for k in (1, 7, 100, 250, 2000, 2001):
        g, reps, rem = bench.graph_plan(k)
        assert g * reps + rem == k
        assert 1 <= g <= bench.GRAPH_STEPS and 0 <= rem < g


def test_dam_break_recipe_sizes():
    import bench
    wl = bench.workload("dambreak1m")
    pa = wl["pa"]
    assert int(np.sum(pa["label"] == 0)) == 707 * 1414
    assert len(pa) == 1027986
    # boundary convention of the examples: m = rho = h = 0
    b = pa["label"] != 0
    assert not np.any(pa["m"][b]) and not np.any(pa["h"][b])
    small, height, what = bench.sample("dambreak1m", wl, 60)
    assert int(np.sum(small["label"] == 0)) == 60 * 120
    assert abs(height - 1.2) < 1e-12 and "60x120" in what


def test_roofline_annotations_cover_both_forms():
    import bench
    assert set(bench.LIMITER) == {"mixed", "fp64"}
    assert bench.TRAFFIC_PER_PARTICLE[("dambreak1m", "mixed")] < bench.PAIR_BYTES
    assert bench.STEP_BYTES == 32 + 144 + 24 + 81 + 104
