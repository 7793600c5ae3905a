"""bench.py's host-side logic on the CPU: the graph plan that covers exactly
the requested steps, the workload recipes, the configuration both arms
report and the roofline annotations."""
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
    cfg = bench.arm_config("dambreak1m", wl)
    assert cfg["n_fluid"] == 707 * 1414 and cfg["n_particles"] == 1027986
    assert cfg["workload"].startswith("dambreak1m: ")


def test_roofline_annotations_cover_both_forms():
    import bench
    assert set(bench.LIMITER_FROM_PROFILE) == {"mixed", "fp64"}
    per, when = bench.TRAFFIC_FROM_PROFILE[("dambreak1m", "mixed")]
    assert 0 < per < 2 * bench.PAIR_BYTES and when
    assert bench.STEP_BYTES == 32 + 144 + 24 + 81 + 104


def test_reference_arm_bounds_its_timed_steps(capsys, monkeypatch):
    """--impl reference on the CPU: full steps of the same workload, as many
    of the requested ones as fit in its time budget (here none beyond the
    minimum of one), the requested count kept in `steps` and the timed count
    in `steps_timed`, and the line's metric and configuration those of the
    GPU arm."""
    import argparse
    import json
    import bench
    monkeypatch.setattr(bench, "REFERENCE_BUDGET_S", 0.0)
    args = argparse.Namespace(steps=20, warmup=3, gpus=1)
    bench.run_reference(args, "dambreak3200")
    out = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert out["impl"] == "reference" and out["metric"] == bench.METRIC and out["unit"] == bench.UNIT
    assert out["steps"] == 20 and out["steps_timed"] == 1
    assert out["config"] == bench.arm_config("dambreak3200", bench.workload("dambreak3200"))
    assert "1 of the 20 requested" in out["cpu_baseline"]["sample"]
    assert out["value"] > 0 and out["e2e"]["value"] == out["value"]
    assert out["e2e"]["h2d_bytes_per_step"] == 0 and out["e2e"]["d2h_bytes_per_step"] == 0
