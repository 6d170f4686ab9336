"""bench.py's reference arm on the CPU: one JSON line with the keys and meanings the benchmark
contract fixes (impl, metric, unit, value, cpu_baseline, e2e with no host-device bytes), and under a
multi-rank launch only rank 0 works and prints.  With a GPU the arm steps the pile the GPU formed;
without one (here) it pre-rolls a strip of the fill on the CPU: small sizes, the strip for a
65,536-disc pile is 2,048 discs."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = ["--impl", "reference", "--steps", "1", "--warmup", "3", "--n", "65536", "--schedule", "60:50"]


def run(env_extra):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + ARGS, cwd=ROOT, env=env,
                          capture_output=True, text=True, timeout=300)


@pytest.mark.timeout(300)
def test_reference_arm_line():
    p = run({"WORLD_SIZE": "1", "RANK": "0", "LOCAL_RANK": "0"})
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [x for x in p.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "contact-steps/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] == 1 and "strip" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["workload"].startswith("ball2d_dense_pile_")


@pytest.mark.timeout(120)
def test_reference_arm_other_ranks_exit_quietly():
    p = run({"WORLD_SIZE": "2", "RANK": "1", "LOCAL_RANK": "1"})
    assert p.returncode == 0, p.stderr[-2000:]
    assert not [x for x in p.stdout.splitlines() if x.startswith("{")]


def test_cpu_samplers_of_the_batched_legs():
    """The CPU baselines of bench.py's batched legs (which run inside its GPU legs) on tiny
    batches: a positive rate, one thread per sampled scene at most, and a description."""
    import sys

    import numpy as np
    sys.path.insert(0, ROOT)
    import bench
    from scisim_gb300 import scenes
    b = scenes.ball2d_batch(n_scenes=6, nmax=80, seed=1)
    v, threads, desc = bench.batch_cpu_sample(b, b["q"], b["v"], np.array([0, 2, 5]), 3)
    assert v is not None and v >= 0.0 and 1 <= threads <= 3 and "3 sampled scenes" in desc
    sb = scenes.sphere_batch(n_scenes=4, seed=2, nmin=20, nmax=60)
    v3, threads3, desc3 = bench.sphere_batch_cpu_sample(sb, sb["q"], sb["v"], np.array([1, 3]), 2, 5)
    assert v3 is not None and v3 >= 0.0 and 1 <= threads3 <= 2 and "2 sampled scenes" in desc3
