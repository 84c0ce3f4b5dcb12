"""bench.py's reference arm (the CPU restatement of the reference's path)
prints the benchmark line the harness reads; it needs no GPU."""
import json
import os
import subprocess
import sys

from conftest import REPO


def run_bench(args, env_extra=None):
    env = dict(os.environ)
    env.update(env_extra or {})
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py")] + args,
                         capture_output=True, text=True, timeout=600, cwd=REPO, env=env)
    assert out.returncode == 0, out.stdout[-2000:] + out.stderr[-2000:]
    return out.stdout


def test_reference_arm_prints_the_benchmark_line():
    lines = [l for l in run_bench(["--impl", "reference", "--steps", "2", "--warmup", "1"])
             .splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for key in ("metric", "unit", "dtype", "data", "scaling"):
        assert isinstance(d[key], str) and d[key]
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert (d["steps"], d["warmup"], d["n_gpus"]) == (2, 1, 1)
    assert d["higher_is_better"] is True and d["vs_baseline"] is None
    assert d["config"]["workload"]
    cpu = d["cpu_baseline"]
    assert cpu["kind"] in ("reference", "port") and cpu["cores"] >= 1 and cpu["sample"]
    assert cpu["value"] == d["value"] and cpu["unit"] == d["unit"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    # labelled as the CPU port, and on exactly the engine arm's config
    assert d["reference_class"] == "cpu_port_of_reference_algorithm"
    assert d["comparable_to_reference_cuda_build"] is False
    sys.path.insert(0, REPO)
    import bench
    assert d["config"] == json.loads(json.dumps(bench.WORKLOAD))


def test_reference_arm_runs_on_rank_zero_only():
    out = run_bench(["--impl", "reference", "--steps", "1", "--warmup", "0"],
                    {"RANK": "1", "LOCAL_RANK": "1", "WORLD_SIZE": "2"})
    assert not [l for l in out.splitlines() if l.startswith("{")]
