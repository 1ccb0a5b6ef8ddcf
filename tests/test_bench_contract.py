"""The benchmark's reference arm (CPU only): the JSON line it prints carries the keys and meanings
the benchmark contract fixes, and under a multi-rank launch only rank 0 prints."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(extra_env=None, args=("--steps", "1", "--warmup", "0")):
    env = dict(os.environ)
    env.update(extra_env or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", *args], cwd=ROOT,
                          env=env, capture_output=True, text=True, timeout=600)


def test_reference_arm_prints_one_contract_line():
    r = _run()
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["value"] > 0 and d["unit"] == "k-points/s" and d["higher_is_better"] is True
    assert d["n_gpus"] == 1 and d["steps"] == 1
    assert d["warmup"] >= 3  # at least three warm-up steps, whatever was asked
    assert d["ms_per_step"] > 0 and d["scaling"] == "weak" and d["vs_baseline"] is None
    assert d["dtype"] == "f64" and "synthetic" in d["data"]
    cfg = d["config"]
    assert "workload" in cfg and cfg["k_points_per_gpu"] == 2000 and cfg["bands"] == 16 and cfg["basis"] == 137
    assert not {"model", "global_batch", "seq_len"} & set(cfg)
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_quietly():
    r = _run({"RANK": "1", "LOCAL_RANK": "1", "WORLD_SIZE": "2"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]


def test_cli_as_shipped_baseline_is_one_thread_with_gradients():
    sys.path.insert(0, ROOT)
    import bench

    d = bench.cpu_time_cli_as_shipped(0.5)
    assert d["value"] > 0 and d["cores"] == 1 and d["kind"] == "port" and "gradients" in d["sample"]
