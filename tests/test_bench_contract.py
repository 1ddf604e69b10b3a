"""bench.py's reference arm runs on the CPU: it prints one JSON line with the contract's keys
(the reference's compute shader compiled for the CPU, timed on host threads)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    if "unavailable" in d:  # no reference build on this machine: the one-line reason
        assert isinstance(d["unavailable"], str) and d["unavailable"]
        return
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["value"] > 0 and d["unit"] == "cell-updates/s" and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 0
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["workload"].startswith("world16384")


def test_gpus_2_relaunches_two_ranks():
    """bench.py --gpus 2 outside a torch.distributed environment relaunches itself under
    torch.distributed.run with two ranks (gloo here, as the reference arm uses): one JSON
    line, from rank 0, saying n_gpus 2; the other rank exits 0 without work."""
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", "--workload", "world256",
                        "--steps", "1", "--warmup", "0"], cwd=ROOT, capture_output=True, text=True, timeout=600,
                       env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
    assert d["value"] > 0


def test_replica_pinning_selects_one_gpu_per_rank(monkeypatch):
    """With NCCL, rank i sees only the i-th visible GPU (CUDA_VISIBLE_DEVICES), so the
    library's kernels and torch agree on the device; checked without a GPU by stopping
    before the process group starts."""
    import sandengine_gb300.replicas as R
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "4,5")

    class Stop(Exception):
        pass

    import torch
    monkeypatch.setattr(torch.cuda, "set_device", lambda d: (_ for _ in ()).throw(Stop(d)))
    try:
        R.Replicas("nccl")
    except Stop as e:
        assert e.args[0] == 0
    assert os.environ["CUDA_VISIBLE_DEVICES"] == "5"
