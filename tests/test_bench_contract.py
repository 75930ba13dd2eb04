"""The bench's reference arm on the CPU: `bench.py --impl reference` prints
one JSON line on the same metric, unit, direction and config as the GPU arm
(the ratio of the two is taken over those), with its CPU baseline and an
end-to-end figure that moves no bytes; under torch.distributed only rank 0
prints.  (The GPU arm's line is checked by the GPU runs themselves.)"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _json_lines(out):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def _reference_line(extra_env=None, argv=()):
    env = dict(os.environ)
    env.update(extra_env or {})
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", *argv], cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return _json_lines(r.stdout)


def test_reference_arm_line_matches_the_gpu_arm_contract():
    import bench
    lines = _reference_line()
    assert len(lines) == 1, lines
    d = lines[0]
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "e2e", "cpu_baseline"):
        assert key in d, key
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == "cell-steps/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["steps"] == 1 and d["n_gpus"] == 1
    # the config both arms print for the default workload (the 256-case ensemble)
    args = bench.parse([])
    name, _ = bench.make_cases(args, 0, 0, 1)
    assert d["config"] == bench.config_of(args, name, 1)
    assert d["e2e"] == {"value": d["value"], "unit": "cell-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == "cell-steps/s" and cb["cores"] >= 1
    assert cb["kind"] == "port" and cb["sample"]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_under_torchrun_prints_on_rank_0_only():
    pytest.importorskip("torch.distributed")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"),
           "--gpus", "2", "--impl", "reference", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1 and lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2, lines
