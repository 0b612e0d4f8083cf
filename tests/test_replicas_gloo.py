"""The N > 1 path of bench.py on CPU: two ranks over gloo.

The trace-and-accumulate path runs as independent replicas (one scene per GPU, no data-path
collective); the only cross-rank steps are the barrier around the timed region and the
max-over-ranks of the step time, which these tests exercise with world size 2.
"""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


WORKER = r"""
import json, os, sys
sys.path.insert(0, os.environ["LG_ROOT"])
import torch
import bench
ws, rank, local = bench.dist_setup()
assert ws == 2 and torch.distributed.get_backend() == "gloo"
bench.barrier(ws)
# rank r processed 1000 units in 10 + 5 r ms: the job is bounded by the slow rank
value, ms_max = bench.aggregate(ws, 1000, 10.0 + 5.0 * rank, torch.device("cpu"))
print(json.dumps({"rank": rank, "value": value, "ms_max": ms_max}), flush=True)
torch.distributed.destroy_process_group()
"""


def _launch(code: str, extra_env=None, args=()):
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(r),
                   LOCAL_RANK=str(r), LG_ROOT=str(ROOT), CUDA_VISIBLE_DEVICES="")
        env.update(extra_env or {})
        procs.append(subprocess.Popen([sys.executable, "-c", code, *args], env=env, cwd=ROOT,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        try:
            out, err = p.communicate(timeout=240)
        except subprocess.TimeoutExpired:
            p.kill()
            out, err = p.communicate()
        assert p.returncode == 0, err[-3000:]
        outs.append(out)
    return outs


def test_two_rank_max_over_ranks():
    outs = _launch(WORKER)
    rows = [json.loads(o.strip().splitlines()[-1]) for o in outs]
    for r in rows:
        assert r["ms_max"] == 15.0
        assert r["value"] == pytest.approx(2 * 1000 / 15e-3)


REF = r"""
import os, sys
sys.path.insert(0, os.environ["LG_ROOT"])
sys.argv = ["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
            "--workload", "mid", "--cpu-stride", "16384"]
import bench
bench.main()
"""


def test_reference_arm_prints_once_on_rank_zero():
    outs = _launch(REF)
    assert outs[1].strip() == ""
    line = json.loads(outs[0].strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["value"] > 0 and line["unit"] == "segments/s"
