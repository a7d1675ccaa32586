"""Replicas on several GPUs, checked on the host: two gloo ranks on CPU.

Each rank stands for one GPU reconstructing its own scan.  The job-level
numbers must be the sum of the ranks' pairs over the slowest rank's time,
and every rank must get its own seed; nothing else is exchanged.
"""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

WORKER = r'''
import json, os, sys
sys.path.insert(0, sys.argv[1])
from muontomography_gb300.replicas import Replicas, replica_seed
rep = Replicas("gloo")
pairs = 1000.0 * (rep.rank + 1)      # rank r processed 1000 (r + 1) pairs
ms = 10.0 + 5.0 * rep.rank           # in 10 + 5 r ms
rep.barrier()
out = {"rank": rep.rank, "world": rep.world, "max_ms": rep.max(ms), "sum_pairs": rep.sum(pairs),
       "rate": rep.job_rate(pairs, ms), "seed": replica_seed(7, rep.rank)}
rep.barrier()
rep.close()
print(json.dumps(out), flush=True)
'''


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_replicas_reduce_time_and_work(tmp_path):
    pytest.importorskip("torch.distributed")
    script = tmp_path / "worker.py"
    script.write_text(WORKER)
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, str(script), str(ROOT)], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        try:
            o, e = p.communicate(timeout=120)
        except subprocess.TimeoutExpired:
            p.kill()
            raise
        assert p.returncode == 0, e
        outs.append(json.loads(o.strip().splitlines()[-1]))
    outs.sort(key=lambda d: d["rank"])
    for d in outs:
        assert d["world"] == 2
        assert d["max_ms"] == 15.0
        assert d["sum_pairs"] == 3000.0
        assert d["rate"] == pytest.approx(3000.0 / 0.015)
    assert [d["seed"] for d in outs] == [7, 1007]


def test_single_process_needs_no_group():
    sys.path.insert(0, str(ROOT))
    from muontomography_gb300.replicas import Replicas

    rep = Replicas("gloo")
    assert rep.world == 1 and rep.dist is None
    assert rep.max(3.0) == 3.0 and rep.sum(2.0) == 2.0
    assert rep.job_rate(100.0, 50.0) == 2000.0
    rep.close()
