"""bench.py's multi-GPU mode is replicas only (no exchange step on this path): each rank times its
own solves and rank 0 reports (sum of every rank's converged pairs) / (largest time over ranks).
This runs that bookkeeping on 2 gloo ranks on the CPU, launched like the N > 1 bench
(torch.distributed.run, 127.0.0.1)."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_replica_aggregation_two_gloo_ranks(tmp_path):
    env = dict(os.environ, OMP_NUM_THREADS="1", KF_TEST_OUT=str(tmp_path))
    # the free port is picked here and bound later by torchrun: on a busy host another process can
    # take it in between, so a failed rendezvous is retried on a fresh port
    for attempt in range(3):
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
               "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "tests", "dist_replicas_worker.py")]
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=240, env=env, cwd=ROOT)
        if r.returncode == 0:
            break
    assert r.returncode == 0, r.stderr[-3000:]
    rows = [json.loads((tmp_path / f"rank{k}.json").read_text()) for k in range(2)]
    assert sorted(x["rank"] for x in rows) == [0, 1]
    for x in rows:
        assert x["world"] == 2 and x["t"] == 2.0 and x["w"] == 36.0 and x["value"] == 18.0
