"""The multi-rank path of bench.py on CPU: two gloo ranks started by torch.distributed.run (the
launcher a multi-GPU run uses, on 127.0.0.1) through tmc_gb300.replicas.  Each rank extracts its
own volume (a seed per rank, no collective on the data path); the job time is the maximum over the
ranks, and the whole-job throughput counts the cells of every rank; rank 0 alone reports."""
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


def test_two_gloo_ranks(tmp_path):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={_free_port()}",
           os.path.join(ROOT, "tests", "replicas_worker.py"), str(tmp_path)]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    res = [json.load(open(tmp_path / f"rank{k}.json")) for k in range(2)]
    assert [x["rank"] for x in res] == [0, 1] and all(x["world"] == 2 for x in res)
    assert res[0]["seed"] != res[1]["seed"] and res[0]["checksum"] != res[1]["checksum"]
    assert all(x["slowest"] == 2.5 for x in res)  # max over ranks of 1.5 + rank
    assert [x["reports"] for x in res] == [True, False]
    cells = 15 ** 3
    assert all(abs(x["throughput"] - 2 * cells * 3 / 2.5 / 1e9) < 1e-15 for x in res)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    from tmc_gb300 import replicas
    rep = replicas.Replicas(1, "gloo")
    rep.barrier()
    assert rep.max_over_ranks(3.25) == 3.25
    rep.close()
    assert replicas.reports(0) and not replicas.reports(1)
