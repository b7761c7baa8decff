"""One rank of the two-rank gloo test (tests/test_replicas_gloo.py), started by torch.distributed.run:
the helpers bench.py uses for its multi-GPU runs, on CPU.  Writes this rank's results to
<out>/rank<r>.json."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from tmc_gb300 import replicas, volumes  # noqa: E402


def main(out_dir):
    rank, world, local = replicas.dist_env()
    rep = replicas.Replicas(world, "gloo", local)
    rep.barrier()
    # each replica extracts its own volume: a different seed per rank
    seed = replicas.replica_seed(7, rank)
    vol = volumes.small_noise_volume(16, seed=seed)
    t = 1.5 + rank  # a rank-dependent "time"; the job time is the slowest rank's
    slowest = rep.max_over_ranks(t)
    rep.barrier()
    rep.close()
    res = {"rank": rank, "world": world, "local": local, "seed": seed, "checksum": float(vol.data.astype("float64").sum()),
           "slowest": slowest, "reports": replicas.reports(rank),
           "throughput": replicas.throughput(world, vol.cells, 3, slowest)}
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump(res, f)


if __name__ == "__main__":
    main(sys.argv[1])
