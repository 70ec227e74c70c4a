"""Child process of test_dist.py (one rank of torch.distributed.run): the
bench's replica plumbing -- rank set-up, per-rank seeded workloads,
barrier, max-reduction of the step time."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def main():
    ws, rank, local, td = bench.dist_setup()
    work = bench.heldout_models(rank, 2, 3)
    seeds = [float(m["hs"]) for m, _ in work]
    bench.barrier(td)
    t = bench.allmax(td, 1.0 + rank)
    # one write per line: the two ranks share the pipe
    sys.stdout.flush()
    os.write(1, (json.dumps({"rank": rank, "ws": ws, "max": t, "hs": seeds}) + "\n").encode())
    bench.barrier(td)


if __name__ == "__main__":
    main()
