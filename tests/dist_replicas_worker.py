"""One rank of the replica-bookkeeping test (launched by tests/test_bench_dist.py through
torch.distributed.run, gloo on CPU): bench.py's Dist barrier, max and sum."""
import json
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import bench  # noqa: E402

D = bench.Dist()
D.barrier()
t = D.max(1.0 + D.rank)            # the slowest replica's time
w = D.sum(12 * (D.rank + 1))       # every replica's converged pairs
# one file per rank: two ranks printing to one pipe can interleave their lines
with open(os.path.join(os.environ["KF_TEST_OUT"], f"rank{D.rank}.json"), "w") as f:
    json.dump({"rank": D.rank, "world": D.world, "t": t, "w": w, "value": w / t}, f)
D.close()
