"""Two-rank host-logic probe for the replica path of bench.py, run under
torch.distributed.run by tests/test_replicas_gloo.py (gloo, CPU only)."""
import json
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402

world, rank, local = bench.dist_setup()
mx = bench.dist_max(10.0 * (rank + 1), world)
bench.dist_barrier(world)
# one write per line: the ranks share the launcher's stdout pipe, and a single
# write of less than PIPE_BUF bytes is not interleaved with the other rank's
os.write(1, (json.dumps({"rank": rank, "world": world, "local": local, "max": mx}) + "\n").encode())
