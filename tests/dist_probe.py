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
print(json.dumps({"rank": rank, "world": world, "local": local, "max": mx}), flush=True)
