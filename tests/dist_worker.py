"""Worker for tests/test_replicas.py: runs under torch.distributed.run with the
gloo backend (CPU) and exercises bench.py's replica aggregation."""
import json
import os
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
import bench  # noqa: E402

dist = bench.Dist()
dist.barrier()
# rank r pretends its replica took 1 + r seconds for 10 units
value, total = bench.replica_throughput(dist, 10.0, 1.0 + dist.rank)
dist.barrier()
if dist.rank == 0:
    print(json.dumps({"ws": dist.ws, "value": value, "total": total}), flush=True)
dist.close()
