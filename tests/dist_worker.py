"""Worker of tests/test_bench_dist.py, launched as two gloo ranks by torch.distributed.run:
bench.py's multi-rank helpers (barrier, max over ranks, the broadcast that hands rank 0's
quality result and trained parameters to every rank)."""
import json
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import torch.distributed as dist  # noqa: E402

import bench  # noqa: E402

dist.init_process_group("gloo")
rank, ws = dist.get_rank(), dist.get_world_size()
slowest = bench.max_over_ranks(dist, 1.0 + 2.0 * rank)        # each rank's own frame time
bench.barrier(dist)
obj = [{"learned_at_equal_mse": {"candidates": 4}} if rank == 0 else None, [0.25, -1.5] if rank == 0 else None]
dist.broadcast_object_list(obj, src=0)
print(json.dumps({"rank": rank, "world": ws, "max": slowest, "quality": obj[0], "params": obj[1]}), flush=True)
dist.destroy_process_group()
