"""One rank of the two-process gloo test in test_multirank.py (run as a
script with RANK, WORLD_SIZE, MASTER_PORT and OUT in the environment)."""
import json
import os
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402
import torch.distributed as dist  # noqa: E402

from openholo_gb300 import scenes  # noqa: E402
from openholo_gb300.shard import max_over_ranks, rank_seed, shard  # noqa: E402


def unit_checksum(u: int) -> int:
    img, depth = scenes.depthmap_scene(rank_seed(100, u), 24, 32)
    return int(np.asarray(img, dtype=np.int64).sum() * 1000003 + np.asarray(depth, dtype=np.int64).sum())


def main():
    rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{os.environ['MASTER_PORT']}", rank=rank,
                            world_size=world)
    units = list(range(int(os.environ.get("UNITS", "7"))))
    mine = shard(units, rank, world)
    done = {u: unit_checksum(u) for u in mine}          # this rank's frames, no exchange
    # the test's own check gathers the per-rank results; the path itself has no collective
    gathered = [None] * world
    dist.all_gather_object(gathered, done)
    slowest = max_over_ranks(1.5 * (rank + 1), dist)
    Path(os.environ["OUT"]).write_text(json.dumps({"rank": rank, "mine": mine, "gathered": gathered,
                                                   "slowest": slowest}))
    dist.barrier()
    dist.destroy_process_group()


if __name__ == "__main__":
    main()
