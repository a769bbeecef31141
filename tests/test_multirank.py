"""N > 1 host path on CPU: frame sharding, per-rank seeds and the slowest-
rank timing reduction, run as two gloo ranks (one process each)."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from openholo_gb300 import scenes
from openholo_gb300.shard import max_over_ranks, rank_seed, shard, shard_range

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
@pytest.mark.parametrize("n", [0, 1, 2, 7, 64, 65])
def test_shard_range_partitions(n, world):
    spans = [shard_range(n, r, world) for r in range(world)]
    assert spans[0][0] == 0 and spans[-1][1] == n
    for (a, b), (c, d) in zip(spans, spans[1:]):
        assert b == c
    sizes = [b - a for a, b in spans]
    assert max(sizes) - min(sizes) <= 1
    assert shard(list(range(n)), world - 1, world) == list(range(*spans[-1]))


def test_shard_range_rejects_bad_ranks():
    with pytest.raises(ValueError):
        shard_range(4, 2, 2)
    with pytest.raises(ValueError):
        shard_range(4, 0, 0)
    with pytest.raises(ValueError):
        shard_range(-1, 0, 1)


def test_rank_seeds_give_distinct_frames():
    a = scenes.depthmap_scene(rank_seed(2024, 0), 16, 16)[0]
    b = scenes.depthmap_scene(rank_seed(2024, 1), 16, 16)[0]
    assert not np.array_equal(a, b)
    assert max_over_ranks(3.25) == 3.25           # no process group: the value itself


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks(tmp_path):
    world, units = 2, 7
    port = _free_port()
    procs, outs = [], []
    for r in range(world):
        out = tmp_path / f"rank{r}.json"
        env = dict(os.environ, RANK=str(r), WORLD_SIZE=str(world), LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), OUT=str(out), UNITS=str(units))
        procs.append(subprocess.Popen([sys.executable, str(ROOT / "tests" / "multirank_worker.py")], env=env))
        outs.append(out)
    for p in procs:
        assert p.wait(timeout=120) == 0
    res = [json.loads(o.read_text()) for o in outs]
    # disjoint contiguous shards covering every unit, in rank order
    assert res[0]["mine"] + res[1]["mine"] == list(range(units))
    # every rank's results equal the single-process ones
    sys.path.insert(0, str(ROOT / "tests"))
    from multirank_worker import unit_checksum
    merged = {}
    for part in res[0]["gathered"]:
        merged.update({int(k): v for k, v in part.items()})
    assert merged == {u: unit_checksum(u) for u in range(units)}
    assert res[0]["gathered"] == res[1]["gathered"]
    # slowest-rank reduction
    assert res[0]["slowest"] == res[1]["slowest"] == 3.0


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "3", "--warmup", "3"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
