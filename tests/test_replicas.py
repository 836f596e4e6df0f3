"""The multi-GPU host logic on CPU: two gloo ranks (127.0.0.1) shard a multi-view batch by view,
render their views with the oracle, and rank 0 checks the gathered results against a single-process
render; the job time is the maximum over ranks and throughput counts all ranks' units."""
import ast
import hashlib
import os
import socket

import numpy as np
import pytest

from malevich_gb300 import replicas, scenes


def test_shard_is_a_balanced_partition():
    for n in (0, 1, 5, 64, 67):
        for world in (1, 2, 3, 8):
            got = [list(replicas.shard(n, r, world)) for r in range(world)]
            assert sum(got, []) == list(range(n))
            sizes = [len(g) for g in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.shard(4, 2, 2)


def test_without_a_process_group_the_local_values_are_the_job_values():
    assert replicas.job_time(1.5) == 1.5
    assert replicas.total_units(7) == 7
    assert replicas.throughput(10, 2.0) == 5.0


def _frames():
    return scenes.config3_batched(seed=7, n_views=5, n_meshes=4, resolutions=(48, 64), tri_range=(200, 2000),
                                  draws_per_view=(1, 3), tex_size=32, n_textures=2)


def _digest(out):
    h = hashlib.sha256()
    for k in ("color", "depth", "vis_tri"):
        h.update(np.ascontiguousarray(out[k]).tobytes())
    return h.hexdigest()


def _rank_main(rank, world, port, result_path):
    import torch.distributed as dist
    from oracle import pyoracle
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        frames = _frames()
        mine = {i: _digest(pyoracle.render_oracle(frames[i], threads=1)) for i in replicas.shard(len(frames), rank, world)}
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        seconds = 1.0 + rank                       # rank 1 is the slow one
        t = replicas.job_time(seconds, dist)
        units = replicas.total_units(len(mine), dist)
        rate = replicas.throughput(len(mine), seconds, dist)
        if rank == 0:
            merged = {}
            for g in gathered:
                assert not set(g) & set(merged)    # no view rendered twice
                merged.update(g)
            with open(result_path, "w") as f:
                f.write(repr({"merged": merged, "t": t, "units": units, "rate": rate}))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_shard_views_and_agree_with_one_process(tmp_path):
    import torch.multiprocessing as mp
    from oracle import pyoracle
    pyoracle.oracle_lib()                          # built before the ranks start
    out = tmp_path / "result.txt"
    mp.start_processes(_rank_main, args=(2, _free_port(), str(out)), nprocs=2, join=True, start_method="spawn")
    res = ast.literal_eval(out.read_text())
    frames = _frames()
    want = {i: _digest(pyoracle.render_oracle(f, threads=1)) for i, f in enumerate(frames)}
    assert res["merged"] == want
    assert res["t"] == 2.0                         # the slowest rank's time
    assert res["units"] == len(frames)
    assert res["rate"] == len(frames) / 2.0
