"""Replica rendering across ranks (world_size 2, gloo, CPU): disjoint sample
ranges rendered per rank and one film all-reduce equal a single-process
render of all samples.  The per-rank renderer here is the CPU oracle (the
host logic is the same for the GPU path tracer)."""
import os

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from mray_gb300 import replicas


def test_sample_ranges_partition():
    for total, world in [(16, 2), (17, 4), (5, 8), (64, 3)]:
        seen = []
        for r in range(world):
            s, c = replicas.sample_range(total, r, world)
            seen += list(range(s, s + c))
        assert seen == list(range(total))


def _worker(rank, world, port, out_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle
    from mray_gb300 import scenes
    S = oracle.PtScene(scenes.box_scene(0))
    cam = scenes.box_camera()

    def render(start, count):
        img = S.render(S.params(24, 20, count, cam, seed=3, sample_start=start), threads=2)
        return torch.from_numpy(img)
    film = replicas.render_sharded(render, 8, rank, world)
    if rank == 0:
        np.save(out_path, film.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_film_equals_single_render(tmp_path):
    import oracle
    from mray_gb300 import scenes
    out = str(tmp_path / "film.npy")
    port = 29500 + (os.getpid() % 1000)
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    got = np.load(out)
    S = oracle.PtScene(scenes.box_scene(0))
    want = S.render(S.params(24, 20, 8, scenes.box_camera(), seed=3), threads=2)
    np.testing.assert_allclose(got, want, rtol=1e-6, atol=1e-6)
    assert np.all(got[..., 3] == 8.0)


def test_more_ranks_than_samples_raises_on_every_rank():
    # every rank must raise before any of them reaches the film all-reduce
    calls = []
    for rank in range(4):
        with pytest.raises(ValueError):
            replicas.render_sharded(lambda s, c: calls.append((s, c)), 3, rank, 4)
    assert calls == []
