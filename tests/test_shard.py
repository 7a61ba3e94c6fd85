"""Sharding a frame over ranks: the sample-range partition and the exact
merge of per-shard means and variances, run as world-size-2 gloo ranks on
CPU; and, on one GPU, two shards of a render merging into the unsharded
render."""
import os
import socket

import numpy as np
import pytest

from lisa_gb300 import shard


def test_sample_ranges_cover_the_frame():
    for spp in (1, 7, 16, 256):
        for world in (1, 2, 3, 8):
            ranges = [shard.sample_range(k, world, spp) for k in range(world)]
            covered = sorted(i for f, c in ranges for i in range(f, f + c))
            assert covered == list(range(spp))
    with pytest.raises(ValueError):
        shard.sample_range(2, 2, 8)
    assert shard.scene_partition(5, 2) == [[0, 2, 4], [1, 3]]


def test_merge_is_exact():
    rng = np.random.default_rng(0)
    x = rng.normal(size=(37, 4, 3))
    parts = [x[:10], x[10:11], x[11:]]
    m, v, n = shard.merge([p.mean(0) for p in parts],
                          [p.var(0, ddof=1) if len(p) > 1 else np.zeros((4, 3)) for p in parts],
                          [len(p) for p in parts])
    assert n == 37
    np.testing.assert_allclose(m, x.mean(0), rtol=1e-12)
    np.testing.assert_allclose(v, x.var(0, ddof=1), rtol=1e-10)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rng = np.random.default_rng(42)
    samples = rng.normal(size=(64, 5, 3))  # the same "frame" on every rank
    first, count = shard.sample_range(rank, world, 64)
    mine = samples[first:first + count]
    res = shard.gather_merge(mine.mean(0), mine.var(0, ddof=1), count)
    if rank == 0:
        m, v, n = res
        ok = n == 64 and np.allclose(m, samples.mean(0), rtol=1e-12) and np.allclose(v, samples.var(0, ddof=1))
        out.put(bool(ok))
    dist.barrier()
    dist.destroy_process_group()


def test_gather_merge_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(k, 2, port, q)) for k in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    assert q.get(timeout=5) is True


@pytest.mark.gpu
def test_two_shards_merge_into_the_unsharded_render(gpu):
    import lisa_gb300 as L
    from lisa_gb300 import scenes

    sc = scenes.cornell_box(width=32, height=24, num_samples=8, num_bounces=5)
    full = L.Renderer(L.params_from_scene(sc))
    full.render()
    fm, fv = full.image(variance=True)
    ms, vs, cs = [], [], []
    for k in range(2):
        first, count = shard.sample_range(k, 2, 8)
        r = L.Renderer(L.params_from_scene(sc, num_samples=count))
        r.set_sample_offset(first)
        r.render()
        m, v = r.image(variance=True)
        ms.append(m)
        vs.append(v)
        cs.append(count)
    m, v, n = shard.merge(ms, vs, cs)
    assert n == 8
    np.testing.assert_allclose(m, fm, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(v, fv, rtol=1e-3, atol=1e-6)
