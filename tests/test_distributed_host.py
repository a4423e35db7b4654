"""The multi-process path on CPU: two gloo ranks shard a sample stream (the
host-side replay), gather it in rank order and agree with one process; the
bench's barrier and max-over-ranks timing."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, result_dir):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        from theboss_gb300 import _native
        from theboss_gb300.distributed import gather_rows, shard

        inp = [1] * 6 + [0] * 6
        w = [1 / 7] * 7
        N = 101
        np.random.seed(17)
        kept, popped, uni = _native.gccb_predraw(inp, w, N)  # every rank replays the whole stream
        first, count = shard(N, rank, world)
        rows = np.concatenate([kept[first:first + count, None], popped[first:first + count],
                               uni[first:first + count]], axis=1)
        full = gather_rows(rows)
        after = np.random.random()
        t = bench._max_over_ranks(float(rank + 1), world)
        bench._barrier(world)
        np.save(os.path.join(result_dir, f"rank{rank}.npy"), full)
        np.save(os.path.join(result_dir, f"rank{rank}_extra.npy"), np.array([after, t, count]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reassemble_the_single_process_stream(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    from theboss_gb300 import _native

    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    np.random.seed(17)
    inp = [1] * 6 + [0] * 6
    w = [1 / 7] * 7
    kept, popped, uni = _native.gccb_predraw(inp, w, 101)
    single = np.concatenate([kept[:, None], popped, uni], axis=1)
    after = np.random.random()
    counts = []
    for r in range(world):
        full = np.load(tmp_path / f"rank{r}.npy")
        assert np.array_equal(full, single)
        extra = np.load(tmp_path / f"rank{r}_extra.npy")
        assert extra[0] == after          # both ranks leave numpy's generator where one process does
        assert extra[1] == float(world)   # max over ranks
        counts.append(int(extra[2]))
    assert counts == [51, 50]


def test_shard_bounds():
    from theboss_gb300.distributed import shard

    for n in (0, 1, 7, 100, 10007):
        for world in (1, 2, 3, 8):
            parts = [shard(n, r, world) for r in range(world)]
            assert parts[0][0] == 0 and sum(c for _, c in parts) == n
            assert all(parts[r][0] + parts[r][1] == parts[r + 1][0] for r in range(world - 1))
            assert max(c for _, c in parts) - min(c for _, c in parts) <= 1
    with pytest.raises(ValueError):
        shard(10, 2, 2)
