"""Sample-range sharding over two ranks (gloo on the CPU): the ranks' ranges
partition the frame's samples, and the summed per-rank accumulators equal the
single-rank render (the oracle stands in for the per-rank GPU render, with
the same per-sample PCG32 streams)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from voidray_gb300.shard import sample_range


def test_sample_ranges_partition():
    for total in (0, 1, 7, 64, 1001):
        for world in (1, 2, 3, 8):
            got = sorted(sample_range(total, r, world) for r in range(world))
            at = 0
            for first, count in got:
                assert first == at
                at += count
            assert at == total
            assert max(c for _, c in got) - min(c for _, c in got) <= 1
    with pytest.raises(ValueError):
        sample_range(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, total, out_dir):
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    sys.path.insert(0, str(root))
    sys.path.insert(0, str(root / "oracle"))
    import torch
    import torch.distributed as dist

    import pyoracle
    from voidray_gb300 import workloads as W
    from voidray_gb300.shard import reduce_image, sample_range

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    scene, st = W.cornell_box(rr_depth=3)
    first, count = sample_range(total, rank, world)
    w = h = 24
    img, _ = pyoracle.OracleScene(scene).render(st, count, w, h, seed=3, first_sample=first, threads=1)
    buf = torch.from_numpy(np.ascontiguousarray(img[..., :3], dtype=np.float64))
    reduce_image(buf)
    np.save(os.path.join(out_dir, f"rank{rank}.npy"), buf.numpy())
    dist.destroy_process_group()


def test_two_rank_render_sums_to_single_rank(tmp_path, oracle):
    from voidray_gb300 import workloads as W

    total = 8
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, total, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    a, b = np.load(tmp_path / "rank0.npy"), np.load(tmp_path / "rank1.npy")
    assert np.array_equal(a, b)  # every rank holds the sum
    scene, st = W.cornell_box(rr_depth=3)
    full, _ = oracle.OracleScene(scene).render(st, total, 24, 24, seed=3, threads=1)
    assert np.allclose(a, full[..., :3], rtol=1e-5, atol=1e-7)
