"""Row-band sharding of one problem over ranks: the band cut, and two gloo
ranks on the CPU that each compute their band (with the oracle standing in
for the GPU) and gather the condensed result on rank 0."""
import os
import socket

import numpy as np
import pytest

from stablebear_gb300 import _native as nat
from stablebear_gb300 import shard


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("skip", [nat.SKIP_LOWER_NODIAG, nat.SKIP_LOWER, nat.SKIP_NONE])
def test_row_bands_cover_align_and_balance(skip):
    for n in (1, 500, 1024, 5000, 100_000):
        for ws in (1, 2, 3, 8):
            bands = shard.row_bands(n, ws, skip, n_cols=777 if skip == nat.SKIP_NONE else None)
            assert len(bands) == ws and bands[0][0] == 0 and bands[-1][1] == n
            for (a, b), (c, d) in zip(bands, bands[1:]):
                assert b == c and a <= b
            for a, b in bands:
                if a == b:
                    continue  # an empty band (fewer windows than ranks)
                assert a % shard.WINDOW == 0 and (b % shard.WINDOW == 0 or b == n)
            if n >= 100_000:
                nc = 777 if skip == nat.SKIP_NONE else n
                sizes = [shard.output_start(skip, b, nc) - shard.output_start(skip, a, nc) for a, b in bands]
                # balanced to within one window of rows
                assert max(sizes) - min(sizes) <= 2 * shard.WINDOW * nc


def _rank_main(rank, world, port, pts, off, want_path):
    import torch
    import torch.distributed as dist
    from oracle import oracle as orc
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        n = len(off) - 1
        rb, re = shard.row_bands(n, world)[rank]
        rows = np.arange(rb, re, dtype=np.uint64)
        if len(rows):
            vals, _ = orc.evaluate_rows(pts, off, rows, threads=1)
        else:
            vals = np.zeros(0, np.float32)
        lo, hi = shard.band_output_range(nat.SKIP_LOWER_NODIAG, n, rb, re)
        assert len(vals) == hi - lo
        total = n * (n - 1) // 2
        full = shard.gather_to_rank0(lo, torch.from_numpy(np.ascontiguousarray(vals, np.float32)), total)
        if rank == 0:
            np.testing.assert_array_equal(full.numpy(), np.load(want_path))
        else:
            assert full is None
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_gather_the_condensed_matrix(tmp_path):
    import torch.multiprocessing as mp
    from oracle import oracle as orc
    from stablebear_gb300 import synthetic
    pts, off = synthetic.gaussian(2300, synthetic.uniform_lengths(1, 20), np.float32, seed=5)
    want = orc.evaluate(pts, off, threads=1)
    path = str(tmp_path / "want.npy")
    np.save(path, want)
    mp.spawn(_rank_main, args=(2, _free_port(), pts, off, path), nprocs=2, join=True)
