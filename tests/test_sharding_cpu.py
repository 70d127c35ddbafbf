"""Batch sharding without a GPU: fyg_partition's contiguous cost-balanced shards, and the
one-process-per-device path as world_size-2 gloo ranks on the CPU (each rank takes its shard of
the mixed-length batch from fyg_partition and transforms it; the gathered shards must cover the
batch exactly once and reproduce the unsharded result)."""
import math
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fyfft_gb300 as fg  # noqa: E402
from fyfft_gb300.workloads import uneven_lengths  # noqa: E402
from oracle import oracle as O  # noqa: E402


def _lib_or_skip():
    try:
        fg.lib()
    except RuntimeError as e:
        pytest.skip(str(e))


@pytest.mark.parametrize("count,parts", [(64, 1), (64, 2), (64, 3), (10, 4), (3, 8), (0, 2), (4096, 8)])
def test_uniform_partition(count, parts):
    _lib_or_skip()
    b = fg.partition(count, parts)
    assert b[0] == 0 and b[-1] == count and len(b) == parts + 1
    sizes = np.diff(b)
    assert (sizes >= 0).all() and sizes.max() - sizes.min() <= 1


@pytest.mark.parametrize("parts", [1, 2, 3, 4, 8])
def test_uneven_partition_is_contiguous_and_balanced(parts):
    _lib_or_skip()
    lengths = uneven_lengths(4096, 2)
    b = fg.partition(lengths, parts)
    assert b[0] == 0 and b[-1] == len(lengths) and all(x <= y for x, y in zip(b, b[1:]))
    cost = [sum(n * math.log2(n) for n in lengths[b[i]:b[i + 1]]) for i in range(parts)]
    largest = max(n * math.log2(n) for n in lengths)
    # every shard is within one transform's cost of the ideal share
    assert max(cost) - sum(cost) / parts <= largest


def test_partition_rejects_bad_arguments():
    _lib_or_skip()
    with pytest.raises(fg.FygError):
        fg.partition(10, 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, lengths, result_path):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    b = fg.partition(lengths, world)
    lo, hi = b[rank], b[rank + 1]
    # every rank derives the same partition on its own
    allb = [None] * world
    dist.all_gather_object(allb, b)
    assert all(x == b for x in allb)
    # this rank's shard: inputs from the seeded stream at the shard's offsets, transformed
    offs = np.concatenate([[0], np.cumsum(lengths)])
    x = O.fill_random(2, int(offs[-1]), np.complex64, "uniform")
    mine = [O.fft(x[offs[k]:offs[k + 1]]) for k in range(lo, hi)]
    shards = [None] * world
    dist.all_gather_object(shards, (lo, hi, mine))
    if rank == 0:
        got = {}
        for (a, z, ys) in shards:
            for k, y in zip(range(a, z), ys):
                assert k not in got
                got[k] = y
        assert sorted(got) == list(range(len(lengths)))
        ok = all(np.array_equal(got[k], O.fft(x[offs[k]:offs[k + 1]])) for k in range(len(lengths)))
        with open(result_path, "w") as f:
            f.write("ok" if ok else "mismatch")
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_the_mixed_batch(tmp_path):
    _lib_or_skip()
    import torch.multiprocessing as mp
    lengths = uneven_lengths(96, 5)
    path = str(tmp_path / "result.txt")
    mp.start_processes(_rank, args=(2, _free_port(), lengths, path), nprocs=2, join=True, start_method="spawn")
    assert open(path).read() == "ok"
