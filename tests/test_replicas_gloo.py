"""The multi-rank bench path on CPU: two gloo ranks, no GPU.

Ranks run independent replicas; the only cross-rank step is the max of the
timed region, which must agree on every rank."""
import os
import socket

import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
  with socket.socket() as s:
    s.bind(('127.0.0.1', 0))
    return s.getsockname()[1]


def _worker(rank, world, port, out):
  os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port),
                    RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
  dist.init_process_group('gloo', rank=rank, world_size=world)
  try:
    import bench  # pylint: disable=import-outside-toplevel
    out[rank] = bench.max_over_ranks(1.5 + rank)
    w, r, l = bench._dist()  # pylint: disable=protected-access
    assert (w, r, l) == (world, rank, rank)
  finally:
    dist.destroy_process_group()


def test_two_rank_max_over_ranks():
  world = 2
  with mp.get_context('spawn').Manager() as m:
    out = m.dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    assert dict(out) == {0: 2.5, 1: 2.5}


def test_single_process_is_identity():
  import bench  # pylint: disable=import-outside-toplevel
  assert bench.max_over_ranks(3.25) == 3.25
