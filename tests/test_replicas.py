"""bench.py's N-GPU mode runs independent replicas (no data-path collective): the timing
barrier and the max over ranks, exercised with two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "CUDA_VISIBLE_DEVICES": ""})
    from curvami_gb300.replicas import Replicas

    r = Replicas()
    r.barrier()
    out[rank] = (r.rank, r.world, r.max(1.5 + rank), r.max(-rank))
    r.barrier()
    r.close()


def test_two_replicas_agree_on_the_slowest_rank():
    port = _free_port()
    with mp.get_context("spawn").Manager() as mgr:   # no fork of a threaded process
        out = mgr.dict()
        mp.start_processes(_rank, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
        res = dict(out)
    assert res[0] == (0, 2, 2.5, 0.0) and res[1] == (1, 2, 2.5, 0.0)


def test_single_process_needs_no_process_group(monkeypatch):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    from curvami_gb300.replicas import Replicas

    r = Replicas()
    assert (r.rank, r.world) == (0, 1) and r.max(3.0) == 3.0
    r.barrier()
    r.close()
