"""The multi-GPU form of the benchmark on the host: replicas over disjoint
sample ranges, the step time reduced as the MAX over ranks, the whole-job
rate.  Two gloo ranks on the CPU run the same helpers bench.py runs under
torchrun (no GPU)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from conftest import ROOT

import sys
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        # each rank's own step times; the MAX over ranks reaches every rank
        mine = [10.0 + rank, 3.0 - rank, 7.0]
        out[rank] = bench.max_over_ranks(mine, world, 'cpu')
    finally:
        dist.destroy_process_group()


def test_step_time_is_the_max_over_two_gloo_ranks():
    world = 2
    port = _free_port()
    ctx = mp.get_context('spawn')
    with ctx.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_rank_main, args=(world, port, out), nprocs=world, join=True,
                           start_method='spawn')
        res = dict(out)
    assert res[0] == res[1] == [11.0, 3.0, 7.0]


def test_single_rank_reduction_is_the_identity():
    assert bench.max_over_ranks([1.5, 2.5], 1, 'cpu') == [1.5, 2.5]


def test_replicas_take_disjoint_ranges_of_the_same_draws():
    """Rank r's disorder offsets are samples r S .. (r + 1) S - 1 of one seeded
    draw, so N replicas compute what one device would on N S samples."""
    import qspectra_gb300 as qg
    from qspectra_gb300 import workloads as wl
    H = wl.fmo7_hamiltonian()
    ham = qg.ElectronicHamiltonian(H, bath=qg.DebyeBath(qg.CM_K * 77, 35, 106),
                                   dipoles=[[1, 0, 0]] * 7, disorder=wl.fwhm_for_sd(80.0),
                                   random_seed=1)
    S, world = 6, 3
    whole = ham.disorder_offsets(S * world)
    parts = [ham.disorder_offsets(S, start=bench.replica_sample_start(r, S))
             for r in range(world)]
    assert np.array_equal(np.concatenate(parts), whole)
    starts = [bench.replica_sample_start(r, S) for r in range(world)]
    assert starts == [0, S, 2 * S]


def test_whole_job_rate_counts_every_rank():
    assert bench.whole_job_rate(1, 2.0) == pytest.approx(500.0)
    assert bench.whole_job_rate(4, 2.0) == pytest.approx(2000.0)
