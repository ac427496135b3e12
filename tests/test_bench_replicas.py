'''The replica path of the benchmark on the host: two gloo ranks (127.0.0.1) each report the
slowest rank's time and the units both processed (the matvec does not shard: N GPUs run N
independent replicas with no collective on the data path, only this reduction of the clocks).'''
import importlib.util
import os
import pathlib
import socket

import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = pathlib.Path(__file__).resolve().parents[1]


def _bench():
    spec = importlib.util.spec_from_file_location('bench_under_test', ROOT / 'bench.py')
    module = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(module)
    return module


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank(rank, world, port, results):
    os.environ.update(MASTER_ADDR = '127.0.0.1', MASTER_PORT = str(port))
    dist.init_process_group('gloo', rank = rank, world_size = world)
    try:
        bench = _bench()
        mine = 100.0 * (rank + 1)  # rank 1 is the slow one
        results[rank] = bench.job_rate(mine, steps = 10, world = world)
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank_and_the_whole_job():
    world = 2
    # the manager process started with spawn, like the ranks (no fork of a threaded process)
    with mp.get_context('spawn').Manager() as manager:
        results = manager.dict()
        mp.spawn(_rank, args = (world, _free_port(), results), nprocs = world, join = True)
        for rank in range(world):
            total_ms, rate = results[rank]
            assert total_ms == 200.0
            assert abs(rate - world * 10 / 0.2) < 1e-9


def test_one_process_is_its_own_job():
    total_ms, rate = _bench().job_rate(50.0, steps = 5, world = 1)
    assert total_ms == 50.0 and abs(rate - 100.0) < 1e-9
