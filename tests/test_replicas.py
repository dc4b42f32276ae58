"""The N > 1 path of bench.py is replicas (one independent solve per GPU):
its host logic -- the whole job's time is the slowest rank's, rank 0 alone
runs the reference arm -- on CPU with the gloo backend, world size 2."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, values, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out[rank] = bench.reduce_max(values[rank], dist, "cpu")
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_reduce_max_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    values = [0.25, 0.75]
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, values, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == out[1] == 0.75


def test_reduce_max_single_rank():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_max(1.5, None, "cpu") == 1.5


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    args = bench.parse()
    called = []
    monkeypatch.setattr(bench, "oracle_solve", lambda *a, **k: called.append(1))
    monkeypatch.setattr(bench, "load_oracle", lambda: called.append(1))
    bench.run_reference(args)
    assert not called
    assert capsys.readouterr().out == ""


def test_reference_arm_prints_the_gpu_arms_metric(monkeypatch, capsys):
    """Rank 0's reference line carries the metric string and the config the
    GPU arm prints for the same workload (the solve itself is stubbed out);
    it reports the whole solves it timed as its steps."""
    import json
    import numpy as np
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "0")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--steps", "2", "--warmup", "1"])
    args = bench.parse()
    C = np.zeros((5, 5, 5, 21))

    class _O:
        @staticmethod
        def fapply(*a):
            return None

    class _BC:
        @staticmethod
        def tables():
            return None, None

    monkeypatch.setattr(bench, "workload", lambda cfg, n=0: ("tiny", 5, C, None, _BC(), 0.25))
    monkeypatch.setattr(bench, "load_oracle", lambda: (_O(), 4))
    monkeypatch.setattr(bench, "oracle_solve", lambda *a, **k: (None, None, {"seconds": 2.0, "f_cycles": 7}))
    bench.run_reference(args)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    guess = bool(args.guess) and os.path.exists(args.guess)
    assert line["impl"] == "reference"
    assert line["metric"] == bench.metric_name(5, guess)
    assert line["config"] == bench.config_dict("tiny", 5, C)
    assert line["steps"] == 2 and line["warmup"] == 1
    assert line["value"] == 2.0 and line["e2e"]["value"] == 2.0
