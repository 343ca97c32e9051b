"""Multi-process path of the benchmark on CPU (gloo, world size 2): every rank steps its own
replica of the workload (here the oracle on a small domain, standing in for one GPU's model),
the job's time is the slowest rank's and its work the sum over ranks. No collective touches the
data path; the only collective is the max of the ranks' times."""

import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import sys
    import time
    from pathlib import Path

    root = Path(__file__).resolve().parent.parent
    for p in (root / "wflow.jl_gb300", root / "oracle", root):
        sys.path.insert(0, str(p))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import bench
    import oracle_py as O
    from wflow_gb300 import synthetic

    dist.init_process_group("gloo", rank=rank, world_size=world)
    dom = synthetic.make_domain(16, 1000.0, seed=5)
    cfg = synthetic.make_config(86400.0)
    orc = O.OracleModel(cfg, dom)
    t0 = time.perf_counter()
    for s in range(3):
        orc.set_forcing(*synthetic.forcing(s, cfg.dt, dom.n_land, seed=5))
        orc.step()
    local = time.perf_counter() - t0 + 0.05 * rank  # ranks differ in speed
    value, job = bench.whole_job_rate(local, dom.n_land, 3)
    np.save(os.path.join(out_dir, f"r{rank}.npy"),
            np.concatenate([[local, job, value], orc.get(synthetic.abi.FIELD["RIVER_Q"])]))
    dist.destroy_process_group()


def test_replicas_gloo_two_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    r = [np.load(tmp_path / f"r{k}.npy") for k in range(world)]
    locals_ = [x[0] for x in r]
    for x in r:
        assert x[1] == pytest.approx(max(locals_))          # job time = slowest rank
        assert x[2] == pytest.approx(256 * 3 * world / max(locals_))  # work summed over ranks
    assert np.array_equal(r[0][3:], r[1][3:])               # replicas compute the same state
