"""bench.py's multi-GPU path is replicas: each rank solves its own mesh, the
ranks meet at a barrier, the time is the slowest rank's and the value counts
every rank's points.  The rank logic runs here as two gloo ranks on CPU; the
reference arm runs on rank 0 alone."""
from __future__ import annotations

import contextlib
import io
import json
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    assert bench.dist_env() == (rank, world, rank)
    # rank 1 is the slow one; every rank must report its time
    ms, value = bench.replica_rate(100.0 + 50.0 * rank, n=1000, niter=10, steps=2,
                                   world=world)
    dist.barrier()
    dist.destroy_process_group()
    Path(out_dir, f"r{rank}.json").write_text(json.dumps({"ms": ms, "value": value}))


def test_replica_rate_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2,
                       start_method="spawn", join=True)
    res = [json.loads((tmp_path / f"r{k}.json").read_text()) for k in range(2)]
    for r in res:
        assert r["ms"] == 150.0                     # max over ranks
        assert r["value"] == pytest.approx(2 * 1000 * 10 * 2 / 0.150 / 1e9)


def test_replica_rate_one_rank():
    sys.path.insert(0, str(ROOT))
    import bench
    ms, value = bench.replica_rate(40.0, n=500, niter=4, steps=5, world=1)
    assert ms == 40.0 and value == pytest.approx(500 * 4 * 5 / 0.040 / 1e9)


def test_reference_arm_runs_on_rank_zero_only():
    sys.path.insert(0, str(ROOT))
    import bench

    class A:
        pass
    a = A()
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.run_reference(a, rank=1, world=2)   # returns before touching a
    assert buf.getvalue() == ""


def test_global_ids_match_set_vert_box():
    """The bench's numpy global numbering is set_vert_box's (the oracle's
    restatement of prox_dssum.f:42-73) on a brick box."""
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests"))
    import numpy as np
    import bench
    import oracle_lib as O
    for nel, lx in ((3, 5), (2, 12), (1, 2)):
        nelt = nel ** 3
        ref = O.set_vert_box(lx, nelt, nel, nel, nel, np.arange(1, nelt + 1))
        assert np.array_equal(bench.global_ids(nel, lx), ref)


def test_reference_arm_line_small_case():
    """The reference arm on a small box prints one line with the workload
    config our arm prints, the CPU baseline it measured and no copies."""
    sys.path.insert(0, str(ROOT))
    import bench

    class A:
        pass
    a = A()
    a.nel, a.lx, a.niter, a.steps, a.warmup, a.cpu_sample_iters, a.gpus = 2, 6, 100, 2, 1, 3, 1
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.run_reference(a, rank=0, world=1)
    line = json.loads(buf.getvalue().strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["config"] == bench.workload_config(2, 6, 100)
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["higher_is_better"] is True and line["unit"] == bench.UNIT
