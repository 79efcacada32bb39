"""The multi-GPU path of bench.py is replicas (frames and targets are
independent; no data-path collective): each rank times its own batch, the
job's step time is the slowest rank's, and the job's throughput counts the
units of all ranks.  Checked here with two gloo ranks on CPU:
whole_job's max-over-ranks reduction, per-rank seeding of the workload, and
that only rank 0 of the reference arm produces a line.
"""
import io
import json
import os
import socket
from contextlib import redirect_stdout

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, outdir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    w, r, _ = bench.dist_env()
    ms_max, value = bench.whole_job(10.0 * (rank + 1), 1000, w, "cpu")
    bcfg = dict(bench.BATCH_SMALL, frames=1, views=(1, 1), view_res=(32,), targets=1, target_res=(32, 32))
    wl = bench.batch_workload(bcfg, rank)
    buf = io.StringIO()

    class A:
        workload, small, steps, warmup, gpus = "plain", True, 0, 0, world

    if rank != 0:
        with redirect_stdout(buf):
            bench.run_reference(A)  # only rank 0 works and prints
    dist.barrier()
    json.dump(dict(rank=r, world=w, ms_max=ms_max, value=value, printed=buf.getvalue(),
                   ray0=[float(x) for x in wl["targets"][0]["dir"][0]]),
              open(os.path.join(outdir, f"rank{rank}.json"), "w"))
    dist.destroy_process_group()


def test_two_replicas_gloo(tmp_path):
    if not dist.is_gloo_available():
        pytest.skip("gloo backend not available")
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    for r, d in enumerate(res):
        assert d["rank"] == r and d["world"] == world
        assert d["ms_max"] == pytest.approx(20.0)            # the slowest rank's step time
        assert d["value"] == pytest.approx(2 * 1000 / 0.020)  # units of both ranks over it
    assert res[1]["printed"] == ""
    assert res[0]["ray0"] != res[1]["ray0"]  # each replica renders its own seeded targets
