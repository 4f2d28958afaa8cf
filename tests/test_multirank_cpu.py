"""The multi-rank path of bench.py on CPU: two gloo ranks (world size 2,
127.0.0.1) run the rendezvous, barrier and max-over-ranks helpers, each rank
draws its own ensemble shard (seed 4 + rank, no data-path collective), and
the whole-job value uses the slowest rank's time.  The reference arm runs on
rank 0 only."""
import json
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, outdir):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(ws),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "lowrankintegrators.jl_gb300"))
    import bench
    import workloads
    ws_, rk, local, dist = bench.dist_setup()
    assert (ws_, rk) == (ws, rank) and dist is not None
    bench.rank_barrier(dist)
    t_max = bench.rank_max(1.0 + rank, dist)   # rank 1 is the slow one
    shard = workloads.lyapunov_ensemble(count=8, seed=4 + rank, limit=2)
    value = bench.weak_value(ws, 10, t_max)
    with open(os.path.join(outdir, f"rank{rank}.json"), "w") as f:
        json.dump({"t_max": t_max, "value": value, "first_n": int(shard[0].U.shape[0]),
                   "first_s": float(shard[0].A[1][0])}, f)
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    ws, port = 2, _free_port()
    mp.start_processes(_rank_main, args=(ws, port, str(tmp_path)), nprocs=ws, join=True, start_method="spawn")
    r = [json.load(open(tmp_path / f"rank{i}.json")) for i in range(ws)]
    assert r[0]["t_max"] == r[1]["t_max"] == 2.0
    assert r[0]["value"] == r[1]["value"] == pytest.approx(ws * 10 / 2.0)
    # independent shards: different draws on the two ranks
    assert (r[0]["first_n"], r[0]["first_s"]) != (r[1]["first_n"], r[1]["first_s"])


def test_reference_arm_rank_nonzero_is_silent(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        count, cpu_sample_every, steps, warmup = 64, 64, 1, 3

    bench.run_reference(Args(), 2, 1)
    assert capsys.readouterr().out == ""
