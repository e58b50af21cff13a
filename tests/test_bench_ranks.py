"""The N-GPU bench path runs independent replicas (no collective on the data
path): the whole-job value is the units all ranks processed over the slowest
rank's time.  Checked here with two gloo ranks on the host: the rank set-up of
bench.py (torchrun environment, gloo without CUDA) and its reductions."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(ws), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    try:
        import bench
        r, w, lr, dist = bench.dist_init()
        assert dist is not None and dist.get_backend() == "gloo"
        # replica r processed (r + 1) * 1000 units in (r + 1) * 0.5 s
        units, secs = (r + 1) * 1000.0, (r + 1) * 0.5
        out = dict(rank=r, ws=w, mx=bench.rank_max(secs, dist), sm=bench.rank_sum(units, dist),
                   rate=bench.replica_rate(units, secs, dist))
        parts = [None] * w
        dist.all_gather_object(parts, [float(r)] * (r + 1))
        out["gathered"] = sorted(x for p in parts for x in p)
        dist.barrier()
        dist.destroy_process_group()
        q.put(out)
    except Exception as e:  # reported to the parent
        q.put(dict(rank=rank, error=repr(e)))


def test_replica_reductions_two_gloo_ranks():
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    outs = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for o in outs:
        assert "error" not in o, o
        assert o["ws"] == 2
        assert o["mx"] == 1.0          # the slowest replica
        assert o["sm"] == 3000.0       # all replicas' units
        assert o["rate"] == 3000.0     # 3000 units / 1.0 s
        assert o["gathered"] == [0.0, 1.0, 1.0]


def test_single_rank_reductions_are_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.rank_max(2.5, None) == 2.5
    assert bench.rank_sum(7.0, None) == 7.0
    assert bench.replica_rate(10.0, 2.0, None) == 5.0
    assert bench.dist_init()[3] is None or int(os.environ.get("WORLD_SIZE", "1")) > 1


def test_reference_arm_other_ranks_do_no_work(capsys):
    """Under torchrun only rank 0 times the reference's CPU path; the other
    ranks return at once and print nothing."""
    import argparse
    sys.path.insert(0, ROOT)
    import bench
    bench.run_reference(argparse.Namespace(workload="blast3d"), 1, 2)
    assert capsys.readouterr().out == ""
