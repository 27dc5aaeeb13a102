"""The replica path of bench.py on the host: two gloo ranks (world size 2,
127.0.0.1 rendezvous), each timing its own independent work.  The job's time
is the slowest rank's, every rank learns it, and the ranks exchange nothing
else."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world)})
    from exwave_gb300.replicas import Replicas
    rep = Replicas("gloo")
    assert (rep.world_size, rep.rank) == (world, rank)
    rep.barrier()
    # each rank's own "timed region": different durations per rank
    mine = 10.0 + 5.0 * rank
    slowest = rep.max(mine)
    rep.barrier()
    with open(os.path.join(out_dir, "rank%d.txt" % rank), "w") as f:
        f.write("%r %r\n" % (mine, slowest))
    rep.close()


def test_two_gloo_ranks_reduce_the_slowest_time(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    vals = [open(tmp_path / ("rank%d.txt" % r)).read().split() for r in range(2)]
    assert [float(v[0]) for v in vals] == [10.0, 15.0]
    assert all(float(v[1]) == 15.0 for v in vals)


def test_single_process_needs_no_group(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    from exwave_gb300.replicas import Replicas
    rep = Replicas("gloo")
    assert rep.world_size == 1 and rep.rank == 0
    rep.barrier()
    assert rep.max(3.5) == 3.5
    rep.close()


@pytest.mark.parametrize("rank", [1, 3])
def test_other_ranks_leave_the_reference_arm(monkeypatch, capsys, rank):
    """bench.py --impl reference under torchrun: only rank 0 runs and prints."""
    import importlib.util
    monkeypatch.setenv("WORLD_SIZE", "4")
    monkeypatch.setenv("RANK", str(rank))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(root, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    monkeypatch.setattr("sys.argv", ["bench.py", "--impl", "reference", "--gpus", "4"])
    bench.main()
    assert capsys.readouterr().out == ""
