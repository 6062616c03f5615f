"""Replica timing of bench.py on CPU: two gloo ranks, each reporting its own
time; every rank must see the maximum (the job ends with its slowest replica)."""
import os
import socket

import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys
    import torch
    import torch.distributed as dist
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks(torch, dist, 10.0 + 5.0 * rank, device="cpu")
        q.put((rank, got))
    finally:
        dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert res == [(0, 15.0), (1, 15.0)]


def test_single_rank_is_identity():
    import torch
    import bench
    assert bench.max_over_ranks(torch, None, 3.5) == 3.5


def _replica_rank(rank, world, port, q):
    """One replica rank of bench.py's timing path on the CPU: a tiny lid
    cavity (the oracle as the solve), barrier, timed steps, max over ranks."""
    import sys
    import torch
    import torch.distributed as dist
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    from oracle import oracle as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        n = 8 + 4 * rank  # ranks of unequal speed: the slower one sets the time
        o = O.LidOracle(n, n, n, 100.0, 0.1)
        ms = bench.timed_replica(torch, dist, lambda k: o.run(k), 4, 3, bench.HostClock(),
                                 device="cpu")
        q.put((rank, ms, bench.replica_mlups(world, 12 ** 3, 4, ms)))
    finally:
        dist.destroy_process_group()


def test_replica_timing_path_two_gloo_ranks():
    from oracle import oracle as O
    O.build()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_replica_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(300)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    (r0, ms0, v0), (r1, ms1, v1) = res
    assert (r0, r1) == (0, 1) and ms0 == ms1 > 0 and v0 == v1
    assert abs(v0 - 2 * 12 ** 3 * 4 / (ms0 * 1e-3) / 1e6) < 1e-9 * v0


def test_replica_command_and_world_check(monkeypatch):
    import bench
    cmd = bench.replica_command(4, ["--steps", "3", "--gpus", "4"], 29511)
    assert cmd[1:3] == ["-m", "torch.distributed.run"]
    assert "--nproc-per-node=4" in cmd and "127.0.0.1" in cmd and "29511" in cmd
    assert cmd[-5].endswith("bench.py") and cmd[-4:] == ["--steps", "3", "--gpus", "4"]
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    assert bench.world_check(1) == (False, None)
    assert bench.world_check(4) == (True, None)
    monkeypatch.setenv("WORLD_SIZE", "4")
    assert bench.world_check(4) == (False, None)
    monkeypatch.setenv("WORLD_SIZE", "2")
    spawn, err = bench.world_check(4)
    assert not spawn and "WORLD_SIZE=2" in err


def test_world_size_mismatch_fails_loudly():
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--gpus", "4", "--impl",
                        "reference", "--workload", "lid64"], cwd=root,
                       env=dict(os.environ, WORLD_SIZE="2", RANK="0"), capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 2 and "WORLD_SIZE=2 but --gpus 4" in r.stderr
