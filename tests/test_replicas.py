"""Replica timing of bench.py on CPU: two gloo ranks (world size 2) run the
same setup, barrier and max-over-ranks reduction the GPU run uses, and the
reference arm does no work on ranks other than 0."""
import os
import socket

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), CRT_BENCH_BACKEND="gloo")
    import bench
    dist, r, w = bench.dist_setup()
    assert (r, w) == (rank, ws)
    bench.barrier(dist)
    t = bench.max_over_ranks(dist, 1.0 + rank, "cpu")  # each rank's own elapsed time
    q.put((rank, t))
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_max():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    res = dict(q.get(timeout=5) for _ in range(2))
    assert res == {0: 2.0, 1: 2.0}


def test_single_process_needs_no_process_group(monkeypatch):
    import bench
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    dist, r, w = bench.dist_setup()
    assert dist is None and (r, w) == (0, 1)
    assert bench.max_over_ranks(None, 3.5) == 3.5


def test_reference_arm_idle_on_other_ranks():
    import argparse

    import bench
    args = argparse.Namespace(steps=2, warmup=1)
    assert bench.run_reference(args, None, 1, 2) is None


def test_clock_summary_keeps_the_timed_region():
    """bench.Clocks keeps the nvidia-smi samples read inside the timed region
    (plus one interval after it) and reports throttle reasons from them."""
    import bench
    c = bench.Clocks(0)
    row = lambda t, mhz, cap: [t, str(mhz), "2070", "900", "Not Active", "Not Active", "Not Active", cap]  # noqa: E731
    c.samples = [row(0.9, 1500, "Not Active"), row(1.05, 2070, "Not Active"), row(1.2, 2070, "Active"),
                 row(2.5, 1200, "Not Active")]
    c.t0, c.t1 = 1.0, 1.18
    s = c.summary()
    assert s["samples"] == 2 and s["sm_mhz"] == 2070.0 and s["reasons"] == ["sw_power_cap"]
    assert c.summary() == s  # no side effects
    c.t0, c.t1 = 3.0, 3.1  # nothing inside: the last samples stand in
    assert c.summary()["samples"] == 2
