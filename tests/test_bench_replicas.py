"""The N > 1 path of bench.py on CPU: two gloo ranks, replicas only (each rank runs its
own copy of the workload), the job's time is the slowest rank's and the value is the
work of all replicas over that time; the reference arm runs on rank 0 alone."""
import os
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    assert bench.dist_env() == (rank, world, rank)
    # per-rank timed totals (ms over 4 steps): rank 1 is the slow replica
    local = [40.0 + 20.0 * rank, 50.0 + 10.0 * rank]
    t_ms, t_e2e = bench.max_over_ranks(local, dist, "cpu")
    value = bench.job_throughput(world, 1000, t_ms, 4)
    q.put((rank, t_ms, t_e2e, value))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_replica():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(2))
    for rank, t_ms, t_e2e, value in got:
        assert (t_ms, t_e2e) == (60.0, 60.0)
        # 2 replicas x 1000 units per step, 15 ms per step
        assert value == pytest.approx(2 * 1000 / 15e-3)


def test_reference_arm_non_zero_rank_exits_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_single_process_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks([1.0, 2.0], None, "cpu") == [1.0, 2.0]
    assert bench.job_throughput(1, 500, 100.0, 10) == pytest.approx(500 / 10e-3)


def test_method_and_bodies_options(monkeypatch):
    """--bodies and --method select one Barnes-Hut configuration of a given size (no
    calibration ladder); the ladder's rows carry theta, flags, alpha and ratio."""
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setattr(sys, "argv", ["bench.py", "--bodies", "4096", "--method", "1.0,27,0.00275,0.13"])
    args = bench.parse_args()
    wl = bench.make_workload(args)
    assert wl.n == 4096 and wl.bodies.shape == (4096, 4)
    assert wl.fixed == (1.0, 27, 0.00275, 0.13)
    assert wl.config()["workload"] == "bh_bulge_disk_4096"
    monkeypatch.setattr(sys, "argv", ["bench.py", "--bodies", "2048", "--method", "0.5,0"])
    wl = bench.make_workload(bench.parse_args())
    assert wl.fixed == (0.5, 0, None, 0.1)
    for entry in bench.BarnesHutWorkload.ladder:
        theta, flags, alpha, ratio = entry[:4]
        assert len(entry) == 4 or (len(entry) == 5 and 0.0 <= entry[4] <= 1.0 and (flags & 17) == 17)
        assert (alpha is not None) == bool(flags & 16) and 0 < ratio <= 0.5
        # with the error-bound opening theta is only the geometric cap
        assert 0 < theta <= (2.0 if flags & 16 else 1.0)



def test_reference_arm_small_case():
    """`--impl reference` on a small Barnes-Hut case, on CPU: the restated
    parallel::BarnesHut walks every target once over the K steps and prints the
    contract's line (value, e2e with no copies, cpu_baseline describing the run)."""
    import json
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--bodies", "4096",
                        "--steps", "2", "--warmup", "1"], capture_output=True, text=True, timeout=600,
                       env=dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0"))
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([x for x in r.stdout.splitlines() if x.startswith("{")][-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "bodies/s"
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["config"]["n_bodies"] == 4096
