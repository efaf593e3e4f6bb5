"""CPU tests of the bench's N>1 path.  The step does not shard (no exchange
between GPUs), so ``bench.py --gpus N`` runs N replicas, one rank each; what
crosses ranks is host logic over gloo: the barriers around the timed region,
the max of the ranks' times, and the reference arm's rule that rank 0 alone
runs and prints while the other ranks exit 0 without work.  Run here as two
processes on 127.0.0.1, world size 2."""
import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, q):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": "2",
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    d.barrier()
    # the timed region's figure: each rank's time, the job's is the slowest
    got = d.allmax(10.0 + 5.0 * rank)
    d.barrier()
    d.close()
    q.put((rank, d.world, got))


def test_dist_two_ranks_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert res == [(0, 2, 15.0), (1, 2, 15.0)]


def test_reference_arm_under_torchrun_prints_once_from_rank_zero():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "2", "--warmup", "1",
           "--nx", "64", "--ny", "32", "--nz", "32"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["unit"] == "Mcell-steps/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 2
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
