"""The benchmark's multi-process plumbing on the CPU: two gloo ranks.

``bench.py`` runs one process per GPU; the ranks share nothing on the data
path (independent lattices / requests) and meet only in a barrier and a max
over ranks.  Here that plumbing runs as two gloo ranks, and the reference arm
runs under the real launcher with world size 2 (rank 0 alone prints).
"""
import json
import multiprocessing
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, out):
    os.environ.update({"WORLD_SIZE": "2", "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "XK_BENCH_BACKEND": "gloo"})
    sys.path.insert(0, ROOT)
    import bench
    from xentica_gb300.batch import ensemble_workload
    dist = bench.Dist()
    try:
        dist.barrier()
        top = dist.max(1.5 + rank)
        # each rank seeds its own lattices, as run_ours does
        widths, heights, rules, _, cells = ensemble_workload(3, 2041 + 7919 * rank)
        out.put((rank, dist.world, top, int(cells.sum()), list(rules)))
    finally:
        dist.close()


def test_barrier_and_max_over_two_gloo_ranks():
    ctx = multiprocessing.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2, 2]
    assert [r[2] for r in res] == [2.5, 2.5]          # the max reaches every rank
    assert res[0][3:] != res[1][3:]                    # ranks hold different lattices


def test_reference_arm_under_the_launcher():
    env = dict(os.environ, XK_BENCH_BACKEND="gloo")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "0", "--cpu-seconds", "1", "--instances", "4"]
    proc = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert proc.returncode == 0, proc.stderr[-2000:]
    lines = [l for l in proc.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1                             # rank 0 alone prints
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0
