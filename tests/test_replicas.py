"""The replica path of `bench.py --gpus N` on CPU: two ranks over gloo.

Calls are independent, so N GPUs run N replicas with no collective on the
data path; the ranks only meet in a barrier around the timed region and in
the maximum over ranks of its time.  Checked here without a GPU:
  * two ranks set up through the environment torchrun provides, pass the
    barrier and agree on the maximum of their times;
  * the reference arm launched by torchrun with two processes: rank 0 alone
    runs the CPU BLAS and prints one line (whole-job fields for two
    replicas), the other rank exits 0 without work.
"""
import json
import os
import socket
import subprocess
import sys
import textwrap

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


RANK_SCRIPT = textwrap.dedent("""
    import argparse, json, sys
    sys.path.insert(0, {root!r})
    import bench
    ws, rank, local = bench.dist_setup(argparse.Namespace(impl="reference"))
    bench.barrier(ws)
    t = bench.max_over_ranks(ws, 1.5 + rank)
    bench.barrier(ws)
    print(json.dumps({{"rank": rank, "local": local, "ws": ws, "max": t}}), flush=True)
""")


def test_two_gloo_ranks_meet_in_barrier_and_max():
    port = free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT.format(root=ROOT)], env=env, cwd=ROOT,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        try:
            outs.append(p.communicate(timeout=180))
        except subprocess.TimeoutExpired:
            for q in procs:
                q.kill()
            raise
    for p, (_, err) in zip(procs, outs):
        assert p.returncode == 0, err[-2000:]
    res = sorted((json.loads(out.strip().splitlines()[-1]) for out, _ in outs), key=lambda d: d["rank"])
    assert [d["rank"] for d in res] == [0, 1] and [d["local"] for d in res] == [0, 1]
    assert all(d["ws"] == 2 and d["max"] == 2.5 for d in res)


def test_reference_arm_under_torchrun_prints_one_line():
    port = free_port()
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
                        "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1"],
                       capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["steps"] == 1
    assert d["config"]["parallelism"] == "replicas"
    assert d["value"] > 0 and d["e2e"]["value"] == d["value"] and d["cpu_baseline"]["kind"] == "reference"
