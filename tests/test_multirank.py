"""The multi-GPU path of bench.py is independent replicas (the solve does not shard): ranks
only meet at the barrier around the timed region and at the max-over-ranks of the elapsed
time. These run as two gloo ranks on the CPU."""
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import os, sys, json, time
sys.path.insert(0, {root!r})
import bench
world, rank, local = bench.dist_setup()
assert world == 2 and local == rank
assert os.environ["CUDA_VISIBLE_DEVICES"] == str(local)   # one GPU per rank
bench.barrier(world)
t = bench.reduce_max(world, 10.0 * (rank + 1))            # the slowest rank's time is the job's
time.sleep(0.05 * rank)
bench.barrier(world)
print(json.dumps({{"rank": rank, "max": t}}))
"""


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_gloo_ranks_barrier_and_max():
    port = free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD.format(root=ROOT)], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e[-2000:]
    import json
    res = sorted(json.loads(o.strip().splitlines()[-1])["max"] for o, _ in outs)
    assert res == [20.0, 20.0]


def test_reference_arm_multi_mesh_workloads_report_unavailable():
    """batch/serve have no reference CPU arm (one mesh per process in the reference): the
    arm prints its unavailable line and exits 0, on every rank count."""
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "batch"],
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    import json
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and "unavailable" in line
