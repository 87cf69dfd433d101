"""bench.py with N > 1 replicas, on the CPU: two ranks as torchrun starts
them (RANK / WORLD_SIZE / LOCAL_RANK / MASTER_*), gloo instead of NCCL.  The
path has no exchange step, so the only cross-rank work is the timed region's
barrier and the slowest rank's time, which sets the whole job's rate."""
import json
import os
import socket
import subprocess
import sys

from conftest import ROOT

RANK_SCRIPT = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
import bench
R = bench.Replicas()
R.barrier()
ms = 100.0 + 50.0 * R.rank          # rank 1 is the slow one
slowest = R.max(ms)
R.barrier()
steps = 20
print(json.dumps({"rank": R.rank, "world": R.world, "device": R.device, "slowest": slowest,
                  "value": R.world * steps / (slowest / 1e3)}))
R.close()
"""


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _env(rank: int, world: int, port: int) -> dict:
    env = dict(os.environ)
    env.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
               MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
    return env


def test_two_replicas_agree_on_the_slowest_rank():
    port = _free_port()
    procs = [subprocess.Popen([sys.executable, "-c", RANK_SCRIPT, str(ROOT)], env=_env(r, 2, port),
                              stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True) for r in range(2)]
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=180)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    assert sorted(o["rank"] for o in outs) == [0, 1]
    for o in outs:
        assert o["world"] == 2 and o["device"] == "cpu"
        assert o["slowest"] == 150.0                    # max over ranks, not the rank's own time
        assert abs(o["value"] - 2 * 20 / 0.150) < 1e-9  # both replicas' steps over the slowest time


def test_one_process_needs_no_process_group():
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        env.pop(k, None)
    r = subprocess.run([sys.executable, "-c", RANK_SCRIPT, str(ROOT)], env=env, capture_output=True, text=True,
                       timeout=180)
    assert r.returncode == 0, r.stderr
    o = json.loads(r.stdout.strip().splitlines()[-1])
    assert o == {"rank": 0, "world": 1, "device": "cpu", "slowest": 100.0, "value": 200.0}


def test_reference_arm_other_ranks_exit_without_work():
    """Under torchrun only rank 0 runs the reference's host kernels and
    prints; the other ranks return at once, exit 0 and print nothing."""
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "kuhn20_20k"],
                       env=_env(1, 2, _free_port()), capture_output=True, text=True, timeout=180)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
