"""The N>1 path of bench.py on CPU: replicas launched as separate ranks
(torchrun's environment), here over gloo.  Each rank renders its own frames
(no data-path collective); the job's result is the slowest rank's time and
the rays of all ranks.  The reference arm runs on rank 0 only."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]

WORKER = r"""
import json, os, sys
sys.path.insert(0, sys.argv[1])
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
world, rank, local = bench.setup_dist()
ms, rays = bench.reduce_over_ranks(10.0 + rank, 100 * (rank + 1), world, "cpu")
print(json.dumps({"world": world, "rank": rank, "local": local, "ms": ms, "rays": rays}))
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _env(rank, world, port):
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
               LOCAL_RANK=str(rank))
    env.pop("CUDA_VISIBLE_DEVICES", None)
    return env


def test_two_gloo_ranks_take_the_slowest_time_and_all_rays():
    port = _free_port()
    procs = [subprocess.Popen([sys.executable, "-c", WORKER, str(ROOT)], env=_env(r, 2, port), stdout=subprocess.PIPE,
                              stderr=subprocess.PIPE, text=True) for r in range(2)]
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    for rank, o in enumerate(outs):
        assert (o["world"], o["rank"], o["local"]) == (2, rank, rank)
        assert o["ms"] == 11.0 and o["rays"] == 300.0


def test_single_rank_reduction_is_the_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.reduce_over_ranks(7.5, 42, 1, "cpu") == (7.5, 42.0)


def test_reference_arm_runs_on_rank_zero_only():
    port = _free_port()
    res = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2"],
                         env=_env(1, 2, port), capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stderr
    assert res.stdout.strip() == ""


REF_CHILD = r"""
import json, sys, types
sys.path.insert(0, sys.argv[1])
import bench
args = types.SimpleNamespace(steps=1, warmup=0, gpus=1)
out = bench.run_reference(args)
maps = open("/proc/self/maps").read()
print(json.dumps({"line": out, "libwfpt": "libwfpt.so" in maps, "liboracle": "liboracle.so" in maps,
                  "torch": "torch" in sys.modules and "libtorch" in maps}))
"""


def test_reference_arm_maps_no_product_library():
    """The reference arm generates the scene, builds its BVH2 and renders
    with the oracle alone: libwfpt.so is never loaded into its process, and
    its config is the repo arm's workload config."""
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT"):
        env.pop(k, None)
    res = subprocess.run([sys.executable, "-c", REF_CHILD, str(ROOT)], env=env, capture_output=True, text=True,
                         timeout=600)
    assert res.returncode == 0, res.stderr
    o = json.loads(res.stdout.strip().splitlines()[-1])
    assert o["liboracle"] and not o["libwfpt"]
    line = o["line"]
    sys.path.insert(0, str(ROOT))
    import bench
    assert line["config"] == bench.workload_config(268304, 1)
    assert line["impl"] == "reference" and line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
