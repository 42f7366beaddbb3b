"""The N > 1 benchmark path on CPU: independent replicas, max-over-ranks timing over gloo."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    import bench
    w, r, local, pg = bench.dist_setup()
    bench.barrier(pg)
    m = bench.allmax(pg, 10.0 + rank)
    q.put((r, w, local, m))
    pg.destroy_process_group()


def test_two_rank_replica_timing_takes_the_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert [r[0] for r in res] == [0, 1]
    assert all(r[1] == 2 for r in res)
    assert all(r[3] == 11.0 for r in res)


def test_reference_arm_json_line():
    """`bench.py --impl reference` (the oracle port on the host cores) prints one JSON line
    with the contract's keys, the same metric and unit as the GPU arm, zero transfer bytes
    and a cpu_baseline describing the run."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--config", "0",
                        "--steps", "1", "--warmup", "1", "--start-step", "4"], capture_output=True, text=True, timeout=600, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "e2e", "cpu_baseline"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["warmup"] >= 3
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    import bench
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    # the same workload description as the GPU arm's line
    from types import SimpleNamespace
    args = SimpleNamespace(config=0, config_name=d["config"]["workload"], start_step=4, warmup=3, steps=1, gpus=1)
    assert d["config"] == bench.config_dict(args, bench.make_scene(args))
    assert "steps 7-7" in d["cpu_baseline"]["sample"] and d["cpu_baseline"]["cpu_model"]
