"""The multi-rank path of bench.py on CPU: world_size 2 over gloo (127.0.0.1).

With N GPUs every rank runs an independent replica; the whole-job rate is the units all ranks
processed over the slowest rank's time. The reference arm runs on rank 0 alone and prints one line;
the other ranks exit 0 without work.
"""
import json
import os
import socket
import subprocess
import sys
import textwrap

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _launch(argv, world=2, timeout=300):
    port = _free_port()
    procs = []
    for rank in range(world):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), MG_BENCH_BACKEND="gloo")
        procs.append(subprocess.Popen(argv, cwd=ROOT, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                                      text=True))
    out = []
    for p in procs:
        o, e = p.communicate(timeout=timeout)
        out.append((p.returncode, o, e))
    return out


def test_whole_job_rate_takes_the_slowest_rank():
    script = textwrap.dedent("""
        import json, os, sys
        sys.path.insert(0, os.getcwd())
        import bench
        rank, world, dist = bench.dist_init(2)
        rate, sec = bench.whole_job_rate(dist, None, 1000, 1.0 + rank)
        bench.barrier(dist)
        print(json.dumps({"rank": rank, "world": world, "rate": rate, "sec": sec}))
        dist.destroy_process_group()
    """)
    res = _launch([sys.executable, "-c", script])
    for rc, o, e in res:
        assert rc == 0, e
    lines = [json.loads(o.strip().splitlines()[-1]) for _, o, _ in res]
    assert sorted(x["rank"] for x in lines) == [0, 1]
    for x in lines:
        assert x["world"] == 2
        assert x["sec"] == 2.0                 # the slower rank's time, on every rank
        assert x["rate"] == 2 * 1000 / 2.0     # units of both ranks over that time


def test_reference_arm_prints_one_line_from_rank_zero():
    res = _launch([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
                   "--cpu-seconds", "1"])
    (rc0, o0, e0), (rc1, o1, e1) = res
    assert rc0 == 0, e0
    assert rc1 == 0, e1
    assert o1.strip() == ""
    line = json.loads(o0.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["unit"] == "atom-steps/s"
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
