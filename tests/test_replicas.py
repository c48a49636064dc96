"""The N > 1 form of bench.py: N independent replicas whose only
communication is a barrier and a max over ranks of the time (gloo on the
host). Checked here on CPU with two ranks; no GPU, no data-path collective."""
import os
import subprocess
import sys
import textwrap

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_two_replicas_max_and_barrier():
    script = textwrap.dedent("""
        import os, sys, json
        sys.path.insert(0, %r)
        import bench
        rep = bench.Replicas()
        rep.barrier()
        mine = 10.0 * (rep.rank + 1)
        m = rep.max(mine)
        rep.barrier()
        print(json.dumps({"rank": rep.rank, "world": rep.world, "max": m}))
        rep.close()
    """ % ROOT)
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT="29533", WORLD_SIZE="2")
    procs = []
    for r in range(2):
        e = dict(env, RANK=str(r), LOCAL_RANK=str(r))
        procs.append(subprocess.Popen([sys.executable, "-c", script], env=e, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, err = p.communicate(timeout=300)
        assert p.returncode == 0, err
        outs.append(o.strip().splitlines()[-1])
    import json
    got = sorted((json.loads(o) for o in outs), key=lambda d: d["rank"])
    assert [g["world"] for g in got] == [2, 2]
    assert [g["max"] for g in got] == [20.0, 20.0]


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK") if k in os.environ}
    try:
        rep = bench.Replicas()
        assert rep.world == 1 and rep.dist is None
        assert rep.max(3.5) == 3.5
        rep.barrier()
    finally:
        os.environ.update(env)
