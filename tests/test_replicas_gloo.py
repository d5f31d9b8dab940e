"""The N>1 path of bench.py on CPU: replicas over gloo (world size 2, 127.0.0.1).

The step does not shard, so N ranks run N independent replicas; the only collectives are a
barrier and the max/sum of the ranks' times and units (bench.Dist).  The reference arm runs
on rank 0 only; the others exit 0 without work."""
import json
import os
import pathlib
import socket
import subprocess
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _torchrun(args, timeout=300):
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port())] + args
    env = dict(os.environ, OMP_NUM_THREADS="2")
    return subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=timeout)


def test_dist_collectives_world2(tmp_path):
    code = tmp_path / "w.py"
    code.write_text(
        "import sys, json; sys.path.insert(0, %r)\n"
        "import bench\n"
        "d = bench.Dist()\n"
        "d.barrier()\n"
        "mx = d.max(float(d.rank + 1)); sm = d.sum(10.0)\n"
        "out = {'rank': d.rank, 'world': d.world, 'max': mx, 'sum': sm}\n"
        "open(%r + '/rank%%d.json' %% d.rank, 'w').write(json.dumps(out))\n"
        "d.close()\n" % (str(ROOT), str(tmp_path)))
    r = _torchrun([str(code)])
    assert r.returncode == 0, r.stderr[-2000:]
    # one file per rank: the ranks' stdout lines can interleave
    outs = [json.loads((tmp_path / f"rank{k}.json").read_text()) for k in range(2)]
    assert sorted(o["rank"] for o in outs) == [0, 1]
    for o in outs:
        assert o["world"] == 2 and o["max"] == 2.0 and o["sum"] == 20.0


def test_reference_arm_under_torchrun_prints_once():
    r = _torchrun(["bench.py", "--impl", "reference", "--case", "poiseuille_40", "--steps", "1", "--warmup", "3",
                   "--cpu-iters", "5", "--ref-iters", "70"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["n_gpus"] == 2
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
