"""The N>1 path of bench.py on the host: replicas joined by a gloo process
group (barrier, max over ranks), rank 0 alone reporting.  No GPU needed."""
import json
import os
import subprocess
import sys
import textwrap

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = textwrap.dedent("""
    import json, os, sys
    sys.path.insert(0, {root!r})
    import bench
    world, rank, local = bench.dist_setup()
    bench.barrier(world)
    t = bench.allmax(world, float(rank + 1) * 1.5)
    # replicas: every rank processed its own units; rank 0 reports the job
    units = bench.allmax(world, 100.0)
    if rank == 0:
        print(json.dumps({{"world": world, "max": t, "units": units}}), flush=True)
""")


def test_two_rank_gloo_replicas(tmp_path):
    script = tmp_path / "child.py"
    script.write_text(CHILD.format(root=ROOT))
    env = dict(os.environ, MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
                        "--master-addr", "127.0.0.1", "--master-port", "29531", str(script)],
                       capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1  # rank 0 alone prints
    out = json.loads(lines[0])
    assert out["world"] == 2 and out["max"] == 3.0


def test_reference_arm_json_line():
    """bench.py --impl reference on the host (the reference arm the driver
    runs): one JSON line with the contract's keys, the port's core count and
    an e2e block with no copies."""
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1", "--cpu-sample", "2", "--sentences", "40"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT,
                       env=dict(os.environ, MASTER_ADDR="127.0.0.1"))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    out = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "config", "cpu_baseline", "e2e"):
        assert k in out, k
    assert out["impl"] == "reference" and out["value"] > 0 and out["steps"] == 1
    assert out["cpu_baseline"]["kind"] == "port" and out["cpu_baseline"]["cores"] >= 1
    assert out["e2e"]["h2d_bytes_per_step"] == 0 and out["e2e"]["value"] == out["value"]
