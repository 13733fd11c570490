"""bench.py host logic on the CPU: the reference arm's JSON line, and the
two-rank (gloo) launch in which rank 0 alone prints."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--order", "200", "--steps", "1",
                        "--warmup", "0", "--cpu-sample", "64"], cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "eigenvectors/s" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0


def test_reference_arm_two_ranks_gloo():
    env = dict(os.environ, MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", "29631", "bench.py", "--impl",
                        "reference", "--gpus", "2", "--order", "120", "--steps", "1", "--warmup", "0",
                        "--cpu-sample", "32"], cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    assert json.loads(lines[0])["n_gpus"] == 2


def test_max_over_ranks_gloo(tmp_path):
    """The replica time reduction used by the GPU arm (max over ranks)."""
    code = r'''
import os, torch, torch.distributed as dist
dist.init_process_group("gloo")
r = dist.get_rank()
t = torch.tensor([1.0 + r])
dist.all_reduce(t, op=dist.ReduceOp.MAX)
assert t.item() == 2.0
if r == 0: print("ok")
'''
    script = tmp_path / "ranks.py"
    script.write_text(code)
    env = dict(os.environ, MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", "29632", str(script)],
                       cwd=ROOT, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr[-2000:]
