"""bench.py's multi-rank host path on CPU: world-size-2 gloo ranks agree on the max-over-ranks
time and the sum of photons, and the reference arm runs on rank 0 only (the others exit 0)."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(REPO))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(world)
    t = bench.max_over_ranks(1.0 + rank, world)
    n = bench.sum_over_ranks(10 * (rank + 1), world)
    out.put((rank, t, n))
    dist.destroy_process_group()


def test_max_and_sum_over_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2.0, 30.0), (1, 2.0, 30.0)]


def test_reference_arm_under_torchrun_prints_one_line():
    pytest.importorskip("torch")
    env = dict(os.environ, SPPM_REFERENCE_SECONDS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(free_port()), str(REPO / "bench.py"), "--impl", "reference", "--gpus",
           "2", "--steps", "1", "--warmup", "3"]
    p = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=REPO)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"


def test_reference_arm_does_not_load_the_product_library():
    """The CPU reference arm renders the reference host code's scene (a committed fixture) with the
    oracle alone: the product package is never imported and libsppm.so never mapped, and its config
    is the GPU arm's headline config."""
    env = dict(os.environ, SPPM_REFERENCE_SECONDS="1")
    code = (f"import sys; sys.path.insert(0, {str(REPO)!r}); "
            "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3']; "
            "import bench; bench.main(); "
            "maps = open('/proc/self/maps').read(); "
            "print('PRODUCT' if ('libsppm' in maps or any(m.startswith('glslppm_gb300') for m in sys.modules)) "
            "else 'CLEAN')")
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, env=env, cwd=REPO)
    assert p.returncode == 0, p.stderr[-2000:]
    out = p.stdout.strip().splitlines()
    assert out[-1] == "CLEAN"
    d = json.loads(next(ln for ln in out if ln.startswith("{")))
    sys.path.insert(0, str(REPO))
    import bench
    assert d["config"] == bench.headline_config("fp32", 10, 1)
