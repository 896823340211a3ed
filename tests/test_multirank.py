"""The N > 1 path of bench.py on the CPU: replicas only (no data-path
collective), so what runs across ranks is the max-over-ranks timing reduction
and the rank-0-only reference arm.  gloo, world size 2."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        q.put((rank, bench.max_over_ranks([1.0 + rank, 10.0 - rank], "cpu")))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: [2.0, 10.0], 1: [2.0, 10.0]}


def test_reference_arm_under_torchrun(native):
    """Rank 0 alone times the CPU implementation and prints one line; the other
    rank exits 0 without work."""
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
           "--workload", "fbm_256", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["config"]["workload"] == "fbm_256" and line["config"]["nwanted"] == 256
    assert line["e2e"]["h2d_bytes_per_step"] == 0


def test_reference_arm_never_loads_the_library():
    """The reference arm builds its inputs with the oracle's generator and
    times the reference's own code: the library (siting_gb300 and its .so)
    stays unloaded in that process."""
    code = (
        "import runpy, sys\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--workload', 'fbm_256',"
        " '--steps', '1', '--warmup', '0']\n"
        "runpy.run_path('bench.py', run_name='__main__')\n"
        "maps = open('/proc/self/maps').read()\n"
        "bad = [m for m in sys.modules if m.startswith('siting_gb300')]\n"
        "print('LIBRARY', bool(bad) or 'libsiting_gb300' in maps)\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(next(x for x in r.stdout.splitlines() if x.startswith("{")))
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] in ("reference_omp", "port")
    assert "LIBRARY False" in r.stdout
