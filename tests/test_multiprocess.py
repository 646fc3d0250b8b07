"""Multi-rank paths of bench.py on CPU: two gloo ranks on 127.0.0.1.

With N GPUs the bench runs one replica per rank (weak scaling) and takes
the maximum time over the ranks; the reference arm runs on rank 0 alone.
Both paths are exercised here without a GPU."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _allmax_rank(rank, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    ws, r, _, pg = bench._dist()
    out.put((r, ws, bench._allmax(pg, 1.0 + r)))
    pg.destroy_process_group()


def test_time_is_the_maximum_over_two_gloo_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_allmax_rank, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
    assert res == [(0, 2, 2.0), (1, 2, 2.0)]


def test_reference_arm_runs_on_rank_zero_only():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--workload", "vortex2d", "--steps", "1", "--warmup", "0", "--gpus", "2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["cpu_baseline"]["cores"] >= 1


def test_reference_arm_maps_no_device_library():
    """The CPU arm sets its cases up with the oracle's own code: a process that
    builds a case and runs the oracle on it never loads liblfm_gpu.so."""
    code = ("import sys; sys.path.insert(0, %r)\n"
            "import bench\n"
            "import oracle.port as P\n"
            "c = bench.workload('vortex2d')\n"
            "pc = P.PortCase.from_case(c)\n"
            "P.run(pc, pc.q0(), 1, c.delta_t)\n"
            "maps = open('/proc/self/maps').read()\n"
            "print('port' if 'liblfm_port.so' in maps else 'no-port', 'gpu' if 'liblfm_gpu.so' in maps else 'no-gpu')\n"
            % ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    assert r.stdout.split() == ["port", "no-gpu"]
