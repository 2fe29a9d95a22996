"""bench.py at world size 2 on the CPU (gloo): the barrier and the max over
ranks that the multi-replica timing uses, and the reference arm's rule that
only rank 0 works and prints."""
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run_ranks(code, ws=2, timeout=180):
    port = _free_port()
    procs = []
    for r in range(ws):
        env = dict(os.environ, WORLD_SIZE=str(ws), RANK=str(r), LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", code], cwd=ROOT, env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    try:
        for p in procs:
            out, err = p.communicate(timeout=timeout)
            outs.append((p.returncode, out, err))
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
    return outs


def test_barrier_and_max_over_ranks_gloo():
    code = (
        "import sys; sys.path.insert(0, '.')\n"
        "import bench\n"
        "ws, rank, local = bench.dist_init()\n"
        "bench.barrier(ws)\n"
        "v = bench.max_over_ranks(0.25 + rank, ws)\n"
        "print('RANK', rank, ws, local, v)\n"
    )
    outs = _run_ranks(code)
    for r, (rc, out, err) in enumerate(outs):
        assert rc == 0, err
        assert f"RANK {r} 2 {r} 1.25" in out, out


def test_reference_arm_other_ranks_exit_quietly():
    # rank 1 of a two-rank reference run returns before any work and prints nothing
    code = (
        "import sys; sys.path.insert(0, '.')\n"
        "import bench\n"
        "class A: pass\n"
        "a = A(); a.steps = 1; a.warmup = 0; a.ref_sweeps = 1; a.workload = 'zipf4'\n"
        "import os\n"
        "if os.environ['RANK'] == '1':\n"
        "    bench.run_reference(a, bench.WORKLOADS['zipf4'])\n"
        "    print('DONE')\n"
        "else:\n"
        "    bench.dist_init(); print('DONE')\n"
    )
    outs = _run_ranks(code)
    for rc, out, err in outs:
        assert rc == 0, err
        assert out.strip().splitlines()[-1] == "DONE", out
    assert "{" not in outs[1][1]  # no JSON line from rank 1
