"""bench.py at N > 1 ranks: one independent realisation per rank (no
collective on the data path), a host barrier around the timed region and the
maximum step time over ranks. Two gloo ranks on the CPU; each evaluates the
forces of part of its own realisation with the oracle (the CPU stand-in for
the GPU kernel), and the parent checks them against the same realisation
built and evaluated on its own."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    sys.argv = ["bench.py", "--workload", "cfg1", "--n", "2048", "--gpus", str(ws)]
    import bench

    args = bench.parse()
    w, r, _ = bench.dist_env()
    dist = bench.dist_init(w)
    ps, _, _, _, _ = bench.workload(args, r)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    port = pyoracle.Port(threads=1)
    bench.barrier(dist)
    F = port.forces(port.system(0, ps.m, ps.eps, pyoracle.make_params()), ps.x, 0, 63)
    t = bench.allmax(dist, 1.0 + 2.0 * r)  # this rank's step time
    q.put((r, w, t, ps.x[:8].copy(), F))
    dist.destroy_process_group()


def test_two_replicas_gloo():
    mp = pytest.importorskip("torch.multiprocessing")
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, t0, x0, F0), (r1, w1, t1, x1, F1) = out
    assert (r0, r1, w0, w1) == (0, 1, 2, 2)
    assert t0 == t1 == 3.0  # every rank reports the slowest rank's time
    assert not np.allclose(x0, x1)  # independent realisations (seed 1 + rank)
    # each rank's forces are those of its own realisation, built here again
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import bench
    import pyoracle

    sys.argv = ["bench.py", "--workload", "cfg1", "--n", "2048", "--gpus", "2"]
    args = bench.parse()
    port = pyoracle.Port(threads=1)
    for r, F in ((0, F0), (1, F1)):
        ps, _, _, _, _ = bench.workload(args, r)
        ref = port.forces(port.system(0, ps.m, ps.eps, pyoracle.make_params()), ps.x, 0, 63)
        np.testing.assert_array_equal(F, ref)
    assert not np.allclose(F0, F1)
