"""Replica sharding and the end-of-run reduction, with world_size 2 on CPU
(gloo).  Each rank propagates its shard of a seeded workload with the CPU
oracle; the reduced counts must equal a single-process run of all molecules."""
import os
import socket

import numpy as np
import pytest

from ctraj.replicas import shard


def test_shard_partitions_exactly():
    for n in (0, 1, 7, 1000, 10_000_001):
        for world in (1, 2, 3, 8):
            parts = [shard(n, r, world) for r in range(world)]
            assert sum(p[1] for p in parts) == n
            off = 0
            for o, k in parts:
                assert o == off
                off += k
    with pytest.raises(ValueError):
        shard(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parent.parent
    sys.path[:0] = [str(root / "centrex-molecule-trajectories_gb300"), str(root)]
    import torch.distributed as dist

    from ctraj.compiler import compile_beamline
    from ctraj.distributions import host_draw
    from ctraj.replicas import reduce_run, shard
    from ctraj.workloads import lens_beamline, source
    from oracle import oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        cb = compile_beamline(lens_beamline())
        ics = host_draw(*source(), 20_000, seed=4)
        off, n = shard(ics.shape[1], rank, world)
        r = oracle.run(cb, np.ascontiguousarray(ics[:, off:off + n]), outputs=False)
        counts, steps, secs = reduce_run(r["counts"], r["steps"], 0.1 * (rank + 1))
        q.put((rank, counts.tolist(), steps, secs))
    finally:
        dist.destroy_process_group()


def test_two_replicas_reduce_to_the_single_run():
    import multiprocessing as mp

    from ctraj.compiler import compile_beamline
    from ctraj.distributions import host_draw
    from ctraj.workloads import lens_beamline, source
    from oracle import oracle

    oracle.build()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    cb = compile_beamline(lens_beamline())
    full = oracle.run(cb, host_draw(*source(), 20_000, seed=4), outputs=False)
    for rank, counts, steps, secs in res:
        assert counts == full["counts"].tolist()
        assert steps == full["steps"]
        assert secs == pytest.approx(0.2)


def _engine_worker(rank, world, port, n_total, seed, q):
    """A replica: its own engine (libctraj.so) on the GPU, its shard of the
    Philox counters, the end-of-run reduction over gloo."""
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parent.parent
    sys.path[:0] = [str(root / "centrex-molecule-trajectories_gb300"), str(root)]
    import torch.distributed as dist

    from ctraj.compiler import compile_beamline
    from ctraj.distributions import device_spec
    from ctraj.engine import Engine
    from ctraj.replicas import reduce_run, shard
    from ctraj.workloads import lens_beamline, source

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        xd, vd = source()
        cb = compile_beamline(lens_beamline())
        off, n = shard(n_total, rank, world)
        eng = Engine(0)
        r = eng.run(cb, n, xdist=device_spec(xd, "position"), vdist=device_spec(vd, "velocity"), seed=seed,
                    offset=off, timing=True)
        eng.close()
        counts, steps, secs = reduce_run(r.counts, r.molecule_steps, r.extra["front_ms"] + r.extra["lens_ms"])
        q.put((rank, counts.tolist(), steps, secs))
    finally:
        dist.destroy_process_group()


@pytest.mark.gpu
def test_two_engine_replicas_reduce_to_the_single_run():
    """Two processes, each with its own engine, propagate disjoint Philox
    ranges of one seeded run (the replica split bench.py uses under
    torchrun); their reduced counts and molecule-steps equal one run of all
    the molecules.  The replicas' kernels are independent (no collective on
    the data path), so sharing one GPU here changes nothing but speed."""
    import multiprocessing as mp

    n_total, seed = 3_000_001, 17
    ctx = mp.get_context("spawn")  # before this process touches the GPU
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_engine_worker, args=(r, 2, port, n_total, seed, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=600) for _ in procs]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0

    from ctraj.compiler import compile_beamline
    from ctraj.distributions import device_spec
    from ctraj.engine import Engine
    from ctraj.workloads import lens_beamline, source

    xd, vd = source()
    eng = Engine(0)
    try:
        full = eng.run(compile_beamline(lens_beamline()), n_total, xdist=device_spec(xd, "position"),
                       vdist=device_spec(vd, "velocity"), seed=seed)
    finally:
        eng.close()
    for rank, counts, steps, secs in res:
        assert counts == full.counts.tolist()
        assert steps == full.molecule_steps
        assert secs > 0
