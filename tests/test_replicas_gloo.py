"""Multi-GPU host logic on CPU: world size 2 over gloo.  The path runs as independent replicas
(no data-path collective); the job value is the sum of all ranks' particle-steps over the
slowest rank's time, and identical replicas produce identical (deterministic) oracle states."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import sys

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist

    import bench
    import __graft_entry__ as g

    dist.init_process_group("gloo", rank=rank, world_size=world)
    pkg = g.load_package()
    orc = g.load_oracle()
    tank, eos = pkg.dam_break(2, 0.05, (1.0, 0.5), (2.0, 1.0), n_layers=3)
    semi = pkg.dam_break_semidiscretization(tank, eos, 1.75 * 0.05)
    model = orc.Model(semi.config, tank.boundary.coordinates, tank.boundary.mass, tank.fluid.mass)
    v = np.zeros((tank.fluid.n_particles, 3))
    v[:, 2] = tank.fluid.density
    v, u, st = model.integrate(v, tank.fluid.coordinates, 1e-4, 3)
    n = tank.fluid.n_particles + tank.boundary.n_particles
    value, ms = bench.replica_value(dist, 100.0 * (rank + 1), n, 3)
    digest = float(np.sum(u * np.arange(1, u.size + 1)))
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, value, ms, st, digest, n))


def test_replicas_world_size_2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=240) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    (_, v0, ms0, st0, d0, n), (_, v1, ms1, st1, d1, _) = res
    assert st0 == st1 == 0
    assert ms0 == ms1 == 200.0           # max over ranks
    assert v0 == v1 == pytest.approx(n * 3 * 2 / 0.2)
    assert d0 == d1                       # replicas are deterministic and independent
