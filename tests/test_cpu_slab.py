"""Slab decomposition along i2 of one evolution (nrpytutorial_gb300.slab) on
the CPU: the partition, the boundary-condition ownership and gather plan,
and world_size-2 and -3 gloo runs of the distributed RK4 step (halo
exchange, inner-parity gathers across ranks, all-reduced norms) with the
oracle's RHS, which must reproduce the one-grid oracle evolution bit for
bit."""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

import oracle.bcs as ob
import oracle.grid as og
import oracle.wave_maxwell as ow
from nrpytutorial_gb300.slab import SlabPlan, bcmap_layers, slab_ranges
from tests.slab_host import oracle_bcmap

CASES = {
    # phi wrap and theta/r reflections: inner sources on other ranks
    "scalarwave_sinhsph": ("ScalarWave", "SinhSpherical", (10, 6, 12), 4, dict(AMPL=5.0, SINHW=0.3)),
    # outer extrapolation along i2 on the edge ranks
    "maxwell_cartesian": ("Maxwell", "Cartesian", (6, 8, 12), 4, dict(domain=(-2.0, 2.0))),
    # inner maps in i1 (phi) and outer faces in i2 (z)
    "scalarwave_sinhcyl": ("ScalarWave", "SinhCylindrical", (8, 8, 12), 4, {}),
}
PARITY = {"ScalarWave": [0, 0], "Maxwell": [1, 2, 3, 1, 2, 3, 0]}


def _gp(case):
    system, coord, Nxx, order, kw = CASES[case]
    return og.GridParams(coord, Nxx, order // 2 + 1, order, **kw)


def _rhs_fn(case, gp):
    f = ow.scalarwave_rhs_grid if CASES[case][0] == "ScalarWave" else ow.maxwell_rhs_grid
    return lambda u: f(gp, u)


def _initial(case, gp):
    ngf = len(PARITY[CASES[case][0]])
    y = 0.1 * np.random.default_rng(7).standard_normal((ngf,) + gp.shape)
    ob.apply_bcs(ob.build_bcstruct(gp), y, PARITY[CASES[case][0]])
    return y


def test_slab_ranges_partition_the_interior_planes():
    assert slab_ranges(12, 3, 2) == [(3, 9), (9, 15)]
    assert slab_ranges(10, 2, 3) == [(2, 6), (6, 9), (9, 12)]
    r = slab_ranges(1000, 4, 8)
    assert r[0][0] == 4 and r[-1][1] == 1004
    assert all(a[1] == b[0] for a, b in zip(r, r[1:]))
    assert max(b - a for a, b in r) - min(b - a for a, b in r) <= 1
    with pytest.raises(ValueError):
        slab_ranges(8, 3, 3)  # 2 planes per rank < NGHOSTS
    with pytest.raises(ValueError):
        slab_ranges(5, 2, 2)  # < 3 planes: the outer rule reads 3 planes inward


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("world", [2, 3])
def test_every_ghost_point_has_one_owner_and_every_request_a_sender(case, world):
    gp = _gp(case)
    bcmap = oracle_bcmap(gp)
    n = tuple(gp.np)
    plans = [SlabPlan(n, gp.NGHOSTS, bcmap, r, world) for r in range(world)]
    plane = n[0] * n[1]
    for k, (outer, (idst, isrc, _)) in enumerate(bcmap_layers(bcmap)):
        for d in range(3):
            got = np.concatenate([pl.outer[k][d][0].astype(np.int64) + pl.w0 * plane for pl in plans])
            assert sorted(got.tolist()) == sorted(outer[d][0].tolist())
        got = np.concatenate([pl.inner_dest[k].astype(np.int64) + pl.w0 * plane for pl in plans])
        assert sorted(got.tolist()) == sorted(idst.tolist())
        # rank q's requests from rank p are what p sends to q, in q's order
        for q, plq in enumerate(plans):
            for p, plp in enumerate(plans):
                cnt = plq.inner_counts[k][p]
                sent = plp.inner_send[k].get(q)
                assert cnt == (0 if sent is None else len(sent))
        # each request points at its destination's own source
        lookup = dict(zip(idst.tolist(), isrc.tolist()))
        for q, plq in enumerate(plans):
            off = 0
            for p, plp in enumerate(plans):
                cnt = plq.inner_counts[k][p]
                if cnt:
                    dst = plq.inner_dest[k][off:off + cnt].astype(np.int64) + plq.w0 * plane
                    src = plp.inner_send[k][q].astype(np.int64) + plp.w0 * plane
                    assert [lookup[v] for v in dst.tolist()] == src.tolist()
                off += cnt
    # owned planes tile the grid; halos are the neighbours' edge planes
    owned = [pl.owned_global for pl in plans]
    assert owned[0][0] == 0 and owned[-1][1] == n[2]
    assert all(a[1] == b[0] for a, b in zip(owned, owned[1:]))
    for r in range(world - 1):
        a, b = plans[r].halo_send[r + 1]
        c, d = plans[r + 1].halo_recv[r]
        assert plans[r].w0 + a == plans[r + 1].w0 + c and b - a == d - c == gp.NGHOSTS


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, case, nsteps, q):
    try:
        import torch
        import torch.distributed as dist
        os.environ["MASTER_ADDR"] = "127.0.0.1"
        os.environ["MASTER_PORT"] = str(port)
        dist.init_process_group("gloo", rank=rank, world_size=world)
        from nrpytutorial_gb300.slab import DistComm, SlabStepper
        from tests.slab_host import HostSlabOps
        gp = _gp(case)
        y = _initial(case, gp)
        comm = DistComm()
        plans = {rank: SlabPlan(tuple(gp.np), gp.NGHOSTS, oracle_bcmap(gp), rank, world)}
        ops = HostSlabOps(gp, _rhs_fn(case, gp), PARITY[CASES[case][0]], plans, y)
        st = SlabStepper(plans, comm, ops)
        dt = og.find_timestep(gp, 0.5)
        for _ in range(nsteps):
            st.step(dt)
        pl = plans[rank]
        a, b = pl.owned_planes
        mine = ops.buf[rank]["y_n"][:, a:b].clone()
        # norms: all-reduced interior sums of squares
        g = gp.NGHOSTS
        interior = ops.buf[rank]["y_n"][0, g:-g, g:-g, g:-g]
        tot = comm.allreduce_sum({rank: torch.tensor([float((interior ** 2).sum()), float(interior.numel())],
                                                     dtype=torch.float64)})[rank]
        q.put((rank, pl.w0 + a, mine.numpy(), tot.numpy()))
        dist.barrier()
        dist.destroy_process_group()
    except Exception as e:  # report to the parent instead of hanging it
        q.put((rank, "error", repr(e), None))
        raise


@pytest.mark.parametrize("case,world", [("scalarwave_sinhsph", 2), ("maxwell_cartesian", 2),
                                        ("scalarwave_sinhcyl", 3)])
def test_gloo_slab_evolution_matches_the_one_grid_oracle(case, world):
    pytest.importorskip("torch")
    nsteps = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, case, nsteps, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = {}
    try:
        for _ in range(world):
            r, z, y, tot = q.get(timeout=240)
            assert z != "error", y
            res[r] = (z, y, tot)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert all(p.exitcode == 0 for p in procs)
    gp = _gp(case)
    y = _initial(case, gp)
    layers = ob.build_bcstruct(gp)
    post = lambda u: ob.apply_bcs(layers, u, PARITY[CASES[case][0]])
    dt = og.find_timestep(gp, 0.5)
    for _ in range(nsteps):
        y, _, _ = ob.rk4_step(y, dt, _rhs_fn(case, gp), post, gp.NGHOSTS)
    assembled = np.concatenate([res[r][1] for r in range(world)], axis=1)
    assert [res[r][0] for r in range(world)][0] == 0
    assert assembled.shape == y.shape
    assert np.array_equal(assembled, y)
    g = gp.NGHOSTS
    interior = y[0, g:-g, g:-g, g:-g]
    for r in range(world):
        s, n = res[r][2]
        assert n == interior.size
        assert abs(s - float((interior ** 2).sum())) <= 1e-13 * s


def test_grid_slab_is_the_window_of_the_grid():
    from nrpytutorial_gb300 import Grid
    G = Grid("SinhSpherical", (10, 6, 12), FD_order=4, NGHOSTS=3, AMPL=5.0, SINHW=0.3)
    s = G.slab(4, 13)  # planes 4..12: 3 interior planes' worth of halo on each side + 3 owned
    p, q = G.params, s.params
    assert q.Nxx2 == 3 and q.Nxx_plus_2NGHOSTS2 == 9 and s.shape == (9, G.shape[1], G.shape[2])
    assert q.dxx2 == p.dxx2 and q.Nxx0 == p.Nxx0 and q.Nxx1 == p.Nxx1
    # the slab's cell-centred xx2 are the grid's planes 4..12
    xx2 = q.xxmin2 + (np.arange(9) - 3 + 0.5) * q.dxx2
    assert np.allclose(xx2, np.asarray(G.xx[2])[4:13], rtol=0, atol=1e-14)
    assert np.array_equal(s.xx[2], np.asarray(G.xx[2])[4:13])
    with pytest.raises(ValueError):
        G.slab(0, 6)  # no interior plane
