"""Slab-decomposed evolution (nrpytutorial_gb300.slab) on one GPU: two or
three ranks driven in this process (LocalComm; the exchanges hand buffers
over, no kernel waits on another rank) with the library's kernels, against
the one-grid MoL_step_forward_in_time.  Each rank owns whole i2 planes and
writes its points from the same values as the one-grid step, so the owned
planes agree bit for bit where the slab's reference-metric table equals the
grid's (Cartesian and the Spherical family: the tables depend on xx0, xx1
only); SinhCylindrical's table depends on xx2 = z, which a slab recomputes
from its own xxmin2, so there the bound is 1e-13."""
import numpy as np
import pytest

from tests.helpers import grids, smooth_state

pytestmark = pytest.mark.gpu

CASES = [
    ("ScalarWave", "SinhSpherical", (12, 8, 12), 4, 2, dict(AMPL=5.0, SINHW=0.3)),
    ("ScalarWave", "SinhSpherical", (12, 8, 12), 4, 3, dict(AMPL=5.0, SINHW=0.3)),
    ("Maxwell", "Cartesian", (8, 10, 12), 4, 3, dict(domain=(-2.0, 2.0))),
    ("ScalarWave", "SinhCylindrical", (10, 8, 12), 4, 2, {}),
    ("BSSN", "SinhSpherical", (12, 8, 12), 4, 2, dict(AMPL=5.0, SINHW=0.3)),
    ("BSSN", "Cartesian", (10, 10, 12), 4, 3, dict(domain=(-2.0, 2.0))),
]


@pytest.mark.parametrize("system,coord,Nxx,order,world,kw", CASES)
def test_local_ranks_reproduce_the_one_grid_step(cuda, system, coord, Nxx, order, world, kw):
    import torch
    from nrpytutorial_gb300 import Evolution
    from nrpytutorial_gb300.slab import LocalComm, SlabEvolution
    ng = 3
    G, gp = grids(system, coord, Nxx, order, ng=ng, **kw)
    ev = Evolution(system, G, precision="fp64", device=cuda)
    ngf = ev.ngf
    offs = {6: 1.0, 10: 1.0} if system == "BSSN" else None  # alpha, W around flat space
    y = smooth_state(ngf, gp, seed=11, amp=0.02, offsets=offs)
    ev.y_n.copy_(torch.tensor(y, device=cuda))
    ev.apply_bcs(ev.y_n)
    if system == "BSSN":
        ev.enforce_detgammabar(ev.y_n)
    sl = SlabEvolution(system, G, LocalComm(world), device=cuda)
    sl.set_state(ev.y_n)
    dt = G.find_timestep(0.5)
    for _ in range(3):
        ev.step(dt)
        sl.step(dt)
    ref = ev.y_n.cpu().numpy()
    parts = []
    for r in range(world):
        z, mine = sl.owned_state(r)
        parts.append((z, mine.cpu().numpy()))
    parts.sort(key=lambda t: t[0])
    assert parts[0][0] == 0
    got = np.concatenate([p for _, p in parts], axis=1)
    assert got.shape == ref.shape
    if coord == "SinhCylindrical":
        assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
    else:
        assert np.array_equal(got, ref)
    n_sl = sl.l2_norm(0)
    n_ev = ev.l2_norm(ev.y_n, 0)
    assert abs(n_sl - n_ev) <= 1e-13 * n_ev


def test_slab_evolution_rejects_too_many_ranks(cuda):
    from nrpytutorial_gb300.slab import LocalComm, SlabEvolution
    G, _ = grids("ScalarWave", "Cartesian", (8, 8, 8), 4, ng=3, domain=(-1.0, 1.0))
    with pytest.raises(ValueError):
        SlabEvolution("ScalarWave", G, LocalComm(3), device=cuda)  # 8 planes < 3 x 3


def test_slab_rank_has_no_full_grid_step(cuda):
    from nrpytutorial_gb300.slab import LocalComm, SlabEvolution
    G, _ = grids("ScalarWave", "Cartesian", (8, 8, 12), 4, ng=3, domain=(-1.0, 1.0))
    sl = SlabEvolution("ScalarWave", G, LocalComm(2), device=cuda)
    with pytest.raises(RuntimeError):
        sl.local(0).step(0.01)


def test_slab_step_graph_replay_equals_the_eager_step(cuda):
    import torch
    from nrpytutorial_gb300.slab import LocalComm, SlabEvolution
    G, gp = grids("ScalarWave", "SinhSpherical", (12, 8, 12), 4, ng=3, AMPL=5.0, SINHW=0.3)
    y = torch.tensor(smooth_state(2, gp, seed=3, amp=0.1), device=cuda)
    a = SlabEvolution("ScalarWave", G, LocalComm(3), device=cuda)
    b = SlabEvolution("ScalarWave", G, LocalComm(3), device=cuda)
    a.set_state(y)
    b.set_state(y)
    dt = G.find_timestep(0.5)
    replay = b.capture(dt, 2)
    for _ in range(2):
        a.step(dt)
    replay()
    torch.cuda.synchronize()
    for r in range(3):
        assert torch.equal(a.owned_state(r)[1], b.owned_state(r)[1])
