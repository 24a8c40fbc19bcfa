"""MoL_evolve_host, the host-buffer evolution (copy in, n steps, copy out),
against the same steps on the device state, bit for bit.  Pageable host
arrays run eagerly; pinned ones replay a CUDA graph of the call from its
second repetition on, and a changed call (another step count) is captured
afresh."""
import numpy as np
import pytest

from tests.helpers import grids

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["compensated", "fp64"])
@pytest.mark.parametrize("pinned", [True, False])
def test_evolve_host_equals_the_device_steps(cuda, prec, pinned):
    import torch
    from nrpytutorial_gb300 import Evolution
    from tests.test_gpu_compensated import KW, _state
    system, coord, Nxx, order = "BSSN", "SinhSpherical", (12, 10, 8), 4
    G, gp = grids(system, coord, Nxx, order, **KW)
    dt = G.find_timestep(0.5)
    ev = Evolution(system, G, precision=prec, device=cuda)
    ev.y_n.copy_(torch.tensor(_state(system, gp), device=cuda))
    ev.apply_bcs(ev.y_n)
    ev.enforce_detgammabar(ev.y_n)
    start = ev.y_n.cpu().numpy().copy()
    refs = []
    for _ in range(8):
        ev.step(dt)
        torch.cuda.synchronize()
        refs.append(ev.y_n.cpu().numpy().copy())
    if pinned:
        h = torch.empty(start.shape, dtype=torch.float64, pin_memory=True)
        h.copy_(torch.from_numpy(start))
        hn = h.numpy()
    else:
        hn = start.copy()
    for n in range(4):  # one step per call: eager, captured, replayed, replayed
        ev.evolve_host(hn, dt, 1)
        assert np.array_equal(hn, refs[n]), n
    for n in range(2):  # two steps per call: a new configuration
        ev.evolve_host(hn, dt, 2)
        assert np.array_equal(hn, refs[5 + 2 * n]), n


@pytest.mark.parametrize("system,coord,Nxx,prec", [("ScalarWave", "SinhSpherical", (16, 12, 8), "mixed"),
                                                    ("Maxwell", "Cartesian", (12, 12, 12), "fp64")])
def test_evolve_host_other_systems(cuda, system, coord, Nxx, prec):
    import torch
    from nrpytutorial_gb300 import Evolution
    from tests.test_gpu_compensated import KW, _state
    G, gp = grids(system, coord, Nxx, 4, **KW)
    dt = G.find_timestep(0.5)
    ev = Evolution(system, G, precision=prec, device=cuda)
    ev.y_n.copy_(torch.tensor(_state(system, gp), device=cuda))
    ev.apply_bcs(ev.y_n)
    start = ev.y_n.cpu().numpy().copy()
    refs = []
    for _ in range(3):
        ev.step(dt)
        torch.cuda.synchronize()
        refs.append(ev.y_n.cpu().numpy().copy())
    h = torch.empty(start.shape, dtype=torch.float64, pin_memory=True)
    h.copy_(torch.from_numpy(start))
    hn = h.numpy()
    for n in range(3):
        ev.evolve_host(hn, dt, 1)
        assert np.array_equal(hn, refs[n]), n
