"""Discrete adjoint of the Maxwell evolution on the GPU: transposes checked by
dot-product identities (RHS, boundary conditions, one RK4 step), the
toroidal-dipole parameter derivatives, and the gradient of the extraction
observable against central finite differences (h = 1e-6) and against a
PyTorch-autograd reference of the same discrete problem."""
import ctypes as C

import numpy as np
import pytest

from tests.maxwell_torch_ref import TorchMaxwell

pytestmark = pytest.mark.gpu

DOMAIN = (-4.0, 4.0)


def _grid(N=16, order=4):
    from nrpytutorial_gb300 import Grid
    return Grid("Cartesian", (N, N, N), FD_order=order, NGHOSTS=order // 2 + 1, domain=DOMAIN)


def _interior_mask(G, like):
    import torch
    g = G.params.NGHOSTS
    m = torch.zeros_like(like)
    m[:, g:-g, g:-g, g:-g] = 1.0
    return m


def _dot(a, b):
    return float((a * b).sum())


@pytest.mark.parametrize("order", [2, 4, 6])
def test_rhs_adjoint_is_the_transpose(cuda, order):
    import torch
    from nrpytutorial_gb300 import Evolution, _lib
    G = _grid(12, order)
    ev = Evolution("Maxwell", G, device=cuda)
    rng = np.random.default_rng(order)
    x = torch.tensor(rng.standard_normal(ev.y_n.shape), device=cuda)
    y = torch.tensor(rng.standard_normal(ev.y_n.shape), device=cuda) * _interior_mask(G, ev.y_n)
    Lx = torch.zeros_like(x)
    ev.rhs_eval(x, Lx)
    LTy = torch.zeros_like(x)
    _lib.check(ev.lib.Maxwell_rhs_eval_adjoint(C.byref(G.params), _lib.ptr(y), _lib.ptr(LTy)), "adjoint")
    a, b = _dot(Lx, y), _dot(x, LTy)
    assert abs(a - b) <= 1e-12 * max(abs(a), 1.0), (a, b)


def test_bc_adjoint_is_the_transpose(cuda):
    import torch
    from nrpytutorial_gb300 import Evolution, _lib
    G = _grid(10)
    ev = Evolution("Maxwell", G, device=cuda)
    rng = np.random.default_rng(1)
    x = torch.tensor(rng.standard_normal(ev.y_n.shape), device=cuda)
    y = torch.tensor(rng.standard_normal(ev.y_n.shape), device=cuda)
    Bx = x.clone()
    ev.apply_bcs(Bx)
    BTy = y.clone()
    _lib.check(ev.lib.apply_bcs_curvilinear_adjoint(C.byref(G.params), C.byref(ev.bc), 7,
                                                    C.cast(ev.parity, C.POINTER(C.c_int8)), _lib.ptr(BTy)),
               "bc adjoint")
    a, b = _dot(Bx, y), _dot(x, BTy)
    assert abs(a - b) <= 1e-12 * abs(a), (a, b)
    # every ghost point is a boundary point: the transpose leaves no ghost adjoint
    assert float((BTy * (1 - _interior_mask(G, BTy))).abs().max()) == 0.0


def test_rk4_step_adjoint_is_the_transpose(cuda):
    import torch
    from nrpytutorial_gb300 import Evolution, _lib
    G = _grid(12)
    ev = Evolution("Maxwell", G, device=cuda)
    dt = G.find_timestep(0.5)
    rng = np.random.default_rng(2)
    x = torch.tensor(rng.standard_normal(ev.y_n.shape), device=cuda)
    y = torch.tensor(rng.standard_normal(ev.y_n.shape), device=cuda)
    ev.y_n.copy_(x)
    ev.step(dt)
    Phix = ev.y_n.clone()
    lam_in, lam_out = y.clone(), torch.zeros_like(y)
    scratch = torch.zeros((4,) + tuple(y.shape), dtype=torch.float64, device=cuda)
    _lib.check(ev.lib.MoL_adjoint_step_backward(1, None, C.byref(G.params), C.byref(ev.bc), _lib.ptr(lam_in),
                                                _lib.ptr(lam_out), _lib.ptr(scratch), dt), "adjoint step")
    a, b = _dot(Phix, y), _dot(x, lam_out)
    assert abs(a - b) <= 1e-12 * abs(a), (a, b)


def test_toroidal_dipole_matches_oracle_and_derivatives(cuda):
    import torch
    import oracle.grid as og
    import oracle.wave_maxwell as ow
    from nrpytutorial_gb300.adjoint import ExtractionSphere, MaxwellExtraction
    G = _grid(12)
    m = MaxwellExtraction(G, ExtractionSphere(2.0, 4, 8), n_steps=1, device=cuda)
    amp, lam = 0.8, 1.1
    y = torch.zeros_like(m.ev.y_n)
    da, dl = torch.zeros_like(y), torch.zeros_like(y)
    m.initial_data(amp, lam, out=y, d_amp=da, d_lam=dl)
    gp = og.GridParams("Cartesian", (12, 12, 12), 3, 4, domain=DOMAIN)
    ref = ow.toroidal_dipole(gp, 0.0, amp, lam)
    assert np.allclose(y.cpu().numpy(), ref, rtol=1e-13, atol=1e-13)
    h = 1e-6
    fd = (ow.toroidal_dipole(gp, 0.0, amp, lam + h) - ow.toroidal_dipole(gp, 0.0, amp, lam - h)) / (2 * h)
    assert np.allclose(dl.cpu().numpy(), fd, rtol=1e-6, atol=1e-8)
    assert np.allclose(da.cpu().numpy() * amp, ref, rtol=1e-14, atol=1e-14)


def _problem(cuda, keep=True, K=5):
    from nrpytutorial_gb300.adjoint import ExtractionSphere, MaxwellExtraction
    G = _grid(16)
    sph = ExtractionSphere(2.5, ntheta=8, nphi=16)
    return MaxwellExtraction(G, sph, n_steps=24, checkpoint_every=K, keep_samples=keep, device=cuda), sph


def test_gradient_matches_central_differences(cuda):
    m, _ = _problem(cuda)
    amp, lam = 0.9, 1.2
    m.forward(amp, lam)
    g = m.gradient()
    h = 1e-6
    fd = np.array([(m.forward(amp + h, lam) - m.forward(amp - h, lam)) / (2 * h),
                   (m.forward(amp, lam + h) - m.forward(amp, lam - h)) / (2 * h)])
    assert np.allclose(g, fd, rtol=1e-6, atol=0), (g, fd)


def test_gradient_matches_pytorch_autograd_reference(cuda):
    m, sph = _problem(cuda)
    amp, lam = 0.9, 1.2
    J = m.forward(amp, lam)
    g = m.gradient()
    ref = TorchMaxwell(16, DOMAIN, sph.points, sph.weights, n_steps=24)
    Jr, gr = ref.gradient(amp, lam)
    assert abs(J - Jr) <= 1e-12 * Jr, (J, Jr)
    assert np.allclose(g, gr, rtol=1e-10, atol=0), (g, gr)


def test_checkpoint_recompute_gives_the_same_gradient(cuda):
    a, _ = _problem(cuda, keep=True)
    b, _ = _problem(cuda, keep=False, K=5)
    Ja, Jb = a.forward(0.7, 0.9), b.forward(0.7, 0.9)
    assert Ja == Jb
    assert sorted(b.checkpoints) == [0, 5, 10, 15, 20, 24]
    ga, gb = a.gradient(), b.gradient()
    assert np.allclose(ga, gb, rtol=1e-13, atol=0), (ga, gb)


def test_autograd_function(cuda):
    import torch
    from nrpytutorial_gb300.adjoint import extraction_observable
    m, _ = _problem(cuda)
    p = torch.tensor([0.9, 1.2], dtype=torch.float64, requires_grad=True)
    J = extraction_observable(p, m)
    (2.0 * J).backward()
    assert np.allclose(p.grad.numpy(), 2.0 * m.gradient(), rtol=1e-14)
