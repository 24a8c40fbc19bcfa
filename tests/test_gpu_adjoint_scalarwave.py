"""Discrete adjoint of the ScalarWave evolution on the GPU, Cartesian and
curvilinear: transposes checked by dot-product identities (RHS for every
built coordinate family, boundary conditions with inner parity maps, one
RK4 step), the Gaussian-pulse parameter derivatives, and the gradient of the
radial-shell observable with respect to (A, r0, w) against central finite
differences (h = 1e-6, 1e-6 relative) and against a PyTorch-autograd
reference of the same discrete problem (tests/scalarwave_torch_ref.py)."""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import grids

pytestmark = pytest.mark.gpu

SPH_KW = dict(AMPL=6.0, SINHW=0.3)


def _interior_mask(G, like):
    import torch
    g = G.params.NGHOSTS
    m = torch.zeros_like(like)
    m[:, g:-g, g:-g, g:-g] = 1.0
    return m


def _dot(a, b):
    return float((a * b).sum())


def _rel(a, b):
    return abs(a - b) / max(abs(a), abs(b), 1e-300)


@pytest.mark.parametrize("coord,Nxx,order,kw", [
    ("Cartesian", (10, 12, 8), 4, dict(domain=(-2.0, 2.0))),
    ("Cartesian", (10, 10, 10), 8, dict(domain=(-2.0, 2.0))),
    ("Spherical", (12, 8, 8), 2, dict(RMAX=4.0)),
    ("SinhSpherical", (12, 8, 8), 4, SPH_KW),
    ("SinhSphericalv2", (12, 8, 8), 6, SPH_KW),
    ("SinhCylindrical", (10, 8, 10), 4, {}),
    ("Cylindrical", (10, 8, 10), 2, {}),
    ("SinhSymTP", (10, 8, 8), 4, {}),
    ("SymTP", (10, 8, 8), 2, {}),
])
def test_rhs_adjoint_is_the_transpose(cuda, coord, Nxx, order, kw):
    import torch
    from nrpytutorial_gb300 import Evolution, _lib
    G, _ = grids("ScalarWave", coord, Nxx, order, **kw)
    ev = Evolution("ScalarWave", G, device=cuda)
    rng = np.random.default_rng(order + len(coord))
    x = torch.tensor(rng.standard_normal(ev.y_n.shape), device=cuda)
    y = torch.tensor(rng.standard_normal(ev.y_n.shape), device=cuda) * _interior_mask(G, ev.y_n)
    Lx = torch.zeros_like(x)
    ev.rhs_eval(x, Lx)
    LTy = torch.zeros_like(x)
    _lib.check(ev.lib.ScalarWave_rhs_eval_adjoint(ev._rfm(), C.byref(G.params), _lib.ptr(y), _lib.ptr(LTy)),
               "ScalarWave_rhs_eval_adjoint")
    a, b = _dot(Lx, y), _dot(x, LTy)
    assert _rel(a, b) <= 1e-12, (a, b)


def test_rhs_adjoint_rejects_a_missing_rfm(cuda):
    from nrpytutorial_gb300 import Evolution, _lib
    import torch
    G, _ = grids("ScalarWave", "SinhSpherical", (8, 6, 6), 4, **SPH_KW)
    ev = Evolution("ScalarWave", G, device=cuda)
    a, b = torch.zeros_like(ev.y_n), torch.zeros_like(ev.y_n)
    st = ev.lib.ScalarWave_rhs_eval_adjoint(None, C.byref(G.params), _lib.ptr(a), _lib.ptr(b))
    assert st != 0


@pytest.mark.parametrize("coord,kw", [("SinhSpherical", SPH_KW), ("SinhCylindrical", {}), ("SinhSymTP", {})])
def test_bc_adjoint_is_the_transpose_with_inner_parity(cuda, coord, kw):
    import torch
    from nrpytutorial_gb300 import Evolution, _lib
    G, _ = grids("ScalarWave", coord, (10, 8, 8), 4, **kw)
    ev = Evolution("ScalarWave", G, device=cuda)
    rng = np.random.default_rng(5)
    x = torch.tensor(rng.standard_normal(ev.y_n.shape), device=cuda)
    y = torch.tensor(rng.standard_normal(ev.y_n.shape), device=cuda)
    Bx = x.clone()
    ev.apply_bcs(Bx)
    BTy = y.clone()
    _lib.check(ev.lib.apply_bcs_curvilinear_adjoint(C.byref(G.params), C.byref(ev.bc), 2,
                                                    C.cast(ev.parity, C.POINTER(C.c_int8)), _lib.ptr(BTy)),
               "bc adjoint")
    a, b = _dot(Bx, y), _dot(x, BTy)
    assert _rel(a, b) <= 1e-12, (a, b)


@pytest.mark.parametrize("coord,Nxx,order,kw", [
    ("Cartesian", (10, 10, 10), 4, dict(domain=(-2.0, 2.0))),
    ("SinhSpherical", (12, 8, 8), 4, SPH_KW),
    ("SinhCylindrical", (10, 8, 10), 4, {}),
])
def test_rk4_step_adjoint_is_the_transpose(cuda, coord, Nxx, order, kw):
    import torch
    from nrpytutorial_gb300 import Evolution, _lib
    G, _ = grids("ScalarWave", coord, Nxx, order, **kw)
    ev = Evolution("ScalarWave", G, device=cuda)
    dt = G.find_timestep(0.5)
    rng = np.random.default_rng(2)
    x = torch.tensor(rng.standard_normal(ev.y_n.shape), device=cuda)
    y = torch.tensor(rng.standard_normal(ev.y_n.shape), device=cuda)
    ev.y_n.copy_(x)
    ev.step(dt)
    Phix = ev.y_n.clone()
    lam_in, lam_out = y.clone(), torch.zeros_like(y)
    scratch = torch.zeros((4,) + tuple(y.shape), dtype=torch.float64, device=cuda)
    _lib.check(ev.lib.MoL_adjoint_step_backward(ev.sys_id, ev._rfm(), C.byref(G.params), C.byref(ev.bc),
                                                _lib.ptr(lam_in), _lib.ptr(lam_out), _lib.ptr(scratch), dt),
               "adjoint step")
    a, b = _dot(Phix, y), _dot(x, lam_out)
    assert _rel(a, b) <= 1e-12, (a, b)


def _problem(cuda, keep=True, K=5, coord="SinhSpherical", Nxx=(16, 8, 8), n_steps=20):
    from nrpytutorial_gb300.adjoint import ScalarWaveExtraction
    G, gp = grids("ScalarWave", coord, Nxx, 4, **SPH_KW)
    i0 = gp.NGHOSTS + (2 * Nxx[0]) // 3
    return ScalarWaveExtraction(G, i0, n_steps=n_steps, checkpoint_every=K, keep_samples=keep, device=cuda), gp


def test_gaussian_pulse_and_its_derivatives(cuda):
    import torch
    import oracle.grid as og
    m, gp = _problem(cuda)
    A, r0, w = 0.8, 1.5, 0.9
    y = torch.zeros_like(m.ev.y_n)
    d = [torch.zeros_like(y) for _ in range(3)]
    m.initial_data(A, r0, w, out=y, derivs=d)
    # the Cartesian radius: |r(xx0)| (r(xx0) < 0 at the inner ghost points)
    r = np.abs(og.radial(gp.CoordSystem, gp.xx[0], gp.AMPL, gp.SINHW)[0])[None, None, :]

    def u(A, r0, w):
        return A * np.exp(-((r - r0) / w) ** 2) * np.ones(gp.shape)

    got = y.cpu().numpy()
    assert np.allclose(got[0], u(A, r0, w), rtol=1e-13, atol=1e-15)
    assert float(np.abs(got[1]).max()) == 0.0
    h = 1e-6
    fds = [(u(A + h, r0, w) - u(A - h, r0, w)) / (2 * h), (u(A, r0 + h, w) - u(A, r0 - h, w)) / (2 * h),
           (u(A, r0, w + h) - u(A, r0, w - h)) / (2 * h)]
    for k in range(3):
        assert np.allclose(d[k].cpu().numpy()[0], fds[k], rtol=1e-6, atol=1e-9), k


def test_shell_weights_sum_to_the_sphere_area(cuda):
    from nrpytutorial_gb300.adjoint import shell_weights
    m, gp = _problem(cuda, Nxx=(16, 32, 64))
    import oracle.grid as og
    r = float(og.radial(gp.CoordSystem, gp.xx[0][m.i0], gp.AMPL, gp.SINHW)[0])
    assert abs(shell_weights(m.grid, m.i0).sum() / (4 * np.pi * r * r) - 1.0) < 2e-3


def test_gradient_matches_central_differences(cuda):
    m, _ = _problem(cuda)
    A, r0, w = 0.9, 1.5, 0.8
    m.forward(A, r0, w)
    g = m.gradient()
    h = 1e-6
    fd = []
    for k in range(3):
        p, q = [A, r0, w], [A, r0, w]
        p[k] += h
        q[k] -= h
        fd.append((m.forward(*p) - m.forward(*q)) / (2 * h))
    fd = np.array(fd)
    assert np.allclose(g, fd, rtol=1e-6, atol=0), (g, fd)


def test_gradient_matches_pytorch_autograd_reference(cuda):
    from tests.scalarwave_torch_ref import TorchScalarWave
    from nrpytutorial_gb300.adjoint import shell_weights
    m, gp = _problem(cuda, n_steps=12)
    A, r0, w = 0.9, 1.5, 0.8
    J = m.forward(A, r0, w)
    g = m.gradient()
    ref = TorchScalarWave(gp, m.i0, shell_weights(m.grid, m.i0), n_steps=12)
    assert abs(ref.dt - m.dt) <= 1e-15 * m.dt
    Jr, gr = ref.gradient(A, r0, w)
    assert abs(J - Jr) <= 1e-12 * Jr, (J, Jr)
    assert np.allclose(g, gr, rtol=1e-10, atol=0), (g, gr)


def test_checkpoint_recompute_gives_the_same_gradient(cuda):
    a, _ = _problem(cuda, keep=True)
    b, _ = _problem(cuda, keep=False, K=6)
    Ja, Jb = a.forward(0.7, 1.4, 0.9), b.forward(0.7, 1.4, 0.9)
    assert Ja == Jb
    assert sorted(b.checkpoints) == [0, 6, 12, 18, 20]
    ga, gb = a.gradient(), b.gradient()
    assert np.allclose(ga, gb, rtol=1e-13, atol=0), (ga, gb)


def test_autograd_function(cuda):
    import torch
    from nrpytutorial_gb300.adjoint import extraction_observable
    m, _ = _problem(cuda)
    p = torch.tensor([0.9, 1.5, 0.8], dtype=torch.float64, requires_grad=True)
    J = extraction_observable(p, m)
    (3.0 * J).backward()
    assert np.allclose(p.grad.numpy(), 3.0 * m.gradient(), rtol=1e-14)


def test_shell_must_be_interior_and_spherical(cuda):
    from nrpytutorial_gb300.adjoint import ScalarWaveExtraction
    G, gp = grids("ScalarWave", "SinhSpherical", (12, 8, 8), 4, **SPH_KW)
    with pytest.raises(ValueError):
        ScalarWaveExtraction(G, 0, n_steps=2, device=cuda)
    Gc, _ = grids("ScalarWave", "SinhCylindrical", (10, 8, 10), 4)
    with pytest.raises(ValueError):
        ScalarWaveExtraction(Gc, 5, n_steps=2, device=cuda)
