"""Forward-mode (tangent-linear) BSSN on the GPU: the dual-number RHS
against the FP64 RHS and against central differences of it, the
Brill-Lindquist parameter derivatives, the tangent step's value against
the library's unfused FP64 step, and the gradient of the lapse-on-a-shell
observable with respect to the Brill-Lindquist masses and positions against
central differences of the same discrete evolution (h = 1e-6, 1e-6
relative)."""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import grids, per_gf_rel, smooth_state

pytestmark = pytest.mark.gpu

SPH = dict(AMPL=4.0, SINHW=0.3)


def _state(gp, seed=5):
    offs = {6: 1.0, 10: 1.0}  # alpha, W around flat space
    return smooth_state(24, gp, seed=seed, amp=0.02, offsets=offs)


def _tangent_rhs(ev, G, Y, ntan):
    import torch
    from nrpytutorial_gb300 import _lib
    aux = torch.zeros(((ntan + 1) * 6,) + tuple(G.shape), dtype=torch.float64, device=Y.device)
    out = torch.zeros_like(Y)
    _lib.check(ev.lib.BSSN_tangent_rhs_eval(ev._rfm(), C.byref(G.params), ntan, _lib.ptr(Y), _lib.ptr(aux),
                                            _lib.ptr(out)), "BSSN_tangent_rhs_eval")
    return out


@pytest.mark.parametrize("coord,kw", [("Cartesian", dict(domain=(-2.0, 2.0))), ("SinhSpherical", SPH)])
def test_value_path_matches_the_fp64_rhs(cuda, coord, kw):
    import torch
    from nrpytutorial_gb300 import Evolution
    G, gp = grids("BSSN", coord, (10, 8, 8), 4, ng=3, **kw)
    ev = Evolution("BSSN", G, precision="fp64", device=cuda)
    y = torch.tensor(_state(gp), device=cuda)
    ref = torch.zeros_like(y)
    ev.rhs_eval(y, ref)
    got = _tangent_rhs(ev, G, y.clone(), 0)
    g = gp.NGHOSTS
    assert per_gf_rel(got.cpu().numpy(), ref.cpu().numpy(), ng=g) < 1e-13


@pytest.mark.parametrize("coord,kw", [("Cartesian", dict(domain=(-2.0, 2.0))), ("SinhSpherical", SPH)])
@pytest.mark.parametrize("ntan", [1, 2, 4])
def test_tangent_rhs_matches_central_differences(cuda, coord, kw, ntan):
    import torch
    from nrpytutorial_gb300 import Evolution
    G, gp = grids("BSSN", coord, (10, 8, 8), 4, ng=3, **kw)
    ev = Evolution("BSSN", G, precision="fp64", device=cuda)
    y = _state(gp)
    dys = [smooth_state(24, gp, seed=20 + k, amp=0.01) for k in range(ntan)]
    Y = torch.tensor(np.concatenate([y] + dys), device=cuda)
    got = _tangent_rhs(ev, G, Y, ntan).cpu().numpy()
    g = gp.NGHOSTS
    h = 1e-5
    for k in range(ntan):
        yp = torch.tensor(y + h * dys[k], device=cuda)
        ym = torch.tensor(y - h * dys[k], device=cuda)
        rp, rm = torch.zeros_like(yp), torch.zeros_like(ym)
        ev.rhs_eval(yp, rp)
        ev.rhs_eval(ym, rm)
        fd = ((rp - rm) / (2 * h)).cpu().numpy()
        t = got[24 * (k + 1):24 * (k + 2)]
        assert per_gf_rel(t, fd, ng=g) < 1e-6, k
    # the value component is the FP64 RHS whatever the number of tangents
    r0 = _tangent_rhs(ev, G, torch.tensor(y, device=cuda), 0).cpu().numpy()
    assert per_gf_rel(got[:24], r0, ng=g) < 1e-12


def test_one_and_four_tangents_agree(cuda):
    import torch
    from nrpytutorial_gb300 import Evolution
    G, gp = grids("BSSN", "SinhSpherical", (10, 8, 8), 4, ng=3, **SPH)
    ev = Evolution("BSSN", G, precision="fp64", device=cuda)
    y = _state(gp)
    dys = [smooth_state(24, gp, seed=30 + k, amp=0.01) for k in range(4)]
    four = _tangent_rhs(ev, G, torch.tensor(np.concatenate([y] + dys), device=cuda), 4).cpu().numpy()
    g = gp.NGHOSTS
    for k in range(4):
        one = _tangent_rhs(ev, G, torch.tensor(np.concatenate([y, dys[k]]), device=cuda), 1).cpu().numpy()
        assert per_gf_rel(four[24 * (k + 1):24 * (k + 2)], one[24:], ng=g) < 1e-13


@pytest.mark.parametrize("coord,kw", [("Cartesian", dict(domain=(-2.0, 2.0))), ("SinhSpherical", SPH)])
def test_brill_lindquist_derivatives_match_central_differences(cuda, coord, kw):
    import torch
    from nrpytutorial_gb300 import Evolution, _lib
    G, gp = grids("BSSN", coord, (10, 8, 8), 4, ng=3, **kw)
    ev = Evolution("BSSN", G, precision="fp64", device=cuda)
    base = [0.4, 0.3, (0.1, -0.05, 0.6), (-0.1, 0.05, -0.5)]  # m1, m2, x1, x2

    def bl(m1, m2, x1, x2):
        out = torch.zeros((24,) + tuple(G.shape), dtype=torch.float64, device=cuda)
        ev.initial_data_brill_lindquist(m1, x1, m2, x2, gfs=out)
        return out.cpu().numpy()

    pidx = (C.c_int * 4)(0, 1, 4, 5)  # m1, m2, z1, x2
    Y = torch.zeros((5 * 24,) + tuple(G.shape), dtype=torch.float64, device=cuda)
    m1, m2, x1, x2 = base
    _lib.check(ev.lib.BSSN_tangent_initial_data_BrillLindquist(
        C.byref(G.params), m1, (C.c_double * 3)(*x1), m2, (C.c_double * 3)(*x2), 4, pidx, _lib.ptr(Y)), "bl")
    Y = Y.cpu().numpy()
    assert np.array_equal(Y[:24], bl(m1, m2, x1, x2))
    h = 1e-6

    def shifted(q, s):
        m1, m2, x1, x2 = base[0], base[1], list(base[2]), list(base[3])
        if q == 0: m1 += s
        elif q == 1: m2 += s
        elif q <= 4: x1[q - 2] += s
        else: x2[q - 5] += s
        return bl(m1, m2, x1, x2)

    for k, q in enumerate((0, 1, 4, 5)):
        fd = (shifted(q, h) - shifted(q, -h)) / (2 * h)
        t = Y[24 * (k + 1):24 * (k + 2)]
        for gf in (6, 10):  # alpha, W: the only parameter-dependent gridfunctions
            assert np.allclose(t[gf], fd[gf], rtol=1e-6, atol=1e-9 * np.abs(fd[gf]).max()), (q, gf)
        # the others depend on the parameters only through rounding: the
        # data's hDD and lambdaU come from cancelling psi-dependent terms
        # (psi^4 times cbrt(1/psi^12)), whose FP64 noise / h is ~1e-8 here;
        # their derivatives are zero
        others = [gf for gf in range(24) if gf not in (6, 10)]
        assert np.abs(fd[others]).max() < 1e-6 and float(np.abs(t[others]).max()) == 0.0


@pytest.mark.parametrize("coord,kw", [("Cartesian", dict(domain=(-2.0, 2.0))), ("SinhSpherical", SPH)])
def test_plain_tangent_step_matches_the_unfused_fp64_step(cuda, coord, kw):
    import torch
    from nrpytutorial_gb300 import Evolution, _lib
    G, gp = grids("BSSN", coord, (10, 8, 8), 4, ng=3, **kw)
    ev = Evolution("BSSN", G, precision="fp64", device=cuda)
    ev.initial_data_brill_lindquist(0.4, (0.0, 0.0, 0.6), 0.3, (0.0, 0.0, -0.5))
    Y = ev.y_n.clone()
    scratch = torch.zeros(78 * G.ntot, dtype=torch.float64, device=cuda)
    dt = G.find_timestep(0.5)
    for _ in range(3):
        ev.step(dt, fused=False)
        _lib.check(ev.lib.BSSN_tangent_step(ev._rfm(), C.byref(G.params), C.byref(ev.bc), 0, _lib.ptr(Y),
                                            _lib.ptr(scratch), dt), "BSSN_tangent_step")
    # per gridfunction, with an absolute floor from the state's norm for the
    # gridfunctions that vanish by symmetry (the phi components of head-on
    # data, rounding noise at 1e-19)
    a, b = Y.cpu().numpy(), ev.y_n.cpu().numpy()
    floor = 1e-14 * np.linalg.norm(b)
    for gf in range(24):
        assert np.linalg.norm(a[gf] - b[gf]) <= 1e-12 * np.linalg.norm(b[gf]) + floor, gf


def _model(cuda, coord, kw, params, n_steps=8, Nxx=(12, 8, 8)):
    from nrpytutorial_gb300.tangent import BrillLindquistGradient
    G, gp = grids("BSSN", coord, Nxx, 4, ng=3, **kw)
    i0 = gp.NGHOSTS + (2 * Nxx[0]) // 3
    return BrillLindquistGradient(G, i0, n_steps=n_steps, params=params, device=cuda)


BASE = (0.4, (0.0, 0.0, 0.6), 0.3, (0.0, 0.0, -0.5))


@pytest.mark.parametrize("coord,kw,params", [
    ("SinhSpherical", SPH, ("m1", "m2", "z1", "z2")),
    ("Cartesian", dict(domain=(-2.0, 2.0)), ("m1", "x1", "z2")),
])
def test_gradient_matches_central_differences(cuda, coord, kw, params):
    from nrpytutorial_gb300.tangent import PARAMS, BrillLindquistGradient
    m = _model(cuda, coord, kw, params)
    J, g = m.value_and_gradient(*BASE)
    assert J == pytest.approx(m.value_only(*BASE), rel=1e-12)
    theta = np.array([BASE[0], BASE[2], *BASE[1], *BASE[3]], dtype=float)
    h = 1e-6
    for k, name in enumerate(params):
        q = PARAMS.index(name)
        tp, tm = theta.copy(), theta.copy()
        tp[q] += h
        tm[q] -= h
        fd = (m.value_only(*BrillLindquistGradient.unpack(tp)) - m.value_only(*BrillLindquistGradient.unpack(tm))) / (2 * h)
        assert g[k] == pytest.approx(fd, rel=1e-6, abs=1e-9 * abs(J)), (name, g[k], fd)


def test_autograd_function(cuda):
    import torch
    from nrpytutorial_gb300.tangent import brill_lindquist_observable
    m = _model(cuda, "SinhSpherical", SPH, ("m1", "z2"), n_steps=4)
    theta = torch.tensor([0.4, 0.3, 0.0, 0.0, 0.6, 0.0, 0.0, -0.5], dtype=torch.float64, requires_grad=True)
    J = brill_lindquist_observable(theta, m)
    (2.0 * J).backward()
    _, g = m.value_and_gradient(*BASE)
    assert np.allclose(theta.grad.numpy()[[0, 7]], 2.0 * g, rtol=1e-14)
    assert np.all(theta.grad.numpy()[[1, 2, 3, 4, 5, 6]] == 0.0)


def test_rejects_unbuilt_configurations(cuda):
    import torch
    from nrpytutorial_gb300 import Evolution, _lib
    G, gp = grids("BSSN", "Spherical", (8, 6, 6), 4, ng=3, RMAX=4.0)
    ev = Evolution("BSSN", G, precision="fp64", device=cuda)
    Y = torch.zeros((48,) + tuple(G.shape), dtype=torch.float64, device=cuda)
    aux = torch.zeros((12,) + tuple(G.shape), dtype=torch.float64, device=cuda)
    assert ev.lib.BSSN_tangent_rhs_eval(ev._rfm(), C.byref(G.params), 1, _lib.ptr(Y), _lib.ptr(aux),
                                        _lib.ptr(torch.zeros_like(Y))) != 0
    assert ev.lib.BSSN_tangent_rhs_eval(ev._rfm(), C.byref(G.params), 3, _lib.ptr(Y), _lib.ptr(aux),
                                        _lib.ptr(torch.zeros_like(Y))) != 0
