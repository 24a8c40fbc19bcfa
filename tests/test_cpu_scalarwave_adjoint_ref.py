"""CPU checks of the pieces the ScalarWave adjoint tests stand on: the
library's host xx_to_Cart (reference_metric.py:1397-1410) against the
oracle's coordinate maps, and the PyTorch-autograd reference
(tests/scalarwave_torch_ref.py) against the oracle's RK4 step, RHS and
boundary conditions on a curvilinear grid."""
import ctypes as C

import numpy as np
import pytest

import oracle.bcs as ob
import oracle.grid as og
import oracle.wave_maxwell as ow


def _cart_oracle(gp, i0, i1, i2):
    x0, x1, x2 = gp.xx[0][i0], gp.xx[1][i1], gp.xx[2][i2]
    if gp.CoordSystem == og.CART:
        return np.array([x0, x1, x2])
    if og.cylindrical(gp.CoordSystem):
        (rho, _), (z, _) = og.cylinder_maps(gp, x0, x2)
        return np.array([rho * np.cos(x1), rho * np.sin(x1), z])
    r = og.radial(gp.CoordSystem, x0, gp.AMPL, gp.SINHW, gp.const_dr)[0]
    return np.array([r * np.sin(x1) * np.cos(x2), r * np.sin(x1) * np.sin(x2), r * np.cos(x1)])


@pytest.mark.parametrize("coord", ["Cartesian", "Spherical", "SinhSpherical", "SinhSphericalv2", "Cylindrical",
                                   "SinhCylindrical", "SinhCylindricalv2"])
def test_xx_to_cart_matches_the_oracle(coord):
    from nrpytutorial_gb300 import Grid, _lib
    kw = dict(AMPL=6.0, SINHW=0.3) if "Spherical" in coord else {}
    G = Grid(coord, (8, 6, 10), FD_order=4, NGHOSTS=3, **kw)
    gp = og.GridParams(coord, (8, 6, 10), 3, 4, **kw)
    lib = _lib.load()
    x = (C.c_double * 3)()
    rng = np.random.default_rng(0)
    for _ in range(20):
        i = [int(rng.integers(0, n)) for n in gp.np]
        _lib.check(lib.xx_to_Cart(C.byref(G.params), None, i[0], i[1], i[2], x), "xx_to_Cart")
        want = _cart_oracle(gp, *i)
        assert np.allclose(np.array(x[:]), want, rtol=1e-14, atol=1e-14), (coord, i)
    # the caller's coordinate arrays are used when given
    arr = (C.POINTER(C.c_double) * 3)(*[np.ascontiguousarray(G.xx[d]).ctypes.data_as(C.POINTER(C.c_double))
                                        for d in range(3)])
    y = (C.c_double * 3)()
    _lib.check(lib.xx_to_Cart(C.byref(G.params), C.cast(arr, C.c_void_p), 1, 2, 3, y), "xx_to_Cart")
    _lib.check(lib.xx_to_Cart(C.byref(G.params), None, 1, 2, 3, x), "xx_to_Cart")
    assert np.allclose(np.array(x[:]), np.array(y[:]), rtol=1e-15, atol=0)
    assert lib.xx_to_Cart(C.byref(G.params), None, gp.np[0], 0, 0, x) != 0


@pytest.mark.parametrize("coord,kw", [("SinhSpherical", dict(AMPL=6.0, SINHW=0.3)),
                                      ("Spherical", dict(RMAX=4.0))])
def test_torch_reference_steps_like_the_oracle(coord, kw):
    torch = pytest.importorskip("torch")
    from tests.scalarwave_torch_ref import TorchScalarWave
    gp = og.GridParams(coord, (12, 8, 8), 3, 4, **kw)
    ng = gp.NGHOSTS
    w = np.ones(8 * 8)
    ref = TorchScalarWave(gp, ng + 5, w, n_steps=2)
    y0 = ref.initial_data(0.9, 1.2, 0.7).numpy()
    layers = ob.build_bcstruct(gp)

    def post(u):
        ob.apply_bcs(layers, u, [0, 0])

    yo = y0.copy()
    post(yo)
    yt = ref.bcs(torch.tensor(y0)).numpy()
    assert np.allclose(yt, yo, rtol=0, atol=1e-15)
    for _ in range(2):
        yo, _, _ = ob.rk4_step(yo, ref.dt, lambda u: ow.scalarwave_rhs_grid(gp, u), post, ng)
    yt = torch.tensor(yt)
    for _ in range(2):
        yt = ref.step(yt)
    scale = np.abs(yo).max()
    assert np.abs(yt.numpy() - yo).max() <= 1e-13 * scale
