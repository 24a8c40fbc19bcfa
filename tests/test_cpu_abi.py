"""CPU-only checks of the C-ABI library: it loads, exports every function
include/nrgpu.h declares, and its host-side routines (FD coefficients, grid
set-up, CFL timestep, argument validation) agree with the oracle.  No GPU
compute is called."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import oracle.grid as og
from oracle.fd import coeff_table
from tests.conftest import ROOT


def _lib():
    from nrpytutorial_gb300 import _lib as L
    if not os.path.exists(L.LIBPATH):
        from nrpytutorial_gb300 import build
        build.build()
    return L, L.load()


def header_functions():
    txt = open(os.path.join(ROOT, "include", "nrgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?(?:int|double|void|long long|char)\s*\*?\s*(\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    L, lib = _lib()
    names = header_functions()
    assert len(names) >= 35
    for n in names:
        assert hasattr(lib, n), "libnrgpu.so does not export %s" % n
    # and the Python binding declares a prototype for each one
    assert set(names) <= set(L.exported_symbols()), set(names) - set(L.exported_symbols())


@pytest.mark.parametrize("order", [2, 4, 6, 8])
def test_fd_coefficients_match_vandermonde(order):
    L, lib = _lib()
    ref = coeff_table(order)
    for kind in range(3):
        out = (C.c_double * (order + 1))()
        L.check(lib.nrgpu_fd_coeffs(order, kind, out))
        assert np.array_equal(np.array(list(out)), np.array(ref[kind])), (order, kind)


@pytest.mark.parametrize("order", [2, 4, 6, 8])
def test_kreiss_oliger_coefficients_match_oracle(order):
    from oracle.fd import ko_weights
    L, lib = _lib()
    out = (C.c_double * (order + 3))()
    L.check(lib.nrgpu_fd_coeffs(order, 3, out))
    offs, w = ko_weights(order)
    assert offs == list(range(-(order // 2 + 1), order // 2 + 2))
    assert np.array_equal(np.array(list(out)), np.array([float(x) for x in w])), order


@pytest.mark.parametrize("cs", ["Cartesian", "Spherical", "SinhSpherical", "SinhSphericalv2", "Cylindrical",
                                "SinhCylindrical", "SinhCylindricalv2", "SymTP", "SinhSymTP"])
def test_grid_setup_and_timestep_match_oracle(cs):
    from nrpytutorial_gb300 import Grid
    kw = dict(AMPL=64.0, SINHW=0.2, RMAX=10.0)
    G = Grid(cs, (16, 8, 4), FD_order=4, NGHOSTS=3, **kw)
    gp = og.GridParams(cs, (16, 8, 4), 3, 4, **kw)
    for d in range(3):
        assert np.array_equal(G.xx[d], gp.xx[d])
    assert G.find_timestep(0.5) == pytest.approx(og.find_timestep(gp, 0.5), rel=1e-15)
    p = G.params
    assert (p.Nxx_plus_2NGHOSTS0, p.Nxx_plus_2NGHOSTS1, p.Nxx_plus_2NGHOSTS2) == (22, 14, 10)
    assert p.dxx0 == gp.dxx[0] and p.invdx2 == gp.invdx[2]


def test_bad_arguments_return_status_not_abort():
    L, lib = _lib()
    from nrpytutorial_gb300 import Grid
    G = Grid("Cartesian", (8, 8, 8), FD_order=4, NGHOSTS=2)
    p = G.params
    bad = L.paramstruct.from_buffer_copy(p)
    bad.FD_order = 5
    st = lib.ScalarWave_rhs_eval(C.byref(bad), None, None)
    assert st != 0
    st = lib.ScalarWave_rhs_eval(C.byref(p), None, None)
    assert st == 1 and b"NULL" in lib.nrgpu_last_error()
    bad2 = L.paramstruct.from_buffer_copy(p)
    bad2.Nxx_plus_2NGHOSTS1 += 1
    assert lib.rfm_struct__malloc(C.byref(bad2), C.byref(L.rfm_struct())) == 1
    assert lib.nrgpu_fd_coeffs(3, 0, (C.c_double * 4)()) == 1
    assert lib.nrgpu_fd_coeffs(4, 4, (C.c_double * 7)()) == 1
    bad3 = L.paramstruct.from_buffer_copy(p)
    bad3.diss_strength = float("nan")
    assert lib.rfm_struct__malloc(C.byref(bad3), C.byref(L.rfm_struct())) == 1
    assert b"diss_strength" in lib.nrgpu_last_error()


def test_mode_decomposition_refuses_non_spherical_grids():
    """The s = -2 decomposition integrates over a spherical shell; Cartesian
    and Cylindrical-family grids get an argument error, before any device
    access."""
    L, lib = _lib()
    from nrpytutorial_gb300 import Grid
    buf = (C.c_double * 4)()
    for cs in ("Cartesian", "Cylindrical", "SinhCylindrical"):
        G = Grid(cs, (8, 8, 8), FD_order=4, NGHOSTS=3)
        st = lib.BSSN_psi4_spinweightm2_decomposition(C.byref(G.params), buf, 4, 2, buf)
        assert st == 1 and b"spherical" in lib.nrgpu_last_error(), cs


def test_batch_create_validates_before_touching_the_device():
    """Argument errors of the batched ScalarWave API are reported as status
    codes before any CUDA call (so they are checkable without a GPU)."""
    L, lib = _lib()
    h = C.c_void_p()
    nr = (C.c_int * 2)(16, 24)
    args = (32, 8, 0, 10.0, 10.0, 0.2, 1.0, 0.5, 1)
    assert lib.nrgpu_batch_create(2, nr, *args, C.byref(h)) == 1   # Cartesian is not supported
    assert b"Spherical" in lib.nrgpu_last_error()
    ok = (32, 8, 1, 10.0, 10.0, 0.2, 1.0, 0.5)
    assert lib.nrgpu_batch_create(0, nr, *ok, 1, C.byref(h)) == 1  # empty batch
    assert lib.nrgpu_batch_create(2, nr, *ok, 7, C.byref(h)) == 1  # unknown precision
    assert lib.nrgpu_batch_create(2, None, *ok, 1, C.byref(h)) == 1
    assert h.value is None
    assert lib.nrgpu_batch_set_tile(None, 32, 1, 1) == 1
    assert lib.nrgpu_batch_step(None, None) == 1
    assert lib.nrgpu_batch_total_points(None) == -1
    assert lib.nrgpu_batch_free(None) == 0


def test_oracle_mixed_derivative_is_product_of_first():
    from oracle.fd import Stencils
    gp = og.GridParams("Cartesian", (6, 6, 6), 2, 4)
    rng = np.random.default_rng(0)
    f = rng.standard_normal(gp.shape)
    S = Stencils(4, 2, gp.invdx)
    # d_x d_y f equals d_y applied to the x-derivative restricted consistently
    x = np.linspace(-1, 1, 10)
    X2, X1, X0 = np.meshgrid(x, x, x, indexing="ij")
    poly = X0 ** 2 * X1 ** 3 + X2 * X0
    S2 = Stencils(4, 3, [1 / (x[1] - x[0])] * 3)  # upwinded FD4 reaches 3 points
    d01 = S2.d11(poly, 0, 1)
    assert np.allclose(d01, (2 * X0 * 3 * X1 ** 2)[3:-3, 3:-3, 3:-3], atol=1e-10)
    assert np.allclose(S2.dup(poly, 2), X0[3:-3, 3:-3, 3:-3], atol=1e-12)
    assert np.allclose(S2.ddn(poly, 2), X0[3:-3, 3:-3, 3:-3], atol=1e-12)


def test_struct_layouts_match_the_c_header(tmp_path):
    """The ctypes mirrors of paramstruct, rfm_struct, bc_struct and
    MoL_gridfunctions have the C header's size and field offsets (a C
    program compiled against include/nrgpu.h prints them)."""
    import shutil
    import subprocess
    L, _ = _lib()
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    structs = {"paramstruct": L.paramstruct, "rfm_struct": L.rfm_struct}
    for name in ("bc_struct", "MoL_gridfunctions"):
        if hasattr(L, name):
            structs[name] = getattr(L, name)
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "nrgpu.h"', "int main(void) {"]
    for sname, cls in structs.items():
        lines.append('printf("%s sizeof %%zu\\n", sizeof(%s));' % (sname, sname))
        for f in cls._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (sname, f[0], sname, f[0]))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-I" + inc, str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        s, f, v = line.split()
        got[(s, f)] = int(v)
    for sname, cls in structs.items():
        assert got[(sname, "sizeof")] == C.sizeof(cls), sname
        for f in cls._fields_:
            assert got[(sname, f[0])] == getattr(cls, f[0]).offset, (sname, f[0])
