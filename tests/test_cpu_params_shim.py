"""The conversion from a generated driver's paramstruct to the library's
(nrpytutorial_gb300/params_shim.py), compiled as a driver would use it: a C
file includes the reference's generated declare_Cparameters_struct.h
(tests/golden/declare_Cparameters_struct_<config>.h, written by the reference's
NRPy_param_funcs.py:216-304), then nrgpu.h with NRGPU_PARAMSTRUCT renamed, then
the written conversion header; it fills the generated struct as a driver's
main() would and converts.  Every field of the result must equal the
library's own grid set-up for the same grid (nrpytutorial_gb300.Grid), with
no field copied by hand."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")
LIBDIR = os.path.join(ROOT, "nrpytutorial_gb300")

CASES = [
    # (fixture config, CoordSystem, FD order, NGHOSTS, Nxx, {generated field: value}, Grid keywords)
    # generated-struct values as a driver's set_Cparameters_default.h and free_parameters.h set them
    ("bssn_ship_sinhsph_fd4", "SinhSpherical", 4, 3, (128, 64, 16),
     {"AMPL": 64.0, "SINHW": 0.2, "RMAX": 10.0, "eta": 2.0},
     dict(AMPL=64.0, SINHW=0.2, eta=2.0)),
    ("bssn_cart_fd6", "Cartesian", 6, 4, (32, 24, 16),
     {"xmin": -3.0, "xmax": 3.0, "ymin": -2.0, "ymax": 2.0, "zmin": -1.5, "zmax": 1.5, "eta": 1.0},
     dict(domain=((-3.0, 3.0), (-2.0, 2.0), (-1.5, 1.5)), eta=1.0)),
]


@pytest.mark.parametrize("cfg,coord,fd,ng,Nxx,vals,gkw", CASES)
def test_generated_paramstruct_converts_to_library_paramstruct(tmp_path, cfg, coord, fd, ng, Nxx, vals, gkw):
    gcc = shutil.which("gcc")
    if not gcc or not os.path.exists(os.path.join(LIBDIR, "libnrgpu.so")):
        pytest.skip("needs gcc and the built libnrgpu.so")
    from nrpytutorial_gb300 import COORD, Grid, _lib
    from nrpytutorial_gb300.params_shim import generated_fields, shim
    decl = open(os.path.join(GOLD, "declare_Cparameters_struct_%s.h" % cfg)).read()
    assert set(vals) <= set(generated_fields(decl))
    (tmp_path / "declare_Cparameters_struct.h").write_text(decl)
    (tmp_path / "nrgpu_params_from_generated.h").write_text(shim(decl))
    sets = "\n".join("  src.%s = %r;" % (k, v) for k, v in vals.items())
    (tmp_path / "driver.c").write_text("""
#include <string.h>
#define REAL double
#include "declare_Cparameters_struct.h"
#define NRGPU_PARAMSTRUCT nrgpu_paramstruct
#include "nrgpu.h"
#include "nrgpu_params_from_generated.h"
int driver_params(int N0, int N1, int N2, nrgpu_paramstruct *out) {
  paramstruct src;
  memset(&src, 0, sizeof(src));
  src.Nxx0 = N0; src.Nxx1 = N1; src.Nxx2 = N2;
%s
  return nrgpu_params_from_generated(&src, %d, %d, %d, out);
}
""" % (sets, COORD[coord], fd, ng))
    so = tmp_path / "driver.so"
    r = subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"),
                        "-I", str(tmp_path), str(tmp_path / "driver.c"), "-o", str(so), "-L", LIBDIR, "-lnrgpu",
                        "-Wl,-rpath," + LIBDIR], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _lib.load()  # the library (and its CUDA runtime) first, as a driver links it
    drv = C.CDLL(str(so))
    out = _lib.paramstruct()
    assert drv.driver_params(*Nxx, C.byref(out)) == 0
    want = Grid(coord, Nxx, FD_order=fd, NGHOSTS=ng, **gkw).params
    for name, _ in _lib.paramstruct._fields_:
        assert getattr(out, name) == getattr(want, name), name
