"""Writes the C conversion from a generated driver's paramstruct to the
library's, so a NRPy+/SENR driver that switches to libnrgpu copies no fields
by hand.

The reference generates its paramstruct per driver (NRPy_param_funcs.py:
216-304 writes declare_Cparameters_struct.h: every registered C parameter,
sorted by type and name) and keeps three things out of it that the library's
struct carries: the coordinate system, the finite-difference order and the
ghost-zone count (code-generation choices), and the uniform-coordinate domain
(set_Nxx_dxx_invdx_params__and__xx computes it into local arrays).  This tool
reads the generated header and writes `nrgpu_params_from_generated.h`:

    static inline int nrgpu_params_from_generated(const paramstruct *src,
        int CoordSystem, int FD_order, int NGHOSTS, nrgpu_paramstruct *dst);

which copies every field the two structs share by name (values of fields the
generated struct lacks keep the library's defaults, the reference's own
parameter defaults), then completes the grid fields with the library's
set_Nxx_dxx_invdx_params__and__xx from src's Nxx.  The driver includes, in
this order, its declare_Cparameters_struct.h, nrgpu.h with
NRGPU_PARAMSTRUCT defined as nrgpu_paramstruct, and the written header.

    python -m nrpytutorial_gb300.params_shim declare_Cparameters_struct.h > nrgpu_params_from_generated.h
"""
import re
import sys

# The library's defaults for fields a generated struct may lack: the
# reference's own defaults (reference_metric.py, BSSN_gauge_RHSs.py:233,
# ScalarWave/CommonParams.py:24).
DEFAULTS = {"AMPL": 10.0, "SINHW": 0.2, "RMAX": 10.0, "xmin": -10.0, "xmax": 10.0, "ymin": -10.0, "ymax": 10.0,
            "zmin": -10.0, "zmax": 10.0, "eta": 2.0, "wavespeed": 1.0, "const_dr": 0.0625, "RHOMAX": 10.0,
            "ZMIN": -10.0, "ZMAX": 10.0, "AMPLRHO": 10.0, "SINHWRHO": 0.2, "AMPLZ": 10.0, "SINHWZ": 0.2,
            "const_drho": 0.0625, "const_dz": 0.0625, "bScale": 0.5, "SINHWAA": 0.2, "AMAX": 10.0}
# set by the conversion itself, never copied
DERIVED = {"CoordSystem", "FD_order", "NGHOSTS", "Nxx_plus_2NGHOSTS0", "Nxx_plus_2NGHOSTS1", "Nxx_plus_2NGHOSTS2",
           "dxx0", "dxx1", "dxx2", "invdx0", "invdx1", "invdx2", "xxmin0", "xxmin1", "xxmin2", "xxmax0", "xxmax1",
           "xxmax2"}


def library_fields():
    from nrpytutorial_gb300._lib import paramstruct
    return [n for n, _ in paramstruct._fields_]


def generated_fields(text):
    """Field names of a generated declare_Cparameters_struct.h."""
    body = text[text.index("{") + 1:text.rindex("}")]
    names = []
    for line in body.splitlines():
        m = re.match(r"\s*(?:REAL|int|double|float|char)\s+(\w+)\s*(?:\[\d+\])?\s*;", line)
        if m:
            names.append(m.group(1))
    return names


def shim(text, source_name="declare_Cparameters_struct.h"):
    lib = library_fields()
    gen = set(generated_fields(text))
    shared = [n for n in lib if n in gen and n not in DERIVED]
    lines = ["/* nrgpu_params_from_generated.h -- written by nrpytutorial_gb300/params_shim.py",
             " * from %s: the library's paramstruct filled from a generated" % source_name,
             " * driver's.  Shared fields: %s. */" % ", ".join(shared),
             "#ifndef NRGPU_PARAMS_FROM_GENERATED_H", "#define NRGPU_PARAMS_FROM_GENERATED_H",
             "#include <string.h>",
             "static inline int nrgpu_params_from_generated(const paramstruct *src, int CoordSystem, int FD_order,",
             "                                              int NGHOSTS, NRGPU_PARAMSTRUCT *dst) {",
             "  memset(dst, 0, sizeof(*dst));"]
    for n, v in DEFAULTS.items():
        if n in lib:
            lines.append("  dst->%s = %r;" % (n, v))
    lines += ["  dst->CoordSystem = CoordSystem;", "  dst->FD_order = FD_order;", "  dst->NGHOSTS = NGHOSTS;"]
    for n in shared:
        lines.append("  dst->%s = src->%s;" % (n, n))
    lines += ["  const int Nxx[3] = {src->Nxx0, src->Nxx1, src->Nxx2};",
              "  return set_Nxx_dxx_invdx_params__and__xx(0, Nxx, dst, NULL);", "}", "#endif", ""]
    return "\n".join(lines)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: python -m nrpytutorial_gb300.params_shim declare_Cparameters_struct.h")
    sys.stdout.write(shim(open(sys.argv[1]).read(), sys.argv[1].split("/")[-1]))
