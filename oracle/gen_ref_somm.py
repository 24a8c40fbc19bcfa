"""Generate the reference's Sommerfeld radiation boundary condition C into
oracle/_ref/src/somm_<coord>_dr<k>/ (gitignored).

TEST INFRASTRUCTURE (see oracle/__init__.py).  Needs the reference checkout
($NRPY_REFERENCE; run it in the container that has it):

    NRPY_REFERENCE=<checkout> python -m oracle.gen_ref_somm

For each configuration a fresh Python process imports the reference
read-only (no bytecode) and writes what its generator writes for a
Sommerfeld driver (Tutorial-Start_to_Finish-ScalarWaveCurvilinear.ipynb:350-355
with BoundaryCondition "QuadraticExtrapolation&Sommerfeld"): the ScalarWave
gridfunctions uu, vv; Set_up_CurviBoundaryConditions (bcstruct set-up, parity
dot products, eigen-coordinate maps; the static headers copied from the
checkout as that function copies them); sommerfeld_boundary_condition_class
(CurviBoundaryConditions.py:259-658) with the class defaults (value at
infinity 0, radial falloff power 3, speed 1) and the configuration's d_r FD
order, written by write_sommerfeld_file (:556-658: apply_bcs_sommerfeld and
contraction_term); the grid set-up and parameter struct.  A shim of ours
(shim.c) builds the bcstruct as the drivers' main() does and exposes
apply_bcs_sommerfeld to ctypes.  oracle/ref_build.py compiles it.
"""
import os
import shutil
import subprocess
import sys
import textwrap

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref", "src")
# name -> (CoordSystem, d_r FD order); ScalarWave, FD_CENTDERIVS_ORDER 4, NGHOSTS 2
CONFIGS = {"somm_sph_dr2": ("Spherical", 2), "somm_sph_dr4": ("Spherical", 4),
           "somm_sinhsph_dr2": ("SinhSpherical", 2), "somm_sinhsph_dr4": ("SinhSpherical", 4)}
NG = 2
STATIC_BC = ["apply_bcs_curvilinear.h", "BCs_data_structs.h", "bcstruct_freemem.h", "CurviBC_include_Cfunctions.h",
             "driver_bcstruct.h", "set_bcstruct.h", "set_up__bc_gz_map_and_parity_condns.h"]

WORKER = r'''
import os, sys
sys.dont_write_bytecode = True
REF, OUTDIR, COORD, DR = sys.argv[1], sys.argv[2], sys.argv[3], int(sys.argv[4])
sys.path.insert(0, REF)
os.chdir(OUTDIR)
import NRPy_param_funcs as par
import finite_difference as fin  # registers finite_difference::FD_CENTDERIVS_ORDER
import grid as gri
import reference_metric as rfm
par.set_parval_from_str("grid::DIM", 3)
par.set_parval_from_str("reference_metric::CoordSystem", COORD)
rfm.reference_metric()
par.set_parval_from_str("finite_difference::FD_CENTDERIVS_ORDER", 4)
gri.register_gridfunctions("EVOL", ["uu", "vv"])
rfm.set_Nxx_dxx_invdx_params__and__xx_h(OUTDIR)
import CurviBoundaryConditions.CurviBoundaryConditions as cbcs
cbcs.Set_up_CurviBoundaryConditions(os.path.join(OUTDIR, "boundary_conditions/"), verbose=False,
                                    Cparamspath=os.path.join("../"), enable_copy_of_static_Ccodes=False,
                                    BoundaryCondition="QuadraticExtrapolation&Sommerfeld")
bcs = cbcs.sommerfeld_boundary_condition_class(fd_order=DR, vars_at_inf_default=0.,
                                                vars_radial_falloff_power_default=3., vars_speed_default=1.)
bcs.write_sommerfeld_main_Ccode(OUTDIR)
par.generate_Cparameters_Ccodes(OUTDIR)
print("generated Sommerfeld", COORD, DR)
'''


def shim_source():
    return textwrap.dedent("""\
        /* shim.c -- the Sommerfeld drivers' bcstruct set-up and a ctypes entry
         * to the reference's generated apply_bcs_sommerfeld (generated by
         * oracle/gen_ref_somm.py; test infrastructure, never shipped). */
        #include <math.h>
        #include <stdint.h>
        #include <stdio.h>
        #include <stdlib.h>
        #include <string.h>
        #define NGHOSTS %(ng)d
        #define REAL double
        #ifndef M_PI
        #define M_PI 3.141592653589793238462643383279502884L
        #endif
        #include "declare_Cparameters_struct.h"
        #define IDX4S(g,i,j,k) ( (i) + Nxx_plus_2NGHOSTS0 * ( (j) + Nxx_plus_2NGHOSTS1 * ( (k) + Nxx_plus_2NGHOSTS2 * (g) ) ) )
        #define IDX4ptS(g,idx) ( (idx) + (Nxx_plus_2NGHOSTS0*Nxx_plus_2NGHOSTS1*Nxx_plus_2NGHOSTS2) * (g) )
        #define IDX3S(i,j,k) ( (i) + Nxx_plus_2NGHOSTS0 * ( (j) + Nxx_plus_2NGHOSTS1 * ( (k) ) ) )
        #define LOOP_REGION(i0min,i0max, i1min,i1max, i2min,i2max) \\
          for(int i2=i2min;i2<i2max;i2++) for(int i1=i1min;i1<i1max;i1++) for(int i0=i0min;i0<i0max;i0++)
        #include "boundary_conditions/gridfunction_defines.h"
        #include "set_Nxx_dxx_invdx_params__and__xx.h"
        #include "boundary_conditions/CurviBC_include_Cfunctions.h"

        static paramstruct params;
        static bc_struct bcstruct;
        static REAL *xx[3];

        int somm_setup(int N0, int N1, int N2, double AMPL, double SINHW, double RMAX) {
        #include "set_Cparameters_default.h"
          params.RMAX = RMAX;
        #ifdef HAVE_AMPL
          params.AMPL = AMPL; params.SINHW = SINHW;
        #else
          (void)AMPL; (void)SINHW;
        #endif
          const int Nxx[3] = {N0, N1, N2};
          {
            set_Nxx_dxx_invdx_params__and__xx(1, Nxx, &params, xx);
        #include "set_Cparameters-nopointer.h"
            const int Nxx_plus_2NGHOSTS_tot = Nxx_plus_2NGHOSTS0*Nxx_plus_2NGHOSTS1*Nxx_plus_2NGHOSTS2;
        #include "boundary_conditions/driver_bcstruct.h"
            for (int i = 0; i < 3; i++) free(xx[i]);
          }
          set_Nxx_dxx_invdx_params__and__xx(0, Nxx, &params, xx);
          return NUM_EVOL_GFS;
        }

        void somm_apply(const REAL *gfs, REAL *rhs) {
          apply_bcs_sommerfeld(&params, xx, &bcstruct, NUM_EVOL_GFS, evol_gf_parity, (REAL *)gfs, rhs);
        }
        int ref_nghosts(void) { return NGHOSTS; }
        """) % dict(ng=NG)


def generate(ref, name):
    coord, dr = CONFIGS[name]
    d = os.path.join(OUT, name)
    if os.path.isdir(d):
        shutil.rmtree(d)
    os.makedirs(os.path.join(d, "boundary_conditions"))
    src_bc = os.path.join(ref, "CurviBoundaryConditions", "boundary_conditions")
    for f in STATIC_BC:
        shutil.copy(os.path.join(src_bc, f), os.path.join(d, "boundary_conditions"))
    with open(os.path.join(d, "boundary_conditions", "CurviBC_include_Cfunctions.h"), "a") as f:
        f.write('\n#include "apply_bcs_sommerfeld.h"\n#include "apply_bcs_curvilinear.h"')
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1")
    r = subprocess.run([sys.executable, "-c", WORKER, ref, d, coord, str(dr)], capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError("%s: Sommerfeld codegen failed:\n%s" % (name, r.stderr[-4000:]))
    src = shim_source()
    if coord.startswith("Sinh"):
        src = "#define HAVE_AMPL 1\n" + src
    with open(os.path.join(d, "shim.c"), "w") as f:
        f.write(src)
    return d


if __name__ == "__main__":
    ref = os.environ.get("NRPY_REFERENCE")
    if not ref or not os.path.isdir(ref):
        raise SystemExit("set NRPY_REFERENCE to the reference checkout")
    for n in sys.argv[1:] or CONFIGS:
        print(generate(ref, n))
