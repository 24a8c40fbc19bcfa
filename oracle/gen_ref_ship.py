"""Generate the reference's BSSN evolution step in its shipping form into
oracle/_ref/src/bssn_ship_sinhsph_fd4/ (gitignored).

TEST INFRASTRUCTURE and CPU BASELINE (see oracle/__init__.py).  Needs the
reference checkout ($NRPY_REFERENCE; run it in the container that has it):

    NRPY_REFERENCE=<checkout> python -m oracle.gen_ref_ship

A fresh Python process imports the reference read-only (no bytecode) and
follows Tutorial-Start_to_Finish-BSSNCurvilinear-Two_BHs_Collide.ipynb's code
generation cells, so the C is what that driver compiles:
  * rfm_precompute on (cell 10, reference_metric.py:603-886): rfm_struct
    arrays f0_of_xx0 ... instead of transcendental functions in the loops;
  * SIMD_enable and FD_functions_enable on (cell 3): SIMD-intrinsic loops
    (on a host without AVX/SSE2, SIMD/SIMD_intrinsics.h maps them to scalar
    code) and finite_difference_functions.h;
  * Ricci_eval, rhs_eval (covariant 2nd-order Gamma-driver), the
    det(gammabar) rescale, Brill-Lindquist initial_data;
  * MoLtimestepping/RK_MoL.h from MoL_C_Code_Generation("RK4", ...) with the
    driver's RHS_string / post_RHS_string (Ricci_eval, rhs_eval;
    apply_bcs_curvilinear, enforce_detgammabar_constraint);
  * the curvilinear boundary conditions of Set_up_CurviBoundaryConditions
    (the static apply_bcs_curvilinear.h, set_bcstruct.h,
    set_up__bc_gz_map_and_parity_condns.h, driver_bcstruct.h ... copied from
    the checkout into the output directory as that function does, plus its
    generated parity dot products and eigen-coordinate maps).
Differences from the driver, each needed for the benchmark configuration:
no symmetry axis (the configuration evolves 16 phi points), eta and the
grid come from the caller, and a shim of ours (shim.c) holds the driver's
main() set-up and time-loop body as ctypes-callable functions.
oracle/ref_build.py compiles it like the other configurations (strict and
the reference's -Ofast -fopenmp -funroll-loops -march=native flags).
"""
import os
import shutil
import subprocess
import sys
import textwrap

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref", "src")
NAME = "bssn_ship_sinhsph_fd4"
COORD, FD, NG = "SinhSpherical", 4, 3

WORKER = r'''
import os, sys
sys.dont_write_bytecode = True
REF, OUTDIR, COORD, FD = sys.argv[1], sys.argv[2], sys.argv[3], int(sys.argv[4])
sys.path.insert(0, REF)
os.chdir(OUTDIR)
from outputC import lhrh, outCfunction, outC_function_dict
import finite_difference as fin
import NRPy_param_funcs as par
import grid as gri
import reference_metric as rfm

par.set_parval_from_str("grid::DIM", 3)
# cell 3: MoL step with the driver's RHS / post-RHS strings
import MoLtimestepping.C_Code_Generation as MoL
os.makedirs(os.path.join(OUTDIR, "MoLtimestepping"), exist_ok=True)
MoL.MoL_C_Code_Generation("RK4",
    RHS_string="""
Ricci_eval(&rfmstruct, &params, RK_INPUT_GFS, auxevol_gfs);
rhs_eval(&rfmstruct, &params, auxevol_gfs, RK_INPUT_GFS, RK_OUTPUT_GFS);""",
    post_RHS_string="""
apply_bcs_curvilinear(&params, &bcstruct, NUM_EVOL_GFS, evol_gf_parity, RK_OUTPUT_GFS);
enforce_detgammabar_constraint(&rfmstruct, &params,                     RK_OUTPUT_GFS);\n""",
    outdir=os.path.join(OUTDIR, "MoLtimestepping/"))
par.set_parval_from_str("reference_metric::CoordSystem", COORD)
rfm.reference_metric()
par.set_parval_from_str("finite_difference::FD_CENTDERIVS_ORDER", FD)
par.set_parval_from_str("finite_difference::FD_functions_enable", True)
SIMD_enable = True

# cell 8: Brill-Lindquist initial data
import BSSN.BrillLindquist as bl
bl.BrillLindquist()
with open(os.path.join(OUTDIR, "initial_data.h"), "w") as f:
    f.write(outC_function_dict["initial_data"])

# cell 10: BSSN RHSs, Ricci and the rescale with rfm_precompute
import BSSN.BSSN_RHSs as rhs
import BSSN.BSSN_gauge_RHSs as gaugerhs
par.set_parval_from_str("BSSN.BSSN_gauge_RHSs::ShiftEvolutionOption", "GammaDriving2ndOrder_Covariant")
os.makedirs(os.path.join(OUTDIR, "rfm_files"), exist_ok=True)
par.set_parval_from_str("reference_metric::enable_rfm_precompute", "True")
par.set_parval_from_str("reference_metric::rfm_precompute_Ccode_outdir", os.path.join(OUTDIR, "rfm_files/"))
import BSSN.BSSN_quantities as Bq
par.set_parval_from_str("BSSN.BSSN_quantities::LeaveRicciSymbolic", "True")
rhs.BSSN_RHSs()
gaugerhs.BSSN_gauge_RHSs()
Bq.BSSN_basic_tensors()
betaU = Bq.betaU
import BSSN.Enforce_Detgammabar_Constraint as EGC
enf = EGC.Enforce_Detgammabar_Constraint_symb_expressions()
par.set_parval_from_str("BSSN.BSSN_quantities::LeaveRicciSymbolic", "False")
Bq.RicciBar__gammabarDD_dHatD__DGammaUDD__DGammaU()
par.set_parval_from_str("reference_metric::enable_rfm_precompute", "False")
rfm.ref_metric__hatted_quantities()
includes = ["finite_difference_functions.h"]
lhs_names = ["alpha", "cf", "trK"]
rhs_exprs = [gaugerhs.alpha_rhs, rhs.cf_rhs, rhs.trK_rhs]
for i in range(3):
    lhs_names.append("betU" + str(i)); rhs_exprs.append(gaugerhs.bet_rhsU[i])
    lhs_names.append("lambdaU" + str(i)); rhs_exprs.append(rhs.lambda_rhsU[i])
    lhs_names.append("vetU" + str(i)); rhs_exprs.append(gaugerhs.vet_rhsU[i])
    for j in range(i, 3):
        lhs_names.append("aDD" + str(i) + str(j)); rhs_exprs.append(rhs.a_rhsDD[i][j])
        lhs_names.append("hDD" + str(i) + str(j)); rhs_exprs.append(rhs.h_rhsDD[i][j])
lhs_names, rhs_exprs = [list(x) for x in zip(*sorted(zip(lhs_names, rhs_exprs), key=lambda p: p[0]))]
outC_params = "outCverbose=False,SIMD_enable=True"
loopopts = "InteriorPoints,Enable_rfm_precompute,EnableSIMD"
outCfunction(outfile=os.path.join(OUTDIR, "rhs_eval.h"), includes=includes, desc="Evaluate the BSSN RHSs",
             name="rhs_eval",
             params="""rfm_struct *restrict rfmstruct,const paramstruct *restrict params,
                      const REAL *restrict auxevol_gfs,const REAL *restrict in_gfs,REAL *restrict rhs_gfs""",
             body=fin.FD_outputC("returnstring",
                                 [lhrh(lhs=gri.gfaccess("rhs_gfs", n), rhs=e) for n, e in zip(lhs_names, rhs_exprs)],
                                 params=outC_params, upwindcontrolvec=betaU).replace("IDX4", "IDX4S"),
             loopopts=loopopts)
outCfunction(outfile=os.path.join(OUTDIR, "Ricci_eval.h"), includes=includes, desc="Evaluate the Ricci tensor",
             name="Ricci_eval",
             params="""rfm_struct *restrict rfmstruct,const paramstruct *restrict params,
                      const REAL *restrict in_gfs,REAL *restrict auxevol_gfs""",
             body=fin.FD_outputC("returnstring",
                                 [lhrh(lhs=gri.gfaccess("auxevol_gfs", "RbarDD%d%d" % (i, j)), rhs=Bq.RbarDD[i][j])
                                  for i in range(3) for j in range(i, 3)],
                                 params=outC_params).replace("IDX4", "IDX4S"),
             loopopts=loopopts)
# cell 14: the rescale (rfm_precompute form)
EGC.output_Enforce_Detgammabar_Constraint_Ccode(OUTDIR, exprs=enf)
# cell 16: the FD functions the kernels call
fin.output_finite_difference_functions_h(path=OUTDIR)
# cell 18: grid set-up (it registers the eigen-coordinate parameters)
rfm.set_Nxx_dxx_invdx_params__and__xx_h(OUTDIR)
# cell 20: curvilinear boundary conditions (the static files are copied by
# the caller, as Set_up_CurviBoundaryConditions would copy them)
import CurviBoundaryConditions.CurviBoundaryConditions as cbcs
cbcs.Set_up_CurviBoundaryConditions(os.path.join(OUTDIR, "boundary_conditions/"), verbose=False,
                                    Cparamspath=os.path.join("../"), enable_copy_of_static_Ccodes=False)
# the parameter struct last, once every module has registered its parameters
# (the driver calls generate_Cparameters_Ccodes again after the grid set-up)
par.generate_Cparameters_Ccodes(OUTDIR)
print("generated shipping-form BSSN", COORD, FD)
'''

STATIC_BC = ["apply_bcs_curvilinear.h", "BCs_data_structs.h", "bcstruct_freemem.h", "CurviBC_include_Cfunctions.h",
             "driver_bcstruct.h", "set_bcstruct.h", "set_up__bc_gz_map_and_parity_condns.h"]


def shim_source():
    return textwrap.dedent("""\
        /* shim.c -- the Brill-Lindquist driver's main() set-up and time-loop
         * body as ctypes-callable functions around the reference's generated
         * shipping-form C (generated by oracle/gen_ref_ship.py; test
         * infrastructure and CPU baseline, never shipped). */
        #include <math.h>
        #include <stdint.h>
        #include <stdio.h>
        #include <stdlib.h>
        #include <string.h>
        #define NGHOSTS %(ng)d
        #define REAL double
        #include "rfm_files/rfm_struct__declare.h"
        #include "declare_Cparameters_struct.h"
        #include "SIMD/SIMD_intrinsics.h"
        #ifdef SIMD_IS_DISABLED
        #define UPWIND_ALG(UpwindVecU) UpwindVecU > 0.0 ? 1.0 : 0.0
        #endif
        #ifndef M_PI
        #define M_PI 3.141592653589793238462643383279502884L
        #endif
        #ifndef M_SQRT1_2
        #define M_SQRT1_2 0.707106781186547524400844362104849039L
        #endif
        #define wavespeed 1.0
        #define IDX4S(g,i,j,k) ( (i) + Nxx_plus_2NGHOSTS0 * ( (j) + Nxx_plus_2NGHOSTS1 * ( (k) + Nxx_plus_2NGHOSTS2 * (g) ) ) )
        #define IDX4ptS(g,idx) ( (idx) + (Nxx_plus_2NGHOSTS0*Nxx_plus_2NGHOSTS1*Nxx_plus_2NGHOSTS2) * (g) )
        #define IDX3S(i,j,k) ( (i) + Nxx_plus_2NGHOSTS0 * ( (j) + Nxx_plus_2NGHOSTS1 * ( (k) ) ) )
        #define LOOP_REGION(i0min,i0max, i1min,i1max, i2min,i2max) \\
          for(int i2=i2min;i2<i2max;i2++) for(int i1=i1min;i1<i1max;i1++) for(int i0=i0min;i0<i0max;i0++)
        #define LOOP_ALL_GFS_GPS(ii) _Pragma("omp parallel for") \\
          for(int (ii)=0;(ii)<Nxx_plus_2NGHOSTS_tot*NUM_EVOL_GFS;(ii)++)
        #include "boundary_conditions/gridfunction_defines.h"
        #include "set_Nxx_dxx_invdx_params__and__xx.h"
        #include "boundary_conditions/CurviBC_include_Cfunctions.h"
        #include "enforce_detgammabar_constraint.h"
        #include "Ricci_eval.h"
        #include "rhs_eval.h"
        #include "initial_data.h"

        static paramstruct params;
        static rfm_struct rfm_kept;  /* rfm_struct__malloc.h declares its own local rfmstruct */
        static bc_struct bcstruct;
        static REAL *xx[3];
        static REAL *y_n_gfs, *y_nplus1_running_total_gfs, *k_odd_gfs, *k_even_gfs, *auxevol_gfs;
        static long long ntot_;

        /* The driver's main() up to its time loop (Steps 0b-1b), with the
         * grid, eta and the two masses as arguments. */
        int ship_setup(int N0, int N1, int N2, double AMPL, double SINHW, double eta, double m1, double z1,
                       double m2, double z2) {
        #include "set_Cparameters_default.h"
          params.AMPL = AMPL; params.SINHW = SINHW; params.eta = eta;
          params.BH1_posn_x = 0.0; params.BH1_posn_y = 0.0; params.BH1_posn_z = z1; params.BH1_mass = m1;
          params.BH2_posn_x = 0.0; params.BH2_posn_y = 0.0; params.BH2_posn_z = z2; params.BH2_mass = m2;
          const int Nxx[3] = {N0, N1, N2};
          {
            int EigenCoord = 1;
            set_Nxx_dxx_invdx_params__and__xx(EigenCoord, Nxx, &params, xx);
        #include "set_Cparameters-nopointer.h"
            const int Nxx_plus_2NGHOSTS_tot = Nxx_plus_2NGHOSTS0*Nxx_plus_2NGHOSTS1*Nxx_plus_2NGHOSTS2;
        #include "boundary_conditions/driver_bcstruct.h"
            for (int i = 0; i < 3; i++) free(xx[i]);
          }
          set_Nxx_dxx_invdx_params__and__xx(0, Nxx, &params, xx);
          {
        #include "set_Cparameters-nopointer.h"
            const int Nxx_plus_2NGHOSTS_tot = Nxx_plus_2NGHOSTS0*Nxx_plus_2NGHOSTS1*Nxx_plus_2NGHOSTS2;
            ntot_ = Nxx_plus_2NGHOSTS_tot;
            const size_t n = sizeof(REAL) * NUM_EVOL_GFS * (size_t)Nxx_plus_2NGHOSTS_tot;
            y_n_gfs = (REAL *)malloc(n); y_nplus1_running_total_gfs = (REAL *)malloc(n);
            k_odd_gfs = (REAL *)malloc(n); k_even_gfs = (REAL *)malloc(n);
            auxevol_gfs = (REAL *)malloc(sizeof(REAL) * NUM_AUXEVOL_GFS * (size_t)Nxx_plus_2NGHOSTS_tot);
          }
                  {
        #include "set_Cparameters-nopointer.h"
        #include "rfm_files/rfm_struct__malloc.h"
        #include "rfm_files/rfm_struct__define.h"
            rfm_kept = rfmstruct;
          }
          rfm_struct rfmstruct = rfm_kept;
          initial_data(&params, xx, y_n_gfs);
          apply_bcs_curvilinear(&params, &bcstruct, NUM_EVOL_GFS, evol_gf_parity, y_n_gfs);
          enforce_detgammabar_constraint(&rfmstruct, &params, y_n_gfs);
          return NUM_EVOL_GFS;
        }

        /* One pass of the driver's time loop body: MoLtimestepping/RK_MoL.h. */
        void ship_step(double dt) {
          rfm_struct rfmstruct = rfm_kept;
        #include "set_Cparameters-nopointer.h"
          const int Nxx_plus_2NGHOSTS_tot = Nxx_plus_2NGHOSTS0*Nxx_plus_2NGHOSTS1*Nxx_plus_2NGHOSTS2;
        #include "MoLtimestepping/RK_MoL.h"
        }

        long long ship_ntot(void) { return ntot_; }
        void ship_get_state(REAL *out) { memcpy(out, y_n_gfs, sizeof(REAL) * NUM_EVOL_GFS * (size_t)ntot_); }
        void ship_set_state(const REAL *in) { memcpy(y_n_gfs, in, sizeof(REAL) * NUM_EVOL_GFS * (size_t)ntot_); }
        void ship_get_xx(REAL *x0, REAL *x1, REAL *x2) {
          memcpy(x0, xx[0], sizeof(REAL) * params.Nxx_plus_2NGHOSTS0);
          memcpy(x1, xx[1], sizeof(REAL) * params.Nxx_plus_2NGHOSTS1);
          memcpy(x2, xx[2], sizeof(REAL) * params.Nxx_plus_2NGHOSTS2);
        }
        int ref_nghosts(void) { return NGHOSTS; }
        """) % dict(ng=NG)


def generate(ref):
    d = os.path.join(OUT, NAME)
    if os.path.isdir(d):
        shutil.rmtree(d)
    os.makedirs(os.path.join(d, "boundary_conditions"))
    os.makedirs(os.path.join(d, "SIMD"))
    # what Set_up_CurviBoundaryConditions(enable_copy_of_static_Ccodes=True) and
    # the driver's cell 3 (SIMD_enable) copy into the C code directory
    src_bc = os.path.join(ref, "CurviBoundaryConditions", "boundary_conditions")
    for f in STATIC_BC:
        shutil.copy(os.path.join(src_bc, f), os.path.join(d, "boundary_conditions"))
    with open(os.path.join(d, "boundary_conditions", "CurviBC_include_Cfunctions.h"), "a") as f:
        f.write('\n#include "apply_bcs_curvilinear.h"')
    shutil.copy(os.path.join(ref, "SIMD", "SIMD_intrinsics.h"), os.path.join(d, "SIMD"))
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1")
    r = subprocess.run([sys.executable, "-c", WORKER, ref, d, COORD, str(FD)], capture_output=True, text=True,
                       env=env)
    if r.returncode != 0:
        raise RuntimeError("shipping-form codegen failed:\n%s" % r.stderr[-4000:])
    with open(os.path.join(d, "shim.c"), "w") as f:
        f.write(shim_source())
    return d


if __name__ == "__main__":
    ref = os.environ.get("NRPY_REFERENCE")
    if not ref or not os.path.isdir(ref):
        raise SystemExit("set NRPY_REFERENCE to the reference checkout")
    print(generate(ref))
