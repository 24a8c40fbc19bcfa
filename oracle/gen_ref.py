"""Generate the reference's own C kernels into oracle/_ref/src/ (gitignored).

TEST INFRASTRUCTURE (see oracle/__init__.py).  Needs the reference checkout
($NRPY_REFERENCE, required); run it in the container that
has it:

    python -m oracle.gen_ref            # all configurations, in parallel
    python -m oracle.gen_ref bssn_sinhsph_fd4

For each configuration a fresh Python process imports the reference
read-only (no bytecode written), sets its NRPy parameters the way the
start-to-finish drivers do, and writes the C that its code generator emits:
  rhs_eval / Ricci_eval / enforce_detgammabar_constraint /
  Hamiltonian_constraint / initial_data (BSSN; the no-rfm-precompute,
  Read_xxs forms of Tutorial-Start_to_Finish-BSSNCurvilinear-Two_BHs_Collide-
  no_rfm_precompute.ipynb), rhs_eval with Kreiss-Oliger dissipation
  (BSSN_KO: the BSSN RHSs plus BaikalETK's diss_strength * f_dKOD * ReU
  terms), rhs_eval with T^{mu nu} source terms (BSSN_SRC: T4UU as auxevol
  gridfunctions after RbarDD), psi4_eval (BSSN_PSI4: psi_4 in the quasi-Kinnersley tetrad, six
  pieces), rhs_eval (ScalarWave, Maxwell System I, and MaxwellCurvi: System II
  rescaled on the reference metric),
  plus its declare_Cparameters_struct.h / set_Cparameters*.h /
  gridfunction_defines.h.
Nothing of the reference's source is copied: only what its generator prints.
A shim (shim.c, written here, ours) declares the few macros the generated
code expects and exports plain ctypes-callable wrappers.  oracle/ref_build.py
compiles each configuration into a strict FP64 oracle library and a timed
baseline library (the reference's own -Ofast -fopenmp flags).
"""
import os
import subprocess
import sys
import textwrap
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("NRPY_REFERENCE", "")
OUT = os.path.join(HERE, "_ref", "src")

# name -> (system, CoordSystem, FD order, NGHOSTS)
CONFIGS = {
    "bssn_sinhsph_fd4": ("BSSN", "SinhSpherical", 4, 3),
    "bssn_sph_fd4": ("BSSN", "Spherical", 4, 3),
    "bssn_sinhv2_fd4": ("BSSN", "SinhSphericalv2", 4, 3),
    "bssn_sinhcyl_fd4": ("BSSN", "SinhCylindrical", 4, 3),
    "bssn_sinhcylv2_fd4": ("BSSN", "SinhCylindricalv2", 4, 3),
    "bssn_sinhsymtp_fd4": ("BSSN", "SinhSymTP", 4, 3),
    "bssn_cart_fd4": ("BSSN", "Cartesian", 4, 3),
    "bssn_cart_fd6": ("BSSN", "Cartesian", 6, 4),
    "bssn_cart_fd2": ("BSSN", "Cartesian", 2, 2),
    "bssn_cart_fd8": ("BSSN", "Cartesian", 8, 5),
    "bssn_ko_sinhsph_fd4": ("BSSN_KO", "SinhSpherical", 4, 3),
    "bssn_ko_cart_fd6": ("BSSN_KO", "Cartesian", 6, 4),
    "bssn_ko_cart_fd2": ("BSSN_KO", "Cartesian", 2, 2),
    "bssn_ko_cart_fd8": ("BSSN_KO", "Cartesian", 8, 5),
    "bssn_src_sinhsph_fd4": ("BSSN_SRC", "SinhSpherical", 4, 3),
    "bssn_psi4_sph_fd4": ("BSSN_PSI4", "Spherical", 4, 3),
    "sw_cart_fd4": ("ScalarWave", "Cartesian", 4, 2),
    "sw_sinhsph_fd4": ("ScalarWave", "SinhSpherical", 4, 2),
    "maxwell_cart_fd4": ("Maxwell", "Cartesian", 4, 3),
    "maxwell_curvi_sinhsph_fd4": ("MaxwellCurvi", "SinhSpherical", 4, 3),
    "maxwell_curvi_sinhcyl_fd4": ("MaxwellCurvi", "SinhCylindrical", 4, 3),
    "sw_sinhcyl_fd4": ("ScalarWave", "SinhCylindrical", 4, 2),
}

WORKER = r'''
import os, sys
sys.dont_write_bytecode = True
REF, OUTDIR, SYSTEM, COORD, FD = sys.argv[1], sys.argv[2], sys.argv[3], sys.argv[4], int(sys.argv[5])
sys.path.insert(0, REF)
sys.path.insert(0, os.path.join(REF, "UnitTesting"))
os.chdir(OUTDIR)
from outputC import lhrh, outCfunction, outC_function_dict
import finite_difference as fin
import NRPy_param_funcs as par
import grid as gri
import reference_metric as rfm

par.set_parval_from_str("grid::DIM", 3)
par.set_parval_from_str("reference_metric::CoordSystem", COORD)
par.set_parval_from_str("reference_metric::enable_rfm_precompute", "False")
rfm.reference_metric()
par.set_parval_from_str("finite_difference::FD_CENTDERIVS_ORDER", FD)
par.set_parval_from_str("finite_difference::FD_functions_enable", False)

def emit(name, params, body, loopopts):
    txt = outCfunction(outfile="returnstring", desc="", name=name, params=params, body=body, loopopts=loopopts)
    with open(os.path.join(OUTDIR, name + ".h"), "w") as f:
        f.write(txt)

if SYSTEM in ("BSSN", "BSSN_KO", "BSSN_SRC"):
    KO = SYSTEM == "BSSN_KO"
    SRC = SYSTEM == "BSSN_SRC"
    if SYSTEM == "BSSN":
        import BSSN.BrillLindquist as bl
        bl.BrillLindquist()
        with open(os.path.join(OUTDIR, "initial_data.h"), "w") as f:
            f.write(outC_function_dict["initial_data"])
    import BSSN.BSSN_RHSs as rhs
    import BSSN.BSSN_gauge_RHSs as gaugerhs
    import BSSN.BSSN_quantities as Bq
    par.set_parval_from_str("BSSN.BSSN_gauge_RHSs::ShiftEvolutionOption", "GammaDriving2ndOrder_Covariant")
    par.set_parval_from_str("BSSN.BSSN_quantities::LeaveRicciSymbolic", "True")
    rhs.BSSN_RHSs()
    if SRC:
        # T^{mu nu} source terms added as BaikalETK_C_kernels_codegen.py:133-145
        # adds them: before the gauge RHSs, so B^i sees the Lambdabar source.
        import indexedexp as ixp
        import BSSN.BSSN_stress_energy_source_terms as Bsest
        T4UU = ixp.register_gridfunctions_for_single_rank2("AUXEVOL", "T4UU", "sym01", DIM=4)
        Bsest.BSSN_source_terms_for_BSSN_RHSs(T4UU)
        rhs.trK_rhs += Bsest.sourceterm_trK_rhs
        for i in range(3):
            rhs.Lambdabar_rhsU[i] += Bsest.sourceterm_Lambdabar_rhsU[i]
            rhs.lambda_rhsU[i] += Bsest.sourceterm_lambda_rhsU[i]
            for j in range(3):
                rhs.a_rhsDD[i][j] += Bsest.sourceterm_a_rhsDD[i][j]
    gaugerhs.BSSN_gauge_RHSs()
    Bq.BSSN_basic_tensors()
    betaU = Bq.betaU
    import BSSN.Enforce_Detgammabar_Constraint as EGC
    enf = EGC.Enforce_Detgammabar_Constraint_symb_expressions()
    par.set_parval_from_str("BSSN.BSSN_quantities::LeaveRicciSymbolic", "False")
    Bq.RicciBar__gammabarDD_dHatD__DGammaUDD__DGammaU()
    H = gri.register_gridfunctions("AUX", "H")
    import BSSN.BSSN_constraints as bssncon
    bssncon.BSSN_constraints(add_T4UUmunu_source_terms=False)
    rfm.ref_metric__hatted_quantities()
    lhs_names = ["alpha", "cf", "trK"]
    rhs_exprs = [gaugerhs.alpha_rhs, rhs.cf_rhs, rhs.trK_rhs]
    for i in range(3):
        lhs_names.append("betU" + str(i)); rhs_exprs.append(gaugerhs.bet_rhsU[i])
        lhs_names.append("lambdaU" + str(i)); rhs_exprs.append(rhs.lambda_rhsU[i])
        lhs_names.append("vetU" + str(i)); rhs_exprs.append(gaugerhs.vet_rhsU[i])
        for j in range(i, 3):
            lhs_names.append("aDD" + str(i) + str(j)); rhs_exprs.append(rhs.a_rhsDD[i][j])
            lhs_names.append("hDD" + str(i) + str(j)); rhs_exprs.append(rhs.h_rhsDD[i][j])
    if KO:
        # Kreiss-Oliger dissipation added to every evolved gridfunction's RHS
        # the way BaikalETK/BaikalETK_C_kernels_codegen.py:147-171 adds it
        # (diss_strength * sum_k f_dKOD[k] * ReU[k]; the 2nd-order shift
        # condition, so betU is dissipated too).
        import indexedexp as ixp
        diss = par.Cparameters("REAL", "KO_Dissipation", "diss_strength", 0.1)
        ko = {"alpha": ixp.declarerank1("alpha_dKOD"), "cf": ixp.declarerank1("cf_dKOD"),
              "trK": ixp.declarerank1("trK_dKOD")}
        for b in ("betU", "vetU", "lambdaU"):
            t = ixp.declarerank2(b + "_dKOD", "nosym")
            for i in range(3):
                ko[b + str(i)] = t[i]
        for b in ("aDD", "hDD"):
            t = ixp.declarerank3(b + "_dKOD", "sym01")
            for i in range(3):
                for j in range(i, 3):
                    ko[b + str(i) + str(j)] = t[i][j]
        rhs_exprs = [e + sum(diss * ko[n][k] * rfm.ReU[k] for k in range(3)) for n, e in zip(lhs_names, rhs_exprs)]
    lhs_names, rhs_exprs = [list(x) for x in zip(*sorted(zip(lhs_names, rhs_exprs), key=lambda p: p[0]))]
    ev = [lhrh(lhs=gri.gfaccess("rhs_gfs", n), rhs=e) for n, e in zip(lhs_names, rhs_exprs)]
    emit("rhs_eval",
         "const paramstruct *restrict params, REAL *restrict xx[3], const REAL *restrict auxevol_gfs, "
         "const REAL *restrict in_gfs, REAL *restrict rhs_gfs",
         fin.FD_outputC("returnstring", ev, params="outCverbose=False", upwindcontrolvec=betaU).replace("IDX4", "IDX4S"),
         "InteriorPoints,Read_xxs")
    if KO or SRC:
        par.generate_Cparameters_Ccodes(OUTDIR)
        gri.output__gridfunction_defines_h__return_gf_lists(OUTDIR)
        print("generated", SYSTEM, COORD, FD)
        sys.exit(0)
    R = Bq.RbarDD
    emit("Ricci_eval",
         "const paramstruct *restrict params, REAL *restrict xx[3], const REAL *restrict in_gfs, REAL *restrict auxevol_gfs",
         fin.FD_outputC("returnstring",
                        [lhrh(lhs=gri.gfaccess("auxevol_gfs", "RbarDD%d%d" % (i, j)), rhs=R[i][j])
                         for i in range(3) for j in range(i, 3)],
                        params="outCverbose=False").replace("IDX4", "IDX4S"),
         "InteriorPoints,Read_xxs")
    emit("Hamiltonian_constraint",
         "const paramstruct *restrict params, REAL *restrict xx[3], REAL *restrict in_gfs, REAL *restrict aux_gfs",
         fin.FD_outputC("returnstring", lhrh(lhs=gri.gfaccess("aux_gfs", "H"), rhs=bssncon.H),
                        params="outCverbose=False").replace("IDX4", "IDX4S"),
         "InteriorPoints,Read_xxs")
    EGC.output_Enforce_Detgammabar_Constraint_Ccode(OUTDIR, exprs=enf, Read_xxs=True)
elif SYSTEM == "BSSN_PSI4":
    # psi_4 with the quasi-Kinnersley tetrad, real and imaginary parts in the
    # reference's three pieces each, as the Two_BHs_Collide-Psi4 driver
    # generates them (one FD_outputC per piece, CSE_sorting=none).
    import BSSN.Psi4_tetrads as BP4t
    par.set_parval_from_str("BSSN.Psi4_tetrads::TetradChoice", "QuasiKinnersley")
    import BSSN.Psi4 as BP4
    BP4.Psi4()
    names = ["psi4r_0pt", "psi4r_1pt", "psi4r_2pt", "psi4i_0pt", "psi4i_1pt", "psi4i_2pt"]
    gri.register_gridfunctions("AUX", names)
    exprs = BP4.psi4_re_pt + BP4.psi4_im_pt
    body = ""
    for n, e in zip(names, exprs):
        body += "{\n" + fin.FD_outputC("returnstring", lhrh(lhs=gri.gfaccess("aux_gfs", n), rhs=e),
                                        params="outCverbose=False,CSE_sorting=none") + "}\n"
    emit("psi4_eval",
         "const paramstruct *restrict params, REAL *restrict xx[3], const REAL *restrict in_gfs, REAL *restrict aux_gfs",
         body.replace("IDX4", "IDX4S"), "InteriorPoints,Read_xxs")
elif SYSTEM == "ScalarWave":
    if COORD == "Cartesian":
        import ScalarWave.ScalarWave_RHSs as sw
        sw.ScalarWave_RHSs()
        uu_rhs, vv_rhs = sw.uu_rhs, sw.vv_rhs
        params = "const paramstruct *restrict params, REAL *restrict xx[3], const REAL *restrict in_gfs, REAL *restrict rhs_gfs"
    else:
        import ScalarWave.ScalarWaveCurvilinear_RHSs as sw
        sw.ScalarWaveCurvilinear_RHSs()
        uu_rhs, vv_rhs = sw.uu_rhs, sw.vv_rhs
        params = "const paramstruct *restrict params, REAL *restrict xx[3], const REAL *restrict in_gfs, REAL *restrict rhs_gfs"
    emit("rhs_eval", params,
         fin.FD_outputC("returnstring", [lhrh(lhs=gri.gfaccess("rhs_gfs", "uu"), rhs=uu_rhs),
                                         lhrh(lhs=gri.gfaccess("rhs_gfs", "vv"), rhs=vv_rhs)],
                        params="outCverbose=False").replace("IDX4", "IDX4S"),
         "InteriorPoints,Read_xxs")
elif SYSTEM == "MaxwellCurvi":
    # Tutorial-Start_to_Finish-Solving_Maxwells_Equations_in_Vacuum-Curvilinear:
    # System II in rescaled curvilinear form (no rfm precompute here).
    import Maxwell.InitialData  # registers Maxwell.InitialData::System_to_use
    par.set_parval_from_str("Maxwell.InitialData::System_to_use", "System_II")
    import Maxwell.VacuumMaxwell_Flat_Evol_Curvilinear_rescaled as mc
    mc.VacuumMaxwellRHSs_rescaled()
    names = ["aU0", "aU1", "aU2", "eU0", "eU1", "eU2", "psi", "Gamma"]
    exprs = mc.arhsU + mc.erhsU + [mc.psi_rhs, mc.Gamma_rhs]
    emit("rhs_eval",
         "const paramstruct *restrict params, REAL *restrict xx[3], const REAL *restrict in_gfs, REAL *restrict rhs_gfs",
         fin.FD_outputC("returnstring", [lhrh(lhs=gri.gfaccess("rhs_gfs", n), rhs=e) for n, e in zip(names, exprs)],
                        params="outCverbose=False").replace("IDX4", "IDX4S"),
         "InteriorPoints,Read_xxs")
elif SYSTEM == "Maxwell":
    import Maxwell.InitialData  # registers Maxwell.InitialData::System_to_use
    import Maxwell.VacuumMaxwell_Flat_Evol_Cartesian as mw
    par.set_parval_from_str("Maxwell.InitialData::System_to_use", "System_I")
    mw.VacuumMaxwellRHSs()
    names = ["AU0", "AU1", "AU2", "EU0", "EU1", "EU2", "psi"]
    exprs = [mw.ArhsU[0], mw.ArhsU[1], mw.ArhsU[2], mw.ErhsU[0], mw.ErhsU[1], mw.ErhsU[2], mw.psi_rhs]
    emit("rhs_eval",
         "const paramstruct *restrict params, REAL *restrict xx[3], const REAL *restrict in_gfs, REAL *restrict rhs_gfs",
         fin.FD_outputC("returnstring", [lhrh(lhs=gri.gfaccess("rhs_gfs", n), rhs=e) for n, e in zip(names, exprs)],
                        params="outCverbose=False").replace("IDX4", "IDX4S"),
         "InteriorPoints,Read_xxs")
par.generate_Cparameters_Ccodes(OUTDIR)
gri.output__gridfunction_defines_h__return_gf_lists(OUTDIR)
print("generated", SYSTEM, COORD, FD)
'''


def shim_source(system, ng, fields, funcs):
    """Our wrapper around the generated functions (ctypes-friendly)."""
    setters = "\n".join('  if (!strcmp(name, "%s")) { params_.%s = (%s)v; return 0; }' % (n, n, t)
                        for t, n in fields)
    wr = []
    if "rhs_eval" in funcs:
        if system.startswith("BSSN"):
            wr.append("void ref_rhs_eval(REAL *x0, REAL *x1, REAL *x2, const REAL *aux, const REAL *in, REAL *rhs)"
                      " { REAL *xx[3] = {x0, x1, x2}; rhs_eval(&params_, xx, aux, in, rhs); }")
        else:
            wr.append("void ref_rhs_eval(REAL *x0, REAL *x1, REAL *x2, const REAL *aux, const REAL *in, REAL *rhs)"
                      " { REAL *xx[3] = {x0, x1, x2}; (void)aux; rhs_eval(&params_, xx, in, rhs); }")
    if "Ricci_eval" in funcs:
        wr.append("void ref_Ricci_eval(REAL *x0, REAL *x1, REAL *x2, const REAL *in, REAL *aux)"
                  " { REAL *xx[3] = {x0, x1, x2}; Ricci_eval(&params_, xx, in, aux); }")
    if "Hamiltonian_constraint" in funcs:
        wr.append("void ref_Hamiltonian_constraint(REAL *x0, REAL *x1, REAL *x2, REAL *in, REAL *aux)"
                  " { REAL *xx[3] = {x0, x1, x2}; Hamiltonian_constraint(&params_, xx, in, aux); }")
    if "enforce_detgammabar_constraint" in funcs:
        wr.append("void ref_enforce_detgammabar_constraint(REAL *x0, REAL *x1, REAL *x2, REAL *in)"
                  " { REAL *xx[3] = {x0, x1, x2}; enforce_detgammabar_constraint(&params_, xx, in); }")
    if "psi4_eval" in funcs:
        wr.append("void ref_psi4_eval(REAL *x0, REAL *x1, REAL *x2, const REAL *in, REAL *aux)"
                  " { REAL *xx[3] = {x0, x1, x2}; psi4_eval(&params_, xx, in, aux); }")
    if "initial_data" in funcs:
        wr.append("void ref_initial_data(REAL *x0, REAL *x1, REAL *x2, REAL *in)"
                  " { REAL *xx[3] = {x0, x1, x2}; initial_data(&params_, xx, in); }")
    incs = "\n".join('#include "%s.h"' % f for f in funcs)
    return textwrap.dedent("""\
        /* shim.c -- wrapper around reference-generated kernels (generated by
         * oracle/gen_ref.py; test infrastructure, never shipped). */
        #include <math.h>
        #include <stdio.h>
        #include <stdlib.h>
        #include <string.h>
        #define REAL double
        #define NGHOSTS %(ng)d
        #ifndef M_PI
        #define M_PI 3.141592653589793238462643383279502884L
        #endif
        #ifndef M_SQRT1_2
        #define M_SQRT1_2 0.707106781186547524400844362104849039L
        #endif
        #define UPWIND_ALG(UpwindVecU) UpwindVecU > 0.0 ? 1.0 : 0.0
        #include "declare_Cparameters_struct.h"
        #include "gridfunction_defines.h"
        #define IDX4S(g,i,j,k) ( (i) + Nxx_plus_2NGHOSTS0 * ( (j) + Nxx_plus_2NGHOSTS1 * ( (k) + Nxx_plus_2NGHOSTS2 * (g) ) ) )
        #define IDX4ptS(g,idx) ( (idx) + (Nxx_plus_2NGHOSTS0*Nxx_plus_2NGHOSTS1*Nxx_plus_2NGHOSTS2) * (g) )
        #define IDX3S(i,j,k) ( (i) + Nxx_plus_2NGHOSTS0 * ( (j) + Nxx_plus_2NGHOSTS1 * ( (k) ) ) )
        static paramstruct params_;
        %(incs)s
        void ref_defaults(void) { paramstruct params;
        #include "set_Cparameters_default.h"
          params_ = params; }
        int ref_set(const char *name, double v) {
        %(setters)s
          return 1; }
        int ref_nghosts(void) { return NGHOSTS; }
        %(wr)s
        """) % dict(ng=ng, incs=incs, setters=setters, wr="\n".join(wr))


def parse_fields(path):
    fields = []
    for line in open(path):
        line = line.strip()
        if not line or line.startswith("typedef") or line.startswith("}"):
            continue
        decl = line.split(";")[0].split()
        if len(decl) == 2 and decl[0] in ("REAL", "int"):
            fields.append((decl[0] if decl[0] == "int" else "double", decl[1]))
    return fields


def generate(name):
    system, coord, fd, ng = CONFIGS[name]
    d = os.path.join(OUT, name)
    os.makedirs(d, exist_ok=True)
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1")
    r = subprocess.run([sys.executable, "-c", WORKER, REF, d, system, coord, str(fd)],
                       capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError("%s: reference codegen failed:\n%s" % (name, r.stderr[-4000:]))
    funcs = [f for f in ("rhs_eval", "Ricci_eval", "Hamiltonian_constraint", "enforce_detgammabar_constraint",
                         "initial_data", "psi4_eval") if os.path.exists(os.path.join(d, f + ".h"))]
    fields = parse_fields(os.path.join(d, "declare_Cparameters_struct.h"))
    with open(os.path.join(d, "shim.c"), "w") as f:
        f.write(shim_source(system, ng, fields, funcs))
    return name, funcs


def main(names):
    if not REF or not os.path.isdir(REF):
        raise SystemExit("set NRPY_REFERENCE to the reference checkout (now %r)" % REF)
    names = names or list(CONFIGS)
    with ThreadPoolExecutor(max_workers=min(8, len(names))) as ex:
        for name, funcs in ex.map(generate, names):
            print(name, funcs)


if __name__ == "__main__":
    main(sys.argv[1:])
