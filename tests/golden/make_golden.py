"""Regenerates the golden fixtures in tests/golden/ from the reference.

Run in a container that has the reference checkout ($NRPY_REFERENCE,
required) after `python -m oracle.gen_ref` and `python -m oracle.ref_build`:

    python tests/golden/make_golden.py
    python tests/golden/make_golden.py ref:bssn_cart_fd8     # one fixture

Writes:
  senr_bc_spherical_4x4x4.npz  the SENR curvilinear-BC golden file
      CurviBoundaryConditions/SENRout4x4x4-Spherical_NGHOSTS4oFD.txt as an
      int array [1000 points, 10 gridfunctions] (points in i0-fastest order).
  ref_<config>.npz  outputs of the reference-generated C (strict FP64 build)
      on seeded inputs (tests/helpers.py bssn_random_state / numpy
      default_rng): Ricci, rhs_eval, Hamiltonian at interior points,
      enforce_detgammabar_constraint (hDD at all points), Brill-Lindquist
      initial_data (interior points); rhs_eval for ScalarWave / Maxwell
      (System I Cartesian, System II curvilinear rescaled);
      for bssn_ko_*: rhs_eval with Kreiss-Oliger dissipation on seeded
      state and auxevol inputs; for bssn_psi4_*: the six pieces of psi_4;
      for bssn_src_*: rhs_eval with T^{mu nu} source terms (auxevol = 6
      RbarDD + 10 T4UU, seeded).
  ref_bssn_bl_spherical_axisym.npz  the reference's own BSSN validation
      run (Spherical 72x12x2 and 96x16x2, Brill-Lindquist, CFL 1, to
      t = 7.5) through the reference's generated kernels: the 72x12x2
      state and H of both runs at t_final (`evolve`).
  ref_sw_planewave_sinhsph.npz  the reference's curvilinear ScalarWave
      validation run (SinhSpherical 16x8x16 and 24x12x24, plane wave, CFL 1,
      to t = 7) through the reference's generated rhs_eval: the 16x8x16
      state and both runs' error norms at t_final (`evolve_sw`).
  ref_sw_config1.npz  configuration 1 (ScalarWave Cartesian 64^3 and 32^3,
      FD4, CFL 0.5, plane wave, 100 and 50 steps) through the reference's
      generated rhs_eval: central-midplane errors against the exact solution
      at t = 2.5, 5, 15.625 and 4096 sampled points of the final 64^3 state
      (`config1`).
  declare_Cparameters_struct_<config>.h  the reference's generated
      paramstruct declarations of bssn_ship_sinhsph_fd4 and bssn_cart_fd6
      (NRPy_param_funcs.py:216-304), for the params-shim test (`params`).
  ref_sommerfeld.npz  the reference's generated apply_bcs_sommerfeld
      (oracle/gen_ref_somm.py: ScalarWave on Spherical and SinhSpherical
      10x8x6 grids, d_r orders 2 and 4) applied to seeded gridfunctions and
      RHSs: the RHS after the boundary condition (`sommerfeld`).
  swsh_m2.json  the reference's generated spin-weight -2 spherical
      harmonics (C, l <= 8) at five (theta, phi) points.
  fd_coefficients.json  exact FD coefficients of
      finite_difference.compute_fdcoeffs_fdstencl (incl. Kreiss-Oliger).
  trusted_values.json  the reference's trusted-value unit tests for the
      hot-path expressions: md5-seeded symbol values (exactly as
      UnitTesting/cse_simplify_and_evaluate_sympy_expressions.py:53-67
      assigns them) and the 30-digit expected values from
      */tests/trusted_values_dict.py.
"""
import hashlib
import json
import os
import random
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
REF = os.environ.get("NRPY_REFERENCE", "")

KW = dict(AMPL=5.0, SINHW=0.3, RMAX=5.0, domain=(-2.0, 2.0), eta=2.0)
BL = dict(BH1_mass=0.5, BH1_posn_x=0.0, BH1_posn_y=0.0, BH1_posn_z=0.5,
          BH2_mass=0.5, BH2_posn_x=0.0, BH2_posn_y=0.0, BH2_posn_z=-0.5)
FIXTURE_GRIDS = {
    "bssn_cart_fd4": ("Cartesian", (6, 6, 6), 4, 3, 11),
    "bssn_cart_fd6": ("Cartesian", (6, 6, 6), 6, 4, 12),
    "bssn_sinhsph_fd4": ("SinhSpherical", (8, 6, 4), 4, 3, 13),
    "bssn_sph_fd4": ("Spherical", (8, 6, 4), 4, 3, 14),
    "sw_cart_fd4": ("Cartesian", (6, 6, 6), 4, 2, 15),
    "sw_sinhsph_fd4": ("SinhSpherical", (8, 6, 4), 4, 2, 16),
    "maxwell_cart_fd4": ("Cartesian", (6, 6, 6), 4, 3, 17),
    "bssn_ko_sinhsph_fd4": ("SinhSpherical", (8, 6, 4), 4, 3, 18),
    "bssn_ko_cart_fd6": ("Cartesian", (6, 6, 6), 6, 4, 19),
    "bssn_psi4_sph_fd4": ("Spherical", (8, 6, 4), 4, 3, 20),
    "bssn_src_sinhsph_fd4": ("SinhSpherical", (8, 6, 4), 4, 3, 21),
    "maxwell_curvi_sinhsph_fd4": ("SinhSpherical", (8, 6, 4), 4, 3, 22),
    "bssn_cart_fd2": ("Cartesian", (6, 6, 6), 2, 2, 23),
    "bssn_cart_fd8": ("Cartesian", (6, 6, 6), 8, 5, 24),
    "bssn_ko_cart_fd2": ("Cartesian", (6, 6, 6), 2, 2, 25),
    "bssn_ko_cart_fd8": ("Cartesian", (6, 6, 6), 8, 5, 26),
    "bssn_sinhv2_fd4": ("SinhSphericalv2", (8, 6, 4), 4, 3, 27),
    "bssn_sinhcyl_fd4": ("SinhCylindrical", (8, 6, 6), 4, 3, 28),
    "maxwell_curvi_sinhcyl_fd4": ("SinhCylindrical", (8, 6, 6), 4, 3, 29),
    "sw_sinhcyl_fd4": ("SinhCylindrical", (8, 6, 6), 4, 2, 30),
    "bssn_sinhcylv2_fd4": ("SinhCylindricalv2", (8, 6, 6), 4, 3, 31),
    "bssn_sinhsymtp_fd4": ("SinhSymTP", (8, 6, 4), 4, 3, 32),
}
KO_DISS_STRENGTH = 0.3


def senr_bc():
    path = os.path.join(REF, "CurviBoundaryConditions", "SENRout4x4x4-Spherical_NGHOSTS4oFD.txt")
    rows = []
    for line in open(path):
        left, right = line.split("|")
        rows.append([int(v) for v in right.split()])
    vals = np.array(rows, dtype=np.int32)
    np.savez_compressed(os.path.join(HERE, "senr_bc_spherical_4x4x4.npz"), values=vals)
    print("senr", vals.shape)


def ref_outputs(only=None):
    import oracle.grid as og
    from oracle.ref import RefKernels
    from tests.helpers import bssn_random_state
    cart = {"xmin": -2.0, "xmax": 2.0, "ymin": -2.0, "ymax": 2.0, "zmin": -2.0, "zmax": 2.0}
    for cfg, (cs, N, fd, ng, seed) in FIXTURE_GRIDS.items():
        if only and cfg not in only:
            continue
        gp = og.GridParams(cs, N, ng, fd, **KW)
        R = RefKernels(cfg, gp, "strict", extra=dict(cart, **BL))
        g = ng
        I = (slice(None), slice(g, -g), slice(g, -g), slice(g, -g))
        out = dict(seed=seed, Nxx=np.array(N), fd=fd, ng=ng)
        if cfg.startswith("bssn_psi4"):
            # psi_4 (quasi-Kinnersley tetrad) of a seeded state; the six
            # generated pieces are stored, re = pieces 3..5, im = 0..2
            f = bssn_random_state(gp.shape, seed=seed)
            _, parts = R.psi4(f)
            out["psi4_parts"] = parts[I]
        elif cfg.startswith("bssn_src"):
            # rhs_eval with T^{mu nu} source terms: auxevol = 6 RbarDD then
            # 10 T4UU (seeded; T4UU00 kept positive like an energy density)
            f = bssn_random_state(gp.shape, seed=seed)
            aux = 0.1 * np.random.default_rng(seed + 100).standard_normal((16,) + gp.shape)
            aux[6] = np.abs(aux[6])
            out["aux"] = aux
            out["rhs"] = R.rhs_eval(f, aux=aux)[I]
        elif cfg.startswith("bssn_ko"):
            # rhs_eval with Kreiss-Oliger dissipation; RbarDD is an input
            # (auxevol) of the generated rhs_eval, so any seeded values do.
            R = RefKernels(cfg, gp, "strict", extra=dict(cart, diss_strength=KO_DISS_STRENGTH))
            f = bssn_random_state(gp.shape, seed=seed)
            aux = 0.1 * np.random.default_rng(seed + 100).standard_normal((6,) + gp.shape)
            out["aux"] = aux
            out["diss_strength"] = KO_DISS_STRENGTH
            out["rhs"] = R.rhs_eval(f, aux=aux)[I]
        elif cfg.startswith("bssn"):
            f = bssn_random_state(gp.shape, seed=seed)
            ric = R.ricci(f)
            out["ricci"] = ric[I]
            out["rhs"] = R.rhs_eval(f, aux=ric)[I]
            out["hamiltonian"] = R.hamiltonian(f)[g:-g, g:-g, g:-g]
            out["enforce_hDD"] = R.enforce(f)[11:17]
            out["bl_id"] = R.initial_data((24,) + gp.shape)[I]
        else:
            ngf = 8 if cfg.startswith("maxwell_curvi") else 7 if cfg.startswith("maxwell") else 2
            f = np.random.default_rng(seed).standard_normal((ngf,) + gp.shape)
            out["rhs"] = R.rhs_eval(f)[I]
        np.savez_compressed(os.path.join(HERE, "ref_%s.npz" % cfg), **out)
        print(cfg, {k: getattr(v, "shape", v) for k, v in out.items()})


# The reference's own BSSN validation run (Tutorial-Start_to_Finish-
# BSSNCurvilinear-Two_BHs_Collide.ipynb:165-202, 739-741, 1037-1044, 1235-1251):
# Spherical, domain_size 7.5, FD4, RK4, CFL 1.0, Brill-Lindquist m = 0.5 at
# z = +-0.5, grids 72x12x2 and 96x16x2 evolved to t_final = domain_size.
EVOLVE = dict(RMAX=7.5, CFL=1.0, t_final=7.5, grids=((72, 12, 2), (96, 16, 2)))


def evolution():
    """ref_bssn_bl_spherical_axisym.npz: the reference's generated
    initial_data / Ricci_eval / rhs_eval / enforce_detgammabar_constraint /
    Hamiltonian_constraint (strict FP64 build of bssn_sph_fd4) driven through
    the RK4 step and the curvilinear BCs (oracle/bcs.py) for N_final =
    int(t_final/dt + 0.5) steps: the interior state and H of the 72x12x2 run
    and H of the 96x16x2 run at t_final."""
    import oracle.bcs as ob
    import oracle.bssn as obs
    import oracle.grid as og
    from oracle.ref import RefKernels
    out = {}
    for N in EVOLVE["grids"]:
        gp = og.GridParams("Spherical", N, 3, 4, RMAX=EVOLVE["RMAX"], eta=2.0)
        R = RefKernels("bssn_sph_fd4", gp, "strict", extra=dict(BL, eta=2.0))
        layers = ob.build_bcstruct(gp)
        par = [ob.parity_type(n) for n in obs.EVOL]

        def post(f):
            ob.apply_bcs(layers, f, par)
            f[:] = R.enforce(f)

        def rhs(f):
            return R.rhs_eval(f, aux=R.ricci(f))

        y = R.initial_data((24,) + gp.shape)
        post(y)
        dt = og.find_timestep(gp, EVOLVE["CFL"])
        n_final = int(EVOLVE["t_final"] / dt + 0.5)
        k_odd = k_even = None
        for _ in range(n_final):
            y, k_odd, k_even = ob.rk4_step(y, dt, rhs, post, gp.NGHOSTS, k_odd, k_even)
        g = gp.NGHOSTS
        tag = "%dx%dx%d" % N
        out["n_final_" + tag] = n_final
        out["dt_" + tag] = dt
        out["H_" + tag] = R.hamiltonian(y)[g:-g, g:-g, g:-g]
        if N == EVOLVE["grids"][0]:
            out["state_" + tag] = y[:, g:-g, g:-g, g:-g]
        print("evolved", tag, n_final, "steps, dt", dt)
    np.savez_compressed(os.path.join(HERE, "ref_bssn_bl_spherical_axisym.npz"), **out)


# The reference's curvilinear ScalarWave validation run (Tutorial-Start_to_
# Finish-ScalarWaveCurvilinear.ipynb:160-203, 641-648, 781-786): SinhSpherical
# with domain_size 10 and sinh_width 0.4, FD4, RK4, CFL 1.0, quadratic-
# extrapolation BCs, PlaneWave data (wavespeed 1, k = (1, 1, 1)), grids
# 16x8x16 and 24x12x24 evolved to t_final = 0.7 domain_size.
SW_EVOLVE = dict(AMPL=10.0, SINHW=0.4, CFL=1.0, t_final=7.0, grids=((16, 8, 16), (24, 12, 24)))


def evolution_scalarwave():
    """ref_sw_planewave_sinhsph.npz: the reference's generated rhs_eval
    (strict build of sw_sinhsph_fd4) driven through the RK4 step and the
    curvilinear BCs (oracle/bcs.py) from the PlaneWave data (oracle,
    pinned to the reference's trusted values) for N_final =
    int(t_final/dt + 0.5) steps: the 16x8x16 interior state at t_final and,
    for both grids, the notebook's error norm sqrt(mean (u - u_exact)^2)
    over interior points with r < 0.3 domain_size."""
    import oracle.bcs as ob
    import oracle.grid as og
    import oracle.wave_maxwell as ow
    from oracle.ref import RefKernels
    out = {}
    for N in SW_EVOLVE["grids"]:
        gp = og.GridParams("SinhSpherical", N, 2, 4, AMPL=SW_EVOLVE["AMPL"], SINHW=SW_EVOLVE["SINHW"])
        R = RefKernels("sw_sinhsph_fd4", gp, "strict", extra=dict(wavespeed=1.0))
        layers = ob.build_bcstruct(gp)
        y = ow.scalarwave_id_grid(gp, "PlaneWave", 0.0)
        dt = og.find_timestep(gp, SW_EVOLVE["CFL"])
        n_final = int(SW_EVOLVE["t_final"] / dt + 0.5)
        k_odd = k_even = None
        for _ in range(n_final):
            y, k_odd, k_even = ob.rk4_step(y, dt, R.rhs_eval, lambda f: ob.apply_bcs(layers, f, [0, 0]),
                                           gp.NGHOSTS, k_odd, k_even)
        g = gp.NGHOSTS
        tag = "%dx%dx%d" % N
        exact = ow.scalarwave_id_grid(gp, "PlaneWave", n_final * dt)
        X2, X1, X0 = np.meshgrid(gp.xx[2], gp.xx[1], gp.xx[0], indexing="ij")
        r = og.radial(gp.CoordSystem, X0, gp.AMPL, gp.SINHW)[0]
        m = np.zeros(gp.shape, dtype=bool)
        m[g:-g, g:-g, g:-g] = True
        m &= r < 0.3 * SW_EVOLVE["AMPL"]
        out["n_final_" + tag] = n_final
        out["dt_" + tag] = dt
        out["l2_error_" + tag] = float(np.sqrt(np.mean((y[0][m] - exact[0][m]) ** 2)))
        if N == SW_EVOLVE["grids"][0]:
            out["state_" + tag] = y[:, g:-g, g:-g, g:-g]
        print("evolved", tag, n_final, "steps, dt", dt, "L2 error", out["l2_error_" + tag])
    np.savez_compressed(os.path.join(HERE, "ref_sw_planewave_sinhsph.npz"), **out)


# Configuration 1: ScalarWave Cartesian [-10,10]^3, FD4, 2 ghosts, CFL 0.5,
# u = sin(k.x - |k| t), v = -|k| cos(k.x - |k| t), k = (2 pi/20)(1,1,1),
# quadratic-extrapolation outer BCs; 64^3 for 100 RK4 steps and 32^3 for 50
# (the same final time 15.625).  Errors against the exact solution are taken
# the way Tutorial-Start_to_Finish-ScalarWave.ipynb:514-520 takes them: on the
# central half of the z midplane.
C1 = dict(grids=((32, 32, 32), (64, 64, 64)), steps=(50, 100), times=(2.5, 5.0, 15.625), nsample=4096)


def c1_central(e, N, g):
    """|e| on the central half of the z midplane (the notebook's region)."""
    n = N + 2 * g
    lo, hi = int(n * 0.25) + 1, int(np.ceil(n * 0.75))
    return e[n // 2, lo:hi, lo:hi]


PARAM_CFGS = ("bssn_ship_sinhsph_fd4", "bssn_cart_fd6")


def params():
    """declare_Cparameters_struct_<cfg>.h: copies of the reference's generated
    paramstruct declarations (written by oracle/gen_ref*.py into oracle/_ref/src)."""
    import shutil
    for cfg in PARAM_CFGS:
        src = os.path.join(ROOT, "oracle", "_ref", "src", cfg, "declare_Cparameters_struct.h")
        shutil.copy(src, os.path.join(HERE, "declare_Cparameters_struct_%s.h" % cfg))


SOMM = {"somm_sph_dr2": ("Spherical", 2), "somm_sph_dr4": ("Spherical", 4),
        "somm_sinhsph_dr2": ("SinhSpherical", 2), "somm_sinhsph_dr4": ("SinhSpherical", 4)}
SOMM_GRID = dict(Nxx=(10, 8, 6), AMPL=5.0, SINHW=0.3, RMAX=5.0)


def somm_inputs(cfg, shape):
    from tests.helpers import sommerfeld_inputs
    return sommerfeld_inputs(SOMM[cfg], shape)


def sommerfeld():
    """ref_sommerfeld.npz: for each SOMM configuration, the RHS after the
    reference's generated apply_bcs_sommerfeld (strict build)."""
    import ctypes as C
    import oracle.grid as og
    from oracle.ref_build import LIB
    out = {}
    g = SOMM_GRID
    for cfg, (coord, dr) in SOMM.items():
        gp = og.GridParams(coord, g["Nxx"], 2, 4, AMPL=g["AMPL"], SINHW=g["SINHW"], RMAX=g["RMAX"])
        lib = C.CDLL(os.path.join(LIB, "%s.strict.so" % cfg))
        lib.somm_setup.argtypes = [C.c_int] * 3 + [C.c_double] * 3
        lib.somm_setup(*g["Nxx"], g["AMPL"], g["SINHW"], g["RMAX"])
        f, rhs = somm_inputs(cfg, gp.shape)
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
        lib.somm_apply(dp(f), dp(rhs))
        out[cfg] = rhs
    np.savez_compressed(os.path.join(HERE, "ref_sommerfeld.npz"), **out)


def config1():
    """ref_sw_config1.npz: the reference's generated ScalarWave rhs_eval
    (strict build of sw_cart_fd4) through the oracle's RK4 step and face
    extrapolation: for both grids the central-midplane max error against the
    exact solution at the C1 times, and for 64^3 the final state at 4096
    seeded interior sample points."""
    import oracle.bcs as ob
    import oracle.grid as og
    import oracle.wave_maxwell as ow
    from oracle.ref import RefKernels
    out = {}
    for N, nsteps in zip(C1["grids"], C1["steps"]):
        gp = og.GridParams("Cartesian", N, 2, 4)
        R = RefKernels("sw_cart_fd4", gp, "strict", extra=dict(wavespeed=1.0))
        layers = ob.build_bcstruct(gp)
        y = ow.plane_wave(gp, 0.0)
        dt = 0.5 * gp.dxx[0]
        tag = "%d" % N[0]
        k_odd = k_even = None
        for s in range(1, nsteps + 1):
            y, k_odd, k_even = ob.rk4_step(y, dt, R.rhs_eval, lambda f: ob.apply_bcs(layers, f, [0, 0]),
                                           gp.NGHOSTS, k_odd, k_even)
            for t in C1["times"]:
                if abs(s * dt - t) < 1e-9:
                    ex = ow.plane_wave(gp, s * dt)
                    out["err_%s_t%g" % (tag, t)] = float(c1_central(np.abs(y[0] - ex[0]), N[0], 2).max())
        out["dt_" + tag] = dt
        if N[0] == 64:
            rng = np.random.default_rng(C1["nsample"])
            g = gp.NGHOSTS
            idx = np.stack([rng.integers(g, g + N[d], C1["nsample"]) for d in (2, 1, 0)], axis=1)
            out["sample_idx"] = idx
            out["sample_state"] = y[:, idx[:, 0], idx[:, 1], idx[:, 2]]
        print("config 1", tag, {k: v for k, v in out.items() if k.startswith("err_" + tag)})
    np.savez_compressed(os.path.join(HERE, "ref_sw_config1.npz"), **out)


FD_WORKER = r'''
import sys, json
sys.dont_write_bytecode = True
sys.path.insert(0, sys.argv[1])
import NRPy_param_funcs as par
import finite_difference as fin
out = {}
for order in (2, 4, 6, 8):
    par.set_parval_from_str("finite_difference::FD_CENTDERIVS_ORDER", order)
    for op in ("dD0", "dDD00", "dupD0", "ddnD0", "dKOD0"):
        c, st = fin.compute_fdcoeffs_fdstencl(op)
        out["%d_%s" % (order, op.rstrip("0"))] = {"offsets": [s[0] for s in st], "coeffs": [str(x) for x in c]}
print(json.dumps(out))
'''


def fd_coeffs():
    """fd_coefficients.json: finite_difference.compute_fdcoeffs_fdstencl's
    exact coefficients and offsets (first, second, up/downwinded and
    Kreiss-Oliger derivatives along x0) at FD orders 2, 4, 6, 8."""
    r = subprocess.run([sys.executable, "-c", FD_WORKER, REF], capture_output=True, text=True,
                       env=dict(os.environ, PYTHONDONTWRITEBYTECODE="1"), cwd="/tmp")
    if r.returncode != 0:
        raise RuntimeError(r.stderr[-3000:])
    res = json.loads(r.stdout.strip().splitlines()[-1])
    with open(os.path.join(HERE, "fd_coefficients.json"), "w") as f:
        json.dump(res, f, indent=0, sort_keys=True)
    print("fd coefficients", len(res))


SWSH_WORKER = r'''
import os, sys
sys.dont_write_bytecode = True
sys.path.insert(0, sys.argv[1])
os.chdir(sys.argv[2])
import SpinWeight_minus2_SphHarmonics.SpinWeight_minus2_SphHarmonics as S
S.SpinWeight_minus2_SphHarmonics(maximum_l=8, filename=os.path.join(sys.argv[2], "swsh.h"))
'''

SWSH_MAIN = r"""
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#define REAL double
#include "swsh.h"
int main(void) {
  const double th[5] = {0.05, 0.7, 1.5707963267948966, 2.2, 3.1};
  const double ph[5] = {-3.0, -0.4, 0.0, 1.3, 2.9};
  for (int l = 0; l <= 8; l++)
    for (int m = -l; m <= l; m++)
      for (int p = 0; p < 5; p++) {
        double re, im;
        SpinWeight_minus2_SphHarmonics(l, m, th[p], ph[p], &re, &im);
        printf("%d %d %.17g %.17g %.17g %.17g\n", l, m, th[p], ph[p], re, im);
      }
  return 0;
}
"""


def swsh():
    """swsh_m2.json: the reference-generated C of
    SpinWeight_minus2_SphHarmonics (l <= 8, s = -2) evaluated at five
    (theta, phi) points for every (l, m)."""
    import tempfile
    d = tempfile.mkdtemp()
    r = subprocess.run([sys.executable, "-c", SWSH_WORKER, REF, d], capture_output=True, text=True,
                       env=dict(os.environ, PYTHONDONTWRITEBYTECODE="1"))
    if r.returncode != 0:
        raise RuntimeError(r.stderr[-3000:])
    with open(os.path.join(d, "main.c"), "w") as f:
        f.write(SWSH_MAIN)
    exe = os.path.join(d, "swsh")
    subprocess.run(["gcc", "-O2", "-fno-fast-math", "-I" + d, os.path.join(d, "main.c"), "-o", exe, "-lm"],
                   check=True)
    rows = [ln.split() for ln in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
            if ln.strip()]
    out = [[int(a[0]), int(a[1])] + [float(x) for x in a[2:]] for a in rows]
    with open(os.path.join(HERE, "swsh_m2.json"), "w") as f:
        json.dump(out, f)
    print("swsh", len(out))


# ------------------------------------------------------------ trusted values
TRUSTED = [
    # (name, module-relative trusted dict file, dict key, init code, call, globals)
    ("BSSN_RHSs", "BSSN", "BSSN_RHSs__BSSN_RHSs__globals",
     "import BSSN.BSSN_RHSs as M", "M.BSSN_RHSs()", ["cf_rhs", "trK_rhs", "lambda_rhsU", "a_rhsDD", "h_rhsDD"]),
    ("gauge_RHSs", "BSSN", "gauge_RHSs__BSSN_gauge_RHSs__globals",
     "import BSSN.BSSN_RHSs as rhs\nrhs.BSSN_RHSs()\nimport BSSN.BSSN_gauge_RHSs as M", "M.BSSN_gauge_RHSs()",
     ["alpha_rhs", "bet_rhsU", "vet_rhsU"]),
    ("Ricci", "BSSN", "BSSN_quantities__RicciBar__gammabarDD_dHatD__DGammaUDD__DGammaU__globals",
     "import reference_metric as rfm\nrfm.reference_metric()\nrfm.ref_metric__hatted_quantities()\n"
     "import BSSN.BSSN_quantities as M", "M.RicciBar__gammabarDD_dHatD__DGammaUDD__DGammaU()",
     ["RbarDD", "DGammaU"]),
    ("constraints", "BSSN", "BSSN_constraints__BSSN_constraints__globals",
     "import BSSN.BSSN_constraints as M", "M.BSSN_constraints()", ["H", "MU"]),
    ("SW_ID_PlaneWave", "ScalarWave", "InitialData__InitialData__Type__PlaneWave___globals",
     "import ScalarWave.InitialData as M", 'M.InitialData(Type="PlaneWave")', ["uu_ID", "vv_ID"]),
    ("SW_ID_SphericalGaussian", "ScalarWave", "InitialData__InitialData__Type__SphericalGaussian___globals",
     "import ScalarWave.InitialData as M", 'M.InitialData(Type="SphericalGaussian")', ["uu_ID", "vv_ID"]),
    ("ScalarWave_RHSs", "ScalarWave", "ScalarWave_RHSs__ScalarWave_RHSs__globals",
     "import ScalarWave.ScalarWave_RHSs as M", "M.ScalarWave_RHSs()", ["uu_rhs", "vv_rhs"]),
    ("ScalarWaveCurvilinear_RHSs", "ScalarWave", "ScalarWaveCurvilinear_RHSs__ScalarWaveCurvilinear_RHSs__globals",
     "import ScalarWave.ScalarWaveCurvilinear_RHSs as M", "M.ScalarWaveCurvilinear_RHSs()", ["uu_rhs", "vv_rhs"]),
    ("Maxwell_I", "Maxwell", "VacuumMaxwell_Flat_Evol_Cartesian_System_I__VacuumMaxwellRHSs__globals",
     "import NRPy_param_funcs as par\n"
     "par.initialize_param(par.glb_param('char', 'Maxwell.InitialData','System_to_use','System_I'))\n"
     "import Maxwell.VacuumMaxwell_Flat_Evol_Cartesian as M", "M.VacuumMaxwellRHSs()",
     ["ArhsU", "ErhsU", "C", "psi_rhs"]),
]
TRUSTED += [
    ("Psi4", "BSSN", "Psi4__Psi4__specify_tetrad_False__globals",
     "import BSSN.Psi4 as M", "M.Psi4(specify_tetrad=False)", ["psi4_re_pt", "psi4_im_pt"]),
    ("Psi4_tetrads", "BSSN", "Psi4_tetrads__Psi4_tetrads__globals",
     "import BSSN.Psi4_tetrads as M", "M.Psi4_tetrads()", ["l4U", "n4U", "mre4U", "mim4U"]),
]
TRUSTED += [
    ("Maxwell_Curvi", "Maxwell", "MWEvol_Curvi__VacuumMaxwellRHSs_rescaled__globals",
     "import NRPy_param_funcs as par\n"
     "par.initialize_param(par.glb_param('char', 'Maxwell.InitialData','System_to_use','System_II'))\n"
     "import Maxwell.VacuumMaxwell_Flat_Evol_Curvilinear_rescaled as M", "M.VacuumMaxwellRHSs_rescaled()",
     ["erhsU", "arhsU", "psi_rhs", "Gamma_rhs", "C", "G", "EU_Cart", "AU_Cart"]),
]
_RFM_INIT = ("import BSSN.BSSN_quantities as Bq\nimport reference_metric as rfm\nrfm.reference_metric()\n"
             "rfm.ref_metric__hatted_quantities()\nimport BSSN.BSSN_stress_energy_source_terms as M")
TRUSTED += [
    ("Tmunu_BSSN", "BSSN",
     "BSSN_stress_energy_source_terms__stress_energy_source_terms_ito_T4UU_and_ADM_or_BSSN_metricvars___BSSN___globals",
     _RFM_INIT, 'M.stress_energy_source_terms_ito_T4UU_and_ADM_or_BSSN_metricvars("BSSN")',
     ["SDD", "SD", "S", "rho"]),
    ("Tmunu_RHS_sources", "BSSN", "BSSN_stress_energy_source_terms__BSSN_source_terms_for_BSSN_RHSs__globals",
     _RFM_INIT, "M.BSSN_source_terms_for_BSSN_RHSs()",
     ["sourceterm_trK_rhs", "sourceterm_a_rhsDD", "sourceterm_lambda_rhsU", "sourceterm_Lambdabar_rhsU"]),
]
for cs in ("Spherical", "SinhSpherical", "SinhSphericalv2", "Cylindrical", "SinhCylindrical", "SinhCylindricalv2",
           "SymTP", "SinhSymTP", "Cartesian"):
    TRUSTED.append(("rfm_" + cs, "tests", "rfm_%s__reference_metric__True__globals" % cs,
                    "import NRPy_param_funcs as par\n"
                    "import reference_metric as M\n"
                    "par.set_parval_from_str('reference_metric::CoordSystem', '%s')" % cs, "M.reference_metric(True)",
                    ["ReU", "ReDD", "ghatDD", "ghatUU", "detgammahat", "detgammahatdD", "detgammahatdDD",
                     "ReUdD", "ReUdDD", "ReDDdD", "ReDDdDD", "ghatDDdD", "ghatDDdDD", "GammahatUDD",
                     "GammahatUDDdD"]))

WORKER = r'''
import sys, json, hashlib, random
sys.dont_write_bytecode = True
REF = sys.argv[1]
sys.path.insert(0, REF); sys.path.insert(0, REF + "/UnitTesting")
spec = json.loads(sys.argv[2])
exec(spec["init"])
exec(spec["call"])
import sympy as sp
exprs = {}
def expand(name, obj, idx=""):
    if isinstance(obj, list):
        for i, o in enumerate(obj):
            expand(name, o, idx + "[%d]" % i)
    else:
        exprs[name + idx] = sp.sympify(obj)
for g in spec["globals"]:
    expand(g, getattr(M, g))
syms = set()
for e in exprs.values():
    syms |= e.free_symbols
vals = {}
for s in syms:
    n = str(s)
    if n == "M_PI" or n == "M_SQRT1_2":
        continue
    random.seed(int(hashlib.md5(n.encode()).hexdigest(), 16))
    vals[n] = random.random()
print(json.dumps({"inputs": vals, "names": sorted(exprs)}))
'''


def trusted(only=None):
    import importlib.util
    path_json = os.path.join(HERE, "trusted_values.json")
    out = json.load(open(path_json)) if only and os.path.exists(path_json) else {}
    for name, mod, key, init, call, globs in TRUSTED:
        if only and name not in only:
            continue
        spec = json.dumps({"init": init, "call": call, "globals": globs})
        r = subprocess.run([sys.executable, "-c", WORKER, REF, spec], capture_output=True, text=True,
                           env=dict(os.environ, PYTHONDONTWRITEBYTECODE="1"), cwd="/tmp")
        if r.returncode != 0:
            raise RuntimeError("%s: %s" % (name, r.stderr[-3000:]))
        res = json.loads(r.stdout.strip().splitlines()[-1])
        path = os.path.join(REF, mod, "tests", "trusted_values_dict.py") if mod != "tests" else \
            os.path.join(REF, "tests", "trusted_values_dict.py")
        sp_ = importlib.util.spec_from_file_location("tvd_" + name, path)
        sys.path.insert(0, REF)
        m = importlib.util.module_from_spec(sp_)
        sp_.loader.exec_module(m)
        tv = m.trusted_values_dict[key]
        expected = {k: str(v) for k, v in tv.items() if k in res["names"]}
        out[name] = {"key": key, "inputs": res["inputs"], "expected": expected}
        print(name, len(res["inputs"]), "symbols,", len(expected), "values")
    with open(os.path.join(HERE, "trusted_values.json"), "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)


if __name__ == "__main__":
    if not REF or not os.path.isdir(REF):
        raise SystemExit("set NRPY_REFERENCE to the reference checkout")
    what = sys.argv[1:] or ["senr", "ref", "fd", "swsh", "trusted", "evolve", "evolve_sw"]
    if "senr" in what:
        senr_bc()
    if "ref" in what:
        ref_outputs()
    if "fd" in what:
        fd_coeffs()
    if "swsh" in what:
        swsh()
    if "trusted" in what:
        trusted()
    if "evolve" in what:
        evolution()
    if "evolve_sw" in what:
        evolution_scalarwave()
    if "config1" in what:
        config1()
    if "params" in what:
        params()
    if "sommerfeld" in what:
        sommerfeld()
    names = [w[len("trusted:"):] for w in what if w.startswith("trusted:")]
    if names:
        trusted(names)
    cfgs = [w[len("ref:"):] for w in what if w.startswith("ref:")]
    if cfgs:
        ref_outputs(cfgs)
