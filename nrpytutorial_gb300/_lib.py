"""ctypes binding of libnrgpu.so (the C ABI declared in include/nrgpu.h).

The library is the only compute path: if it is missing, importing the
binding raises, and there is no CPU fallback.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libnrgpu.so")

COORD = {"Cartesian": 0, "Spherical": 1, "SinhSpherical": 2, "SinhSphericalv2": 3, "Cylindrical": 4,
         "SinhCylindrical": 5, "SinhCylindricalv2": 6, "SymTP": 7, "SinhSymTP": 8}
SYSTEM = {"ScalarWave": 0, "Maxwell": 1, "BSSN": 2, "MaxwellCurvilinear": 3}
PREC = {"fp64": 0, "mixed": 1, "compensated": 2, "compensated_fp64rk": 3}
BSSN_KERNELS = {"auto": 0, "point": 1, "staged": 2, "fused": 3}
MAX_GHOSTS = 8
MAX_BC_LEVELS = 32


class NrgpuError(RuntimeError):
    pass


class paramstruct(C.Structure):
    _fields_ = [
        ("CoordSystem", C.c_int), ("FD_order", C.c_int), ("NGHOSTS", C.c_int),
        ("Nxx0", C.c_int), ("Nxx1", C.c_int), ("Nxx2", C.c_int),
        ("Nxx_plus_2NGHOSTS0", C.c_int), ("Nxx_plus_2NGHOSTS1", C.c_int), ("Nxx_plus_2NGHOSTS2", C.c_int),
        ("dxx0", C.c_double), ("dxx1", C.c_double), ("dxx2", C.c_double),
        ("invdx0", C.c_double), ("invdx1", C.c_double), ("invdx2", C.c_double),
        ("xxmin0", C.c_double), ("xxmin1", C.c_double), ("xxmin2", C.c_double),
        ("xxmax0", C.c_double), ("xxmax1", C.c_double), ("xxmax2", C.c_double),
        ("AMPL", C.c_double), ("SINHW", C.c_double), ("RMAX", C.c_double),
        ("xmin", C.c_double), ("xmax", C.c_double), ("ymin", C.c_double),
        ("ymax", C.c_double), ("zmin", C.c_double), ("zmax", C.c_double),
        ("eta", C.c_double), ("wavespeed", C.c_double), ("time", C.c_double),
        ("diss_strength", C.c_double), ("enable_stress_energy_source_terms", C.c_int),
        ("const_dr", C.c_double),
        ("RHOMAX", C.c_double), ("ZMIN", C.c_double), ("ZMAX", C.c_double),
        ("AMPLRHO", C.c_double), ("SINHWRHO", C.c_double), ("AMPLZ", C.c_double), ("SINHWZ", C.c_double),
        ("const_drho", C.c_double), ("const_dz", C.c_double),
        ("bScale", C.c_double), ("SINHWAA", C.c_double), ("AMAX", C.c_double),
    ]


class rfm_struct(C.Structure):
    _fields_ = [("CoordSystem", C.c_int), ("N0", C.c_int), ("N1", C.c_int), ("nquant", C.c_int),
                ("table64", C.c_void_p), ("table32", C.c_void_p)]


class bc_struct(C.Structure):
    _fields_ = [
        ("NGHOSTS", C.c_int),
        ("num_ob_gz_pts", C.c_int * MAX_GHOSTS),
        ("num_ib_gz_pts", C.c_int * MAX_GHOSTS),
        ("ob_dir_start", (C.c_int * 4) * MAX_GHOSTS),
        ("ib_start", C.c_int * MAX_GHOSTS),
        ("total_outer", C.c_int), ("total_inner", C.c_int),
        ("outer_dest", C.c_void_p), ("outer_step", C.c_void_p),
        ("inner_dest", C.c_void_p), ("inner_src", C.c_void_p), ("inner_parity", C.c_void_p),
        ("nlev", C.c_int), ("lev_start", C.c_int * (MAX_BC_LEVELS + 1)), ("lev_inner", C.c_int * MAX_BC_LEVELS),
        ("lev_tail", C.c_int), ("lev_dest", C.c_void_p), ("lev_arg", C.c_void_p), ("lev_parity", C.c_void_p),
    ]


class MoL_gridfunctions(C.Structure):
    _fields_ = [("precision", C.c_int), ("y_n_gfs", C.c_void_p),
                ("y_nplus1_running_total_gfs", C.c_void_p), ("k_odd_gfs", C.c_void_p),
                ("k_even_gfs", C.c_void_p), ("auxevol_gfs", C.c_void_p)]


P = C.POINTER
vp = C.c_void_p
_PROTOS = {
    "nrgpu_version": (C.c_int, []),
    "nrgpu_set_stream": (C.c_int, [vp]),
    "nrgpu_get_stream": (vp, []),
    "nrgpu_last_error": (C.c_char_p, []),
    "nrgpu_kernel_launch_count": (C.c_longlong, []),
    "nrgpu_device_status": (C.c_int, [C.c_int]),
    "nrgpu_set_bssn_kernels": (C.c_int, [C.c_int]),
    "nrgpu_get_bssn_kernels": (C.c_int, []),
    "nrgpu_fd_coeffs": (C.c_int, [C.c_int, C.c_int, P(C.c_double)]),
    "set_Nxx_dxx_invdx_params__and__xx": (C.c_int, [C.c_int, P(C.c_int), P(paramstruct), P(P(C.c_double))]),
    "find_timestep": (C.c_double, [P(paramstruct), C.c_double]),
    "rfm_struct__malloc": (C.c_int, [P(paramstruct), P(rfm_struct)]),
    "rfm_struct__define": (C.c_int, [P(paramstruct), P(rfm_struct)]),
    "rfm_struct__freemem": (C.c_int, [P(rfm_struct)]),
    "rfm_struct__download": (C.c_int, [P(rfm_struct), P(C.c_double)]),
    "driver_bcstruct": (C.c_int, [P(paramstruct), P(bc_struct)]),
    "bcstruct_freemem": (C.c_int, [P(bc_struct)]),
    "bcstruct_download": (C.c_int, [P(bc_struct)] + [P(C.c_int)] * 5),
    "apply_bcs_curvilinear": (C.c_int, [P(paramstruct), P(bc_struct), C.c_int, P(C.c_int8), vp]),
    "apply_bcs_curvilinear_f32": (C.c_int, [P(paramstruct), P(bc_struct), C.c_int, P(C.c_int8), vp]),
    "ScalarWave_rhs_eval": (C.c_int, [P(paramstruct), vp, vp]),
    "ScalarWave_rhs_eval_f32": (C.c_int, [P(paramstruct), vp, vp]),
    "ScalarWaveCurvilinear_rhs_eval": (C.c_int, [P(rfm_struct), P(paramstruct), vp, vp]),
    "ScalarWaveCurvilinear_rhs_eval_f32": (C.c_int, [P(rfm_struct), P(paramstruct), vp, vp]),
    "Maxwell_rhs_eval": (C.c_int, [P(paramstruct), vp, vp]),
    "Maxwell_rhs_eval_f32": (C.c_int, [P(paramstruct), vp, vp]),
    "Maxwell_Constraints": (C.c_int, [P(paramstruct), vp, vp]),
    "BSSN_Ricci_eval": (C.c_int, [P(rfm_struct), P(paramstruct), vp, vp]),
    "BSSN_Ricci_eval_f32": (C.c_int, [P(rfm_struct), P(paramstruct), vp, vp]),
    "BSSN_rhs_eval": (C.c_int, [P(rfm_struct), P(paramstruct), vp, vp, vp]),
    "BSSN_rhs_eval_f32": (C.c_int, [P(rfm_struct), P(paramstruct), vp, vp, vp]),
    "BSSN_enforce_detgammabar_constraint": (C.c_int, [P(rfm_struct), P(paramstruct), vp]),
    "BSSN_enforce_detgammabar_constraint_f32": (C.c_int, [P(rfm_struct), P(paramstruct), vp]),
    "BSSN_Hamiltonian_constraint": (C.c_int, [P(rfm_struct), P(paramstruct), vp, vp]),
    "BSSN_Ricci_eval_xx": (C.c_int, [P(paramstruct), P(C.c_void_p), vp, vp]),
    "BSSN_rhs_eval_xx": (C.c_int, [P(paramstruct), P(C.c_void_p), vp, vp, vp]),
    "BSSN_momentum_constraint": (C.c_int, [P(rfm_struct), P(paramstruct), vp, vp]),
    "BSSN_psi4": (C.c_int, [P(rfm_struct), P(paramstruct), vp, vp, C.c_int, C.c_int]),
    "MaxwellCurvilinear_rhs_eval": (C.c_int, [P(rfm_struct), P(paramstruct), vp, vp]),
    "MaxwellCurvilinear_rhs_eval_f32": (C.c_int, [P(rfm_struct), P(paramstruct), vp, vp]),
    "MaxwellCurvilinear_constraints": (C.c_int, [P(rfm_struct), P(paramstruct), vp, vp]),
    "MaxwellCurvilinear_initial_data_toroidal_dipole": (C.c_int, [P(paramstruct), C.c_double, C.c_double,
                                                                  C.c_double, vp]),
    "BSSN_constraints_add_source_terms": (C.c_int, [P(rfm_struct), P(paramstruct), vp, vp, vp, vp]),
    "BSSN_psi4_spinweightm2_decomposition": (C.c_int, [P(paramstruct), vp, C.c_int, C.c_int, vp]),
    "ScalarWave_initial_data": (C.c_int, [P(paramstruct), C.c_int, C.c_double, P(C.c_double), C.c_double, vp]),
    "BSSN_initial_data_BrillLindquist": (C.c_int, [P(paramstruct), C.c_double, P(C.c_double),
                                                   C.c_double, P(C.c_double), vp]),
    "MoL_step_forward_in_time": (C.c_int, [C.c_int, P(rfm_struct), P(paramstruct), P(bc_struct),
                                           P(MoL_gridfunctions), C.c_double]),
    "MoL_step_forward_in_time_unfused": (C.c_int, [C.c_int, P(rfm_struct), P(paramstruct), P(bc_struct),
                                                   P(MoL_gridfunctions), C.c_double]),
    "MoL_substep_rhs": (C.c_int, [C.c_int, P(rfm_struct), P(paramstruct), P(MoL_gridfunctions), C.c_int,
                                  C.c_double, C.c_int]),
    "MoL_step_forward_in_time_sommerfeld": (C.c_int, [C.c_int, P(rfm_struct), P(paramstruct), P(bc_struct),
                                                      P(MoL_gridfunctions), C.c_double]),
    "nrgpu_sommerfeld_params": (C.c_int, [C.c_int, C.c_int, P(C.c_double), P(C.c_double), P(C.c_double)]),
    "apply_bcs_sommerfeld": (C.c_int, [P(paramstruct), P(C.c_void_p), P(bc_struct), C.c_int, P(C.c_int8),
                                       vp, vp]),
    "MoL_evolve_host": (C.c_int, [C.c_int, P(rfm_struct), P(paramstruct), P(bc_struct),
                                  P(MoL_gridfunctions), C.c_double, C.c_int, P(C.c_double)]),
    "nrgpu_l2_norm_sq": (C.c_int, [P(paramstruct), vp, C.c_int, vp, C.c_int, vp]),
    "nrgpu_l2_norm_sq_static": (C.c_int, [P(paramstruct), vp, C.c_int, vp]),
    "Maxwell_rhs_eval_adjoint": (C.c_int, [P(paramstruct), vp, vp]),
    "apply_bcs_curvilinear_adjoint": (C.c_int, [P(paramstruct), P(bc_struct), C.c_int, P(C.c_int8), vp]),
    "nrgpu_bc_outer_points": (C.c_int, [P(paramstruct), C.c_int, vp, vp, C.c_int, vp]),
    "nrgpu_bc_gather_points": (C.c_int, [P(paramstruct), C.c_int, vp, C.c_int, vp, vp]),
    "nrgpu_bc_scatter_parity": (C.c_int, [P(paramstruct), C.c_int, P(C.c_int8), vp, vp, C.c_int, vp, vp]),
    "xx_to_Cart": (C.c_int, [P(paramstruct), vp, C.c_int, C.c_int, C.c_int, P(C.c_double)]),
    "BSSN_tangent_rhs_eval": (C.c_int, [P(rfm_struct), P(paramstruct), C.c_int, vp, vp, vp]),
    "BSSN_tangent_step": (C.c_int, [P(rfm_struct), P(paramstruct), P(bc_struct), C.c_int, vp, vp, C.c_double]),
    "BSSN_tangent_initial_data_BrillLindquist": (C.c_int, [P(paramstruct), C.c_double, P(C.c_double), C.c_double,
                                                           P(C.c_double), C.c_int, P(C.c_int), vp]),
    "BSSN_tangent_shell_accumulate": (C.c_int, [P(paramstruct), C.c_int, vp, C.c_int, C.c_int, vp, C.c_double,
                                                C.c_double, vp]),
    "ScalarWave_rhs_eval_adjoint": (C.c_int, [P(rfm_struct), P(paramstruct), vp, vp]),
    "MoL_adjoint_step_backward": (C.c_int, [C.c_int, P(rfm_struct), P(paramstruct), P(bc_struct), vp, vp, vp,
                                            C.c_double]),
    "ScalarWave_initial_data_gaussian": (C.c_int, [P(paramstruct), C.c_double, C.c_double, C.c_double,
                                                   vp, vp, vp, vp]),
    "nrgpu_shell_sample": (C.c_int, [P(paramstruct), vp, C.c_int, C.c_int, vp, C.c_double, vp, vp]),
    "nrgpu_shell_sample_adjoint": (C.c_int, [P(paramstruct), vp, C.c_int, C.c_int, vp, C.c_double, vp, vp]),
    "Maxwell_initial_data_toroidal_dipole": (C.c_int, [P(paramstruct), C.c_double, C.c_double, C.c_double,
                                                       vp, vp, vp]),
    "nrgpu_sphere_sample": (C.c_int, [P(paramstruct), vp, C.c_int, C.c_int, vp, vp, C.c_int, C.c_double,
                                      vp, vp]),
    "nrgpu_sphere_sample_adjoint": (C.c_int, [P(paramstruct), vp, C.c_int, C.c_int, vp, vp, C.c_int,
                                              C.c_double, vp, vp]),
    "nrgpu_sphere_check": (C.c_int, [P(paramstruct), P(C.c_int)]),
    "nrgpu_dot": (C.c_int, [vp, vp, C.c_longlong, vp, C.c_int, vp]),
    "nrgpu_batch_create": (C.c_int, [C.c_int, P(C.c_int), C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                     C.c_double, C.c_double, C.c_double, C.c_int, P(vp)]),
    "nrgpu_batch_free": (C.c_int, [vp]),
    "nrgpu_batch_total_points": (C.c_longlong, [vp]),
    "nrgpu_batch_offsets": (C.c_int, [vp, P(C.c_longlong), P(C.c_longlong), P(C.c_int)]),
    "nrgpu_batch_timesteps": (C.c_int, [vp, P(C.c_double)]),
    "nrgpu_batch_set_timesteps": (C.c_int, [vp, P(C.c_double)]),
    "nrgpu_batch_initial_data_gaussian": (C.c_int, [vp, P(C.c_double), P(C.c_double), P(C.c_double), vp]),
    "nrgpu_batch_rhs_eval": (C.c_int, [vp, vp, vp]),
    "nrgpu_batch_apply_bcs": (C.c_int, [vp, vp, C.c_int]),
    "nrgpu_batch_step": (C.c_int, [vp, P(MoL_gridfunctions)]),
    "nrgpu_batch_autotune": (C.c_int, [vp, vp, vp, C.c_int, P(C.c_float)]),
    "nrgpu_batch_set_tile": (C.c_int, [vp, C.c_int, C.c_int, C.c_int]),
    "nrgpu_batch_get_tile": (C.c_int, [vp, P(C.c_int), P(C.c_int), P(C.c_int)]),
}

_lib = None


def load():
    """Loads libnrgpu.so and declares every prototype; raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBPATH):
        raise NrgpuError("libnrgpu.so is not built (%s); run __graft_entry__.build() "
                         "or python nrpytutorial_gb300/build.py" % LIBPATH)
    lib = C.CDLL(LIBPATH)
    for name, (res, args) in _PROTOS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return list(_PROTOS)


def check(status, what=""):
    if status != 0:
        msg = load().nrgpu_last_error().decode(errors="replace")
        raise NrgpuError("%s failed (status %d): %s" % (what, status, msg))


def ptr(t):
    """Device (or host) address of a torch tensor / numpy array as c_void_p."""
    if t is None:
        return None
    if hasattr(t, "data_ptr"):
        return C.c_void_p(t.data_ptr())
    return C.c_void_p(t.ctypes.data)


def set_stream(stream):
    """Queue library work on a torch.cuda.Stream (or raw handle)."""
    h = getattr(stream, "cuda_stream", stream)
    check(load().nrgpu_set_stream(C.c_void_p(h)), "nrgpu_set_stream")
