/*
 * nrgpu.h -- C ABI of the GB300 (sm_103a) method-of-lines finite-difference
 * evolution library (libnrgpu.so).
 *
 * What it replaces.  NRPy+/SENR drivers are C programs whose time loop
 * #includes the generated MoLtimestepping/RK_MoL.h; every RK substep there
 * calls a generated rhs_eval (plus Ricci_eval for BSSN), a flat
 * LOOP_ALL_GFS_GPS RK update, apply_bcs_curvilinear and
 * enforce_detgammabar_constraint.  Each entry point below is the drop-in for
 * one of those calls and keeps its argument meaning, its gridfunction layout
 * (IDX4S: i0 fastest, gridfunctions outermost, alphabetical gridfunction
 * order) and its point set (interior points for RHS kernels, all points for
 * the update and the det(gammabar) rescale).  The reference cites are file
 * paths within zachetienne/nrpytutorial.
 *
 * Conventions that differ from the generated C, and why:
 *  - Gridfunction arrays are DEVICE pointers (cudaMalloc'ed or torch CUDA
 *    tensors).  Work is queued on the library's current stream
 *    (nrgpu_set_stream) and is asynchronous; no entry point on the time-step
 *    path synchronises the host or allocates memory.
 *  - Every entry point returns an int status (NRGPU_OK == 0) instead of
 *    calling exit(1); nrgpu_last_error() gives the message.
 *  - Each physical system has its own rhs_eval name, because one library
 *    serves all of them (a SENR driver compiles only one rhs_eval).
 *  - "_f32" variants take FP32 gridfunctions and evaluate the RHS in FP32;
 *    rfm precompute tables, the RK4 state y_n and its running total stay FP64.
 */
#ifndef NRGPU_H
#define NRGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define NRGPU_OK               0
#define NRGPU_ERR_ARG          1  /* bad pointer, size, order or coordinate system */
#define NRGPU_ERR_CUDA         2  /* a CUDA runtime call failed                    */
#define NRGPU_ERR_UNSUPPORTED  3  /* combination not built into this library        */
#define NRGPU_ERR_BCMAP        4  /* ghost-zone map failed its Cartesian/parity check */
#define NRGPU_ERR_SIZE         5  /* grid or batch larger than a fixed limit        */

/* ------------------------------------------------------ coordinate systems */
/* reference_metric.py:100-176 (Spherical, SinhSpherical, SinhSphericalv2),
   :398-428 (Cartesian) */
#define NRGPU_COORD_CARTESIAN        0
#define NRGPU_COORD_SPHERICAL        1
#define NRGPU_COORD_SINHSPHERICAL    2
#define NRGPU_COORD_SINHSPHERICALV2  3  /* r = AMPL (const_dr xx0 + sinh(xx0/SINHW)/sinh(1/SINHW)) */
/* reference_metric.py:226-300: (rho, phi, z); the reference metric depends on
   xx0 and xx2, so its tables are per (i0, i2) column */
#define NRGPU_COORD_CYLINDRICAL      4  /* rho = xx0, z = xx2                                 */
#define NRGPU_COORD_SINHCYLINDRICAL  5  /* rho = AMPLRHO sinh(xx0/SINHWRHO)/sinh(1/SINHWRHO),
                                           z = AMPLZ sinh(xx2/SINHWZ)/sinh(1/SINHWZ)       */
#define NRGPU_COORD_SINHCYLINDRICALV2 6 /* adds AMPLRHO const_drho xx0 to rho and
                                           AMPLZ const_dz xx2 to z (:265-275)               */
/* reference_metric.py:306-383: symmetric TP coordinates, foci at z = +-bScale;
   every scale factor depends on xx0 and xx1 (tables per (i0, i1) column) */
#define NRGPU_COORD_SYMTP            7  /* AA = xx0                                          */
#define NRGPU_COORD_SINHSYMTP        8  /* AA = AMAX sinh(xx0/SINHWAA)/sinh(1/SINHWAA)      */

/* ------------------------------------------------------------- systems */
#define NRGPU_SYS_SCALARWAVE  0   /* uu, vv                                   */
#define NRGPU_SYS_MAXWELL     1   /* AU0..2, EU0..2, psi  (System I)          */
#define NRGPU_SYS_BSSN        2   /* 24 evolved gfs, alphabetical             */
#define NRGPU_SYS_MAXWELL_CURVILINEAR 3  /* Gamma, aU0..2, eU0..2, psi (System II
                                    rescaled, VacuumMaxwell_Flat_Evol_Curvilinear_rescaled.py) */

#define NRGPU_PREC_FP64   0       /* everything FP64                          */
#define NRGPU_PREC_MIXED  1       /* FP32 stage buffers + FP32 RHS, FP64 y_n  */
#define NRGPU_PREC_COMPENSATED 2  /* FP32 RHS on FP32 (hi, lo) pair stage
                                     buffers, FP64 y_n and running total    */
#define NRGPU_PREC_COMPENSATED_FP64RK 3  /* the same FP32 RHS on pair stages, with
                                     the RK4 accumulation (y_n, running total)
                                     and the det(gammabar) rescale in FP64
                                     arithmetic: the mixed-precision form whose
                                     only FP32 arithmetic is the RHS. COMPENSATED
                                     carries the accumulation and rescale in
                                     float-float (48 bits) on the FP32 pipe
                                     instead. Single-grid MoL steps only. */

/* The name of the library's parameter struct.  A generated driver whose own
 * declare_Cparameters_struct.h already defines `paramstruct` defines
 * NRGPU_PARAMSTRUCT (e.g. nrgpu_paramstruct) before including this header;
 * nrpytutorial_gb300/params_shim.py then writes the conversion between the
 * two (nrgpu_params_from_generated). */
#ifndef NRGPU_PARAMSTRUCT
#define NRGPU_PARAMSTRUCT paramstruct
#endif

/*
 * paramstruct: the runtime parameters the generated kernels read through
 * set_Cparameters.h (NRPy_param_funcs.py:216-304 emits the reference's struct).
 * Field names follow the reference's C parameter names.
 */
typedef struct nrgpu_paramstruct_s {
  int    CoordSystem;                 /* NRGPU_COORD_*                          */
  int    FD_order;                    /* 2, 4, 6 or 8 (FD_CENTDERIVS_ORDER)     */
  int    NGHOSTS;                     /* ghost zones per side                   */
  int    Nxx0, Nxx1, Nxx2;            /* interior points                        */
  int    Nxx_plus_2NGHOSTS0, Nxx_plus_2NGHOSTS1, Nxx_plus_2NGHOSTS2;
  double dxx0, dxx1, dxx2;
  double invdx0, invdx1, invdx2;
  double xxmin0, xxmin1, xxmin2;      /* uniform-coordinate domain              */
  double xxmax0, xxmax1, xxmax2;
  double AMPL, SINHW;                 /* SinhSpherical  (reference_metric.py:123) */
  double RMAX;                        /* Spherical      (reference_metric.py:107) */
  double xmin, xmax, ymin, ymax, zmin, zmax;   /* Cartesian (:400-401)          */
  double eta;                         /* Gamma-driver damping (BSSN_gauge_RHSs.py:233) */
  double wavespeed;                   /* ScalarWave/CommonParams.py:24          */
  double time;
  double diss_strength;               /* Kreiss-Oliger dissipation added to every BSSN
                                         RHS (KO_Dissipation::diss_strength,
                                         BaikalETK_C_kernels_codegen.py:147-171); 0 = off */
  int    enable_stress_energy_source_terms;  /* 1: the BSSN RHSs add the T^{mu nu}
                                         source terms (BSSN_stress_energy_source_terms.py,
                                         as BaikalETK_C_kernels_codegen.py:133-145 adds
                                         them); auxevol_gfs then holds 16 gridfunctions:
                                         RbarDD00..22, then T4UU00, 01, 02, 03, 11, 12,
                                         13, 22, 23, 33 (the stage's storage type) */
  double const_dr;                    /* SinhSphericalv2 (reference_metric.py:141) */
  double RHOMAX, ZMIN, ZMAX;          /* Cylindrical (reference_metric.py:233)     */
  double AMPLRHO, SINHWRHO, AMPLZ, SINHWZ;  /* SinhCylindrical (:249-251)          */
  double const_drho, const_dz;        /* SinhCylindricalv2 (reference_metric.py:271) */
  double bScale, SINHWAA, AMAX;       /* SymTP, SinhSymTP (reference_metric.py:308-310) */
} NRGPU_PARAMSTRUCT;

/*
 * rfm_struct: FP64 reference-metric precompute tables (the rfm_precompute
 * arrays of reference_metric.py:603-886, here as dense derived quantities per
 * (i0,iB) column, iB = i1 for the Spherical family and i2 for the Cylindrical
 * family), plus an FP32 copy for the mixed-precision kernels.
 */
typedef struct rfm_struct {
  int     CoordSystem;
  int     N0, N1;            /* table extents = Nxx_plus_2NGHOSTS0 and that of
                                the second coordinate (Nxx_plus_2NGHOSTS1, or
                                Nxx_plus_2NGHOSTS2 for the Cylindrical family) */
  int     nquant;            /* doubles per (i0,iB)                            */
  double *table64;           /* device, [nquant][N1][N0]                       */
  float  *table32;           /* device, same layout                            */
} rfm_struct;

/*
 * bc_struct: the compacted ghost-zone map of set_bcstruct.h:32-124
 * (BCs_data_structs.h:2-49), flattened into device arrays.  Per ghost layer
 * `g` (innermost first) the outer points are grouped by face direction
 * (i0 faces, then i1, then i2, as set_bcstruct.h orders them) and followed by
 * the inner (parity) points.
 */
#define NRGPU_MAX_GHOSTS 8
#define NRGPU_MAX_BC_LEVELS 32
typedef struct bc_struct {
  int  NGHOSTS;
  int  num_ob_gz_pts[NRGPU_MAX_GHOSTS];        /* outer points in layer g   */
  int  num_ib_gz_pts[NRGPU_MAX_GHOSTS];        /* inner points in layer g   */
  int  ob_dir_start[NRGPU_MAX_GHOSTS][4];      /* offsets into outer arrays */
  int  ib_start[NRGPU_MAX_GHOSTS];             /* offsets into inner arrays */
  int  total_outer, total_inner;
  int *outer_dest;      /* device: idx3 of each outer ghost point            */
  int *outer_step;      /* device: FACE*stride toward the interior            */
  int *inner_dest;      /* device: idx3 of each inner ghost point            */
  int *inner_src;       /* device: idx3 of its interior source point         */
  int *inner_parity;    /* device: bit t set <=> parity type t is -1          */
  /* Level schedule of the same points (built by driver_bcstruct): a point's
   * level is 1 + the largest level among the points it reads (interior
   * points 0) in the sequential order above; when no point is read before
   * that order writes it, every level is applied at once with the same
   * arithmetic, which gives the sequential result bit for bit.  nlev = 0:
   * no schedule (the phases above are applied in order). */
  int  nlev;
  int  lev_start[NRGPU_MAX_BC_LEVELS + 1];     /* entries of level l: [lev_start[l], lev_start[l+1]) */
  int  lev_inner[NRGPU_MAX_BC_LEVELS];         /* first inner (parity) entry of level l             */
  int  lev_tail;        /* levels >= lev_tail are small: one block per gridfunction applies them all */
  int *lev_dest;        /* device: idx3 of each entry's ghost point          */
  int *lev_arg;         /* device: outer step, or inner source idx3          */
  int *lev_parity;      /* device: inner parity bits (0 for outer entries)   */
} bc_struct;

/*
 * MoL_gridfunctions: the four RK4 buffers of RK_Allocate_Memory.h
 * (MoLtimestepping/C_Code_Generation.py:97-103) plus auxevol storage.
 * y_n and the running total are always FP64; k_odd/k_even/auxevol are FP64
 * for NRGPU_PREC_FP64 and FP32 otherwise.  All device pointers, each
 * NUM_EVOL_GFS * Nxx_plus_2NGHOSTS_tot values long (auxevol: 6 gfs for BSSN).
 * NRGPU_PREC_COMPENSATED: k_odd/k_even hold interleaved FP32 pairs (float2:
 * hi = FP32(v), lo = FP32(v - hi) of each FP64 stage value v), twice the
 * floats of the MIXED buffers; each step starts by splitting y_n into
 * k_even.  Stencils difference the hi parts (exact in FP32 for neighbouring
 * values within a factor 2) and add the plain stencil of the lo parts, so
 * the FP32 rounding of a value never enters a derivative.
 */
typedef struct MoL_gridfunctions {
  int     precision;                     /* NRGPU_PREC_*                     */
  double *y_n_gfs;
  double *y_nplus1_running_total_gfs;
  void   *k_odd_gfs;
  void   *k_even_gfs;
  void   *auxevol_gfs;
} MoL_gridfunctions;

/* ------------------------------------------------------------ library */
int         nrgpu_version(void);
/* Queue all subsequent work on this cudaStream_t (NULL = legacy default). */
int         nrgpu_set_stream(void *cuda_stream);
void       *nrgpu_get_stream(void);
/* Message of the last failing call in this process. */
const char *nrgpu_last_error(void);
/* Number of kernels this library has launched in this process. */
long long   nrgpu_kernel_launch_count(void);
/* Device status word of the current device: nonzero once a kernel's bounded
 * wait for one of its own asynchronous copies gave up (that kernel stored
 * nothing).  Synchronises the library stream; clear != 0 resets the word.
 * Returns the word, or -NRGPU_ERR_CUDA.  No reference counterpart. */
int         nrgpu_device_status(int clear);
/* Which kernels evaluate BSSN Ricci_eval / rhs_eval (no reference
 * counterpart: the reference has one generated loop per function).
 *   POINT:  one thread per point, every stencil tap read from global memory;
 *   STAGED: a block per 16x4x2 brick (16x4x1 in FP64); each gridfunction's
 *           brick-plus-halo box staged in shared memory by TMA, finite
 *           differences evaluated there, then the algebra;
 *   FUSED:  STAGED with Ricci computed inside the RHS kernel of a MoL step
 *           (auxevol is neither written nor read by the step);
 *   AUTO:   per grid and precision, the family measured fastest for a
 *           whole step on GB300: FP64 and Cartesian grids POINT; curvilinear
 *           grids with FP32 pair stages (the compensated modes) FUSED, SymTP
 *           family STAGED; curvilinear grids with plain FP32 stages STAGED.
 *           A grid the staged kernels cannot take (NGHOSTS other than
 *           FD_order/2 + 1, stage arrays or rows not 16-byte aligned) runs
 *           POINT.
 * Kreiss-Oliger dissipation, T^{mu nu} sources, the no-precompute _xx
 * functions and FP32 arithmetic on FP64 input always run on POINT.
 * Process-wide setting. */
#define NRGPU_BSSN_KERNELS_AUTO   0
#define NRGPU_BSSN_KERNELS_POINT  1
#define NRGPU_BSSN_KERNELS_STAGED 2
#define NRGPU_BSSN_KERNELS_FUSED  3
int         nrgpu_set_bssn_kernels(int mode);
int         nrgpu_get_bssn_kernels(void);
/* FD coefficients the kernels use: kind 0 = centred 1st, 1 = centred 2nd,
 * 2 = upwind (+1 shifted) 1st, 3 = Kreiss-Oliger.  Writes order+1 doubles
 * (offsets -order/2 ... +order/2, shifted by +1 for kind 2), order+3 for
 * kind 3 (offsets -order/2-1 ... order/2+1).  Host only, no GPU needed.
 * finite_difference.py:252-369 computes the reference's. */
int         nrgpu_fd_coeffs(int order, int kind, double *out);

/* --------------------------------------------------------- grid set-up */
/* reference_metric.py:1330-1395 (set_Nxx_dxx_invdx_params__and__xx):
 * sets Nxx*, Nxx_plus_2NGHOSTS*, dxx*, invdx*, xxmin/xxmax from CoordSystem,
 * NGHOSTS and the coordinate parameters already in *params, and fills the
 * caller-allocated host arrays xx[d][Nxx_plus_2NGHOSTS_d] with cell-centred
 * coordinates (xx, or any xx[d], may be NULL: nothing is written there).
 * EigenCoord=1 uses the eigen-coordinate domain (Spherical for the Spherical
 * family), as the reference does before building BC maps. */
int    set_Nxx_dxx_invdx_params__and__xx(int EigenCoord, const int Nxx[3],
                                         NRGPU_PARAMSTRUCT *params, double *xx[3]);
/* reference_metric.py:1397-1410 (xx_to_Cart_h): Cartesian position of
 * grid point (i0, i1, i2), from the host arrays xx[d] (or, where xx or xx[d]
 * is NULL, the cell-centred coordinate of the uniform grid).  Host; returns
 * a status (the reference's function is void). */
int    xx_to_Cart(const NRGPU_PARAMSTRUCT *params, double *xx[3], int i0, int i1, int i2, double xCart[3]);
/* reference_metric.py:1412-1439 (find_timestep): CFL * min over interior
 * points of the proper spacing dxx_i * scalefactor_i, / wavespeed.  Host. */
double find_timestep(const NRGPU_PARAMSTRUCT *params, double CFL_FACTOR);

/* ----------------------------------------------- reference metric tables */
/* rfm_struct__malloc.h / rfm_struct__define.h / rfm_struct__freemem.h
 * (reference_metric.py:871-886).  define() runs an FP64 kernel. */
int rfm_struct__malloc(const NRGPU_PARAMSTRUCT *params, rfm_struct *rfm);
int rfm_struct__define(const NRGPU_PARAMSTRUCT *params, rfm_struct *rfm);
int rfm_struct__freemem(rfm_struct *rfm);
/* Copy the FP64 table back to the host (testing): host buffer of
 * nquant*N0*N1 doubles. */
int rfm_struct__download(const rfm_struct *rfm, double *host);

/* ---------------------------------------------------------- boundaries */
/* boundary_conditions/driver_bcstruct.h:8-44 (set_up__bc_gz_map_and_parity_condns
 * + set_bcstruct), built on the host on the eigen-coordinate grid, uploaded. */
int driver_bcstruct(const NRGPU_PARAMSTRUCT *params, bc_struct *bcstruct);
int bcstruct_freemem(bc_struct *bcstruct);
/* Host copy of the flattened map (testing).  Buffers sized total_outer /
 * total_inner as reported in *bcstruct. */
int bcstruct_download(const bc_struct *bcstruct, int *outer_dest, int *outer_step,
                      int *inner_dest, int *inner_src, int *inner_parity);
/* apply_bcs_curvilinear.h:56-64: per ghost layer, quadratic extrapolation at
 * outer points then parity copy at inner points.  gfs_parity is a HOST array
 * of NUM_GFS parity types (0..9). */
int apply_bcs_curvilinear(const NRGPU_PARAMSTRUCT *params, const bc_struct *bcstruct,
                          int NUM_GFS, const int8_t *gfs_parity, double *gfs);
int apply_bcs_curvilinear_f32(const NRGPU_PARAMSTRUCT *params, const bc_struct *bcstruct,
                              int NUM_GFS, const int8_t *gfs_parity, float *gfs);
/* The same boundary conditions on one slab of a grid split along i2 over
 * several ranks (no counterpart in the reference, whose drivers run one
 * grid in one process).  params describe the slab (its own Nxx2 and
 * xxmin2); indices are the slab's idx3; FP64; device arrays.  A rank applies,
 * per ghost layer, the outer rule to the outer points it owns, one face
 * direction per call in the order i0, i1, i2 (nrgpu_bc_outer_points), then
 * the parity copies of its inner points from source values gathered on the
 * ranks that own them: nrgpu_bc_gather_points packs buf[j*NUM_GFS + gf] =
 * gfs[gf][src[j]], the buffers travel rank to rank, and
 * nrgpu_bc_scatter_parity writes gfs[gf][dest[j]] = +-buf[j*NUM_GFS + gf]
 * (minus where bit gfs_parity[gf] of parity_bits[j] is set; gfs_parity a
 * HOST array).  Arithmetic identical to apply_bcs_curvilinear. */
int nrgpu_bc_outer_points(const NRGPU_PARAMSTRUCT *params, int NUM_GFS, const int *dest, const int *step, int n,
                          double *gfs);
int nrgpu_bc_gather_points(const NRGPU_PARAMSTRUCT *params, int NUM_GFS, const int *src, int n,
                           const double *gfs, double *buf);
int nrgpu_bc_scatter_parity(const NRGPU_PARAMSTRUCT *params, int NUM_GFS, const int8_t *gfs_parity,
                            const int *dest, const int *parity_bits, int n, const double *buf, double *gfs);

/* Sommerfeld radiation boundary condition (CurviBoundaryConditions.py:259-658,
 * apply_bcs_sommerfeld): sets rhs_gfs at every ghost point from the state
 * gfs: outer points rhs = -c (d_r f + (f - f_inf)/r) plus the radial-falloff
 * correction from the point one step inward; inner points copy the RHS with
 * parity.  xx: device coordinate arrays (or NULL for the cell-centred
 * coordinates of params).  FP64.  The per-gridfunction speed c, f_inf and
 * falloff power, and the FD order (2, 4, 6) of d_r, are those of
 * sommerfeld_boundary_condition_class (defaults 1, 0, 3 and 2; the
 * reference writes them into sommerfeld_params.h) and are set by
 * nrgpu_sommerfeld_params (NULL arrays leave values unchanged). */
int nrgpu_sommerfeld_params(int fd_order, int NUM_GFS, const double *speed, const double *f_inf,
                            const double *radial_falloff_power);
int apply_bcs_sommerfeld(const NRGPU_PARAMSTRUCT *params, double *xx[3], const bc_struct *bcstruct, int NUM_GFS,
                         const int8_t *gfs_parity, const double *gfs, double *rhs_gfs);

/* -------------------------------------------------------- RHS kernels */
/* ScalarWave Cartesian: rhs_eval(params, in_gfs, rhs_gfs)
 * (Tutorial-Start_to_Finish-ScalarWave.ipynb, rhs_eval; ScalarWave_RHSs.py:46-71) */
int ScalarWave_rhs_eval(const NRGPU_PARAMSTRUCT *params, const double *in_gfs, double *rhs_gfs);
int ScalarWave_rhs_eval_f32(const NRGPU_PARAMSTRUCT *params, const float *in_gfs, float *rhs_gfs);
/* ScalarWave curvilinear: rhs_eval(rfmstruct, params, in_gfs, rhs_gfs)
 * (ScalarWaveCurvilinear_RHSs.py:43-98) */
int ScalarWaveCurvilinear_rhs_eval(const rfm_struct *rfm, const NRGPU_PARAMSTRUCT *params,
                                   const double *in_gfs, double *rhs_gfs);
int ScalarWaveCurvilinear_rhs_eval_f32(const rfm_struct *rfm, const NRGPU_PARAMSTRUCT *params,
                                       const float *in_gfs, float *rhs_gfs);
/* Vacuum Maxwell System I, Cartesian (VacuumMaxwell_Flat_Evol_Cartesian.py:54-74) */
int Maxwell_rhs_eval(const NRGPU_PARAMSTRUCT *params, const double *in_gfs, double *rhs_gfs);
int Maxwell_rhs_eval_f32(const NRGPU_PARAMSTRUCT *params, const float *in_gfs, float *rhs_gfs);
/* Maxwell divergence constraint C = d_i E^i at interior points
 * (VacuumMaxwell_Flat_Evol_Cartesian.py:49-52) into aux_gfs[0]. */
int Maxwell_Constraints(const NRGPU_PARAMSTRUCT *params, const double *in_gfs, double *aux_gfs);
/* Vacuum Maxwell System II in rescaled curvilinear form
 * (Maxwell/VacuumMaxwell_Flat_Evol_Curvilinear_rescaled.py:22-190; the
 * rhs_eval of Tutorial-Start_to_Finish-Solving_Maxwells_Equations_in_Vacuum-
 * Curvilinear.ipynb): 8 gridfunctions Gamma, aU0..2, eU0..2, psi.  rfm may be
 * NULL on a Cartesian grid.  Constraints C (divergence of E) and G
 * (Gamma - div A) into aux_gfs[0], aux_gfs[1].  Toroidal-dipole data in the
 * grid's basis (Maxwell/InitialData.py:26-117, System II) at every point. */
int MaxwellCurvilinear_rhs_eval(const rfm_struct *rfm, const NRGPU_PARAMSTRUCT *params, const double *in_gfs,
                                double *rhs_gfs);
int MaxwellCurvilinear_rhs_eval_f32(const rfm_struct *rfm, const NRGPU_PARAMSTRUCT *params, const float *in_gfs,
                                    float *rhs_gfs);
int MaxwellCurvilinear_constraints(const rfm_struct *rfm, const NRGPU_PARAMSTRUCT *params, const double *in_gfs,
                                   double *aux_gfs);
int MaxwellCurvilinear_initial_data_toroidal_dipole(const NRGPU_PARAMSTRUCT *params, double amp, double lam,
                                                    double time, double *in_gfs);
/* BSSN conformal Ricci tensor into auxevol_gfs (RbarDD00..22, 6 gfs):
 * Ricci_eval(rfmstruct, params, in_gfs, auxevol_gfs)
 * (BSSN_quantities.py:260-425; Tutorial-Start_to_Finish-BSSNCurvilinear-Two_BHs_Collide.ipynb:501-502) */
int BSSN_Ricci_eval(const rfm_struct *rfm, const NRGPU_PARAMSTRUCT *params,
                    const double *in_gfs, double *auxevol_gfs);
int BSSN_Ricci_eval_f32(const rfm_struct *rfm, const NRGPU_PARAMSTRUCT *params,
                        const float *in_gfs, float *auxevol_gfs);
/* BSSN + gauge RHSs: rhs_eval(rfmstruct, params, auxevol_gfs, in_gfs, rhs_gfs)
 * (BSSN_RHSs.py:28-328, BSSN_gauge_RHSs.py:33-293; ...Two_BHs_Collide.ipynb:477-478) */
int BSSN_rhs_eval(const rfm_struct *rfm, const NRGPU_PARAMSTRUCT *params,
                  const double *auxevol_gfs, const double *in_gfs, double *rhs_gfs);
int BSSN_rhs_eval_f32(const rfm_struct *rfm, const NRGPU_PARAMSTRUCT *params,
                      const float *auxevol_gfs, const float *in_gfs, float *rhs_gfs);
/* The same two functions in the reference's no-precompute form
 * rhs_eval(params, xx, auxevol_gfs, in_gfs, rhs_gfs)
 * (...Two_BHs_Collide-no_rfm_precompute.ipynb:477): the reference metric is
 * evaluated at each point from the caller's coordinate arrays xx[0][i0],
 * xx[1][i1] (device pointers; xx[2] is not read).  FP64. */
int BSSN_Ricci_eval_xx(const NRGPU_PARAMSTRUCT *params, double *xx[3], const double *in_gfs, double *auxevol_gfs);
int BSSN_rhs_eval_xx(const NRGPU_PARAMSTRUCT *params, double *xx[3], const double *auxevol_gfs,
                     const double *in_gfs, double *rhs_gfs);
/* enforce_detgammabar_constraint(rfmstruct, params, in_gfs) at ALL points
 * (Enforce_Detgammabar_Constraint.py:16-75).  FP64 arithmetic on FP64 data;
 * float-float arithmetic (~48 significant bits, FP32 pipe) on FP32 data. */
int BSSN_enforce_detgammabar_constraint(const rfm_struct *rfm, const NRGPU_PARAMSTRUCT *params,
                                        double *in_gfs);
int BSSN_enforce_detgammabar_constraint_f32(const rfm_struct *rfm, const NRGPU_PARAMSTRUCT *params,
                                            float *in_gfs);
/* Hamiltonian constraint H at interior points into aux_gfs[0]
 * (BSSN_constraints.py:19-74; Ricci evaluated inline). */
int BSSN_Hamiltonian_constraint(const rfm_struct *rfm, const NRGPU_PARAMSTRUCT *params,
                                const double *in_gfs, double *aux_gfs);
/* Momentum constraint M^i (rescaled by ReU) at interior points into
 * aux_gfs[0..2] (BSSN_constraints.py:76-126). */
int BSSN_momentum_constraint(const rfm_struct *rfm, const NRGPU_PARAMSTRUCT *params,
                             const double *in_gfs, double *aux_gfs);

/* Matter terms of the constraints (BSSN_stress_energy_source_terms.py:134-161;
 * BSSN_constraints.py:76-80 adds the H one): H[idx] += -16 pi rho and
 * MU[i] += -8 pi S^i / ReU^i at interior points, from the ten T4UU
 * gridfunctions T4UU00, 01, 02, 03, 11, 12, 13, 22, 23, 33 (FP64).  H or MU
 * may be NULL.  Call after BSSN_Hamiltonian_constraint / BSSN_momentum_constraint. */
int BSSN_constraints_add_source_terms(const rfm_struct *rfm, const NRGPU_PARAMSTRUCT *params, const double *in_gfs,
                                      const double *T4UU_gfs, double *H_gf, double *MU_gfs);
/* psi_4 in the quasi-Kinnersley tetrad (BSSN/Psi4.py:14-193 with
 * BSSN/Psi4_tetrads.py:25-193; the reference's psi4() of
 * Tutorial-Start_to_Finish-BSSNCurvilinear-Two_BHs_Collide-Psi4.ipynb writes
 * it as six pieces psi4r_0pt..2pt, psi4i_0pt..2pt): Re psi_4 into
 * psi4_gfs[0], Im psi_4 into psi4_gfs[1] (two gridfunctions of the grid), at
 * interior points with i0_min <= i0 < i0_max (a radial shell or slab; pass
 * -1, -1 for the whole interior).  FP64. */
int BSSN_psi4(const rfm_struct *rfm, const NRGPU_PARAMSTRUCT *params, const double *in_gfs, double *psi4_gfs,
              int i0_min, int i0_max);
/* Spin-weight -2 spherical-harmonic modes of psi_4 on the shell i0 of a
 * Spherical/SinhSpherical grid (driver_psi4_spinweightm2_decomposition and
 * lowlevel_decompose_psi4_into_swm2_modes of the same notebook;
 * SpinWeight_minus2_SphHarmonics.py): modes[2q], modes[2q+1] = Re, Im of
 * sum over interior (theta, phi) of psi4 conj(sY_lm) sin(theta) dxx1 dxx2,
 * q running over l = 2..l_max (<= 12), m = -l..l.  modes: device, 2 *
 * ((l_max+1)^2 - 4) doubles.  psi4_gfs as written by BSSN_psi4. */
int BSSN_psi4_spinweightm2_decomposition(const NRGPU_PARAMSTRUCT *params, const double *psi4_gfs, int i0, int l_max,
                                         double *modes);

/* --------------------------------------------------------- initial data */
/* ScalarWave initial data at ALL points (ScalarWave/InitialData.py:27-88):
 * kind 0 PlaneWave (uu = sin(khat.x - c t) + 2, vv = d uu/dt, khat = kk/|kk|),
 * kind 1 SphericalGaussian (width sigma), at Cartesian positions of the grid's
 * CoordSystem, time `time`, c = params->wavespeed. */
int ScalarWave_initial_data(const NRGPU_PARAMSTRUCT *params, int kind, double time, const double kk[3],
                            double sigma, double *in_gfs);
/* Brill-Lindquist two-puncture data converted to rescaled BSSN variables in
 * the grid's coordinates at ALL points (BrillLindquist.py:48-82,
 * ADM_Exact_Spherical_or_Cartesian_to_BSSNCurvilinear.py:16-135,
 * BSSN_ID_function_string.py:9-45). */
int BSSN_initial_data_BrillLindquist(const NRGPU_PARAMSTRUCT *params,
                                     double BH1_mass, const double BH1_posn[3],
                                     double BH2_mass, const double BH2_posn[3],
                                     double *in_gfs);

/* ------------------------------------------------------- RK4 MoL step */
/* One RK4 step of MoLtimestepping/RK_MoL.h for RK_method "RK4"
 * (C_Code_Generation.py:266-329, Butcher table RK_Butcher_Table_Dictionary.py:86-91):
 * four substeps of RHS -> RK update -> apply_bcs_curvilinear ->
 * (BSSN only) enforce_detgammabar_constraint.  The RK update runs at the
 * interior points, fused into the RHS kernel's epilogue or, for BSSN's
 * staged kernels with FP32 stages and the float-float update
 * (NRGPU_PREC_COMPENSATED, NRGPU_PREC_MIXED), as a separate interior kernel
 * after the RHS kernel stored k (same arithmetic, same bits); ghost points
 * are set by the boundary conditions, as in the reference where every ghost
 * point is a boundary point.  rfm may be NULL for Cartesian grids. */
int MoL_step_forward_in_time(int system, const rfm_struct *rfm, const NRGPU_PARAMSTRUCT *params,
                             const bc_struct *bcstruct, MoL_gridfunctions *gfs, double dt);
/* The same step, unfused, exactly in the reference's order: separate RHS
 * kernel, LOOP_ALL_GFS_GPS update over all points, BCs, rescale. */
int MoL_step_forward_in_time_unfused(int system, const rfm_struct *rfm, const NRGPU_PARAMSTRUCT *params,
                                     const bc_struct *bcstruct, MoL_gridfunctions *gfs, double dt);
/* The kernels of one substep of MoL_step_forward_in_time before its
 * boundary conditions, for timing and profiling a step's dominant kernel.
 * which: 0 every kernel of the substep (the RHS kernel(s) with the RK
 * update), 1 BSSN Ricci_eval only, 2 BSSN rhs_eval only, 3 the RHS
 * kernel(s) without a split step's separate update kernel (the same as 0
 * when the update is fused), 4 that update kernel alone (an error when the
 * step fuses its update).  The buffers must hold a previous step's values
 * (e.g. after one full step). */
int MoL_substep_rhs(int system, const rfm_struct *rfm, const NRGPU_PARAMSTRUCT *params, MoL_gridfunctions *gfs,
                    int stage, double dt, int which);
/* The RK4 step of the reference's Sommerfeld drivers: RHS_string = rhs_eval +
 * apply_bcs_sommerfeld (on the stage's RHS), empty post_RHS_string, the
 * update over every point (C_Code_Generation.py:266-329).  FP64. */
int MoL_step_forward_in_time_sommerfeld(int system, const rfm_struct *rfm, const NRGPU_PARAMSTRUCT *params,
                                        const bc_struct *bcstruct, MoL_gridfunctions *gfs, double dt);
/* Host-buffer form for callers whose state lives in host memory: copies
 * y_n_gfs (host, FP64, pinned or pageable) to gfs->y_n_gfs, runs n_steps
 * steps, copies the state back, and synchronises the stream.  A call that
 * repeats the previous one exactly (same structures' contents, buffers, dt,
 * n_steps <= 16, host array) with a pinned host array replays a CUDA graph
 * of the copies and steps, captured on its second repetition (one graph is
 * kept per process; results are the same bits as the eager call).  Like
 * nrgpu_l2_norm_sq_static, the cached graph belongs to the device's current
 * context: do not call this again after cudaDeviceReset. */
int MoL_evolve_host(int system, const rfm_struct *rfm, const NRGPU_PARAMSTRUCT *params,
                    const bc_struct *bcstruct, MoL_gridfunctions *gfs, double dt,
                    int n_steps, double *y_n_gfs_host);

/* ---------------------------------------------- batched ScalarWave */
/* Many independent curvilinear ScalarWave evolutions (Spherical or
 * SinhSpherical, FD4, NGHOSTS 2, each with its own radial resolution Nr[i]
 * and the shared Ntheta, Nphi) stepped together.  Each instance is exactly the
 * evolution of Tutorial-Start_to_Finish-ScalarWaveCurvilinear.ipynb (RHS
 * ScalarWaveCurvilinear_RHSs.py:43-98, RK4 RK_MoL.h, apply_bcs_curvilinear)
 * with its own find_timestep(CFL_FACTOR) time step; the reference evolves
 * one grid per process and has no batched counterpart.  State arrays are
 * packed instance-major: instance i's gridfunction g starts at
 * base[i] + g*ntot[i] (nrgpu_batch_offsets), nrgpu_batch_total_points
 * values in all.  One RHS launch covers every instance (persistent grid over
 * (instance, i2, i1-block) work items) and one launch per boundary phase
 * covers every instance's ghost zones. */
typedef struct nrgpu_batch nrgpu_batch;
int nrgpu_batch_create(int ninst, const int *Nr, int Ntheta, int Nphi, int CoordSystem,
                       double RMAX, double AMPL, double SINHW, double wavespeed,
                       double CFL_FACTOR, int precision, nrgpu_batch **batch);
int nrgpu_batch_free(nrgpu_batch *batch);
long long nrgpu_batch_total_points(const nrgpu_batch *batch);
/* base[ninst], ntot[ninst]; n0n1n2[3*ninst] (Nxx_plus_2NGHOSTS0..2) may be NULL */
int nrgpu_batch_offsets(const nrgpu_batch *batch, long long *base, long long *ntot, int *n0n1n2);
int nrgpu_batch_timesteps(const nrgpu_batch *batch, double *dt);
int nrgpu_batch_set_timesteps(nrgpu_batch *batch, const double *dt);
/* u = A exp(-(r-r0)^2/w^2), v = 0 at all points of each instance (host
 * arrays A, r0, w of ninst values; y_n_gfs an FP64 device array). */
int nrgpu_batch_initial_data_gaussian(nrgpu_batch *batch, const double *A, const double *r0,
                                      const double *w, double *y_n_gfs);
/* RHS of every instance at interior points (FP64: double in/out; MIXED:
 * float in/out; COMPENSATED: float2 (hi, lo) pairs in, (rhs, 0) pairs out;
 * FP32 arithmetic unless FP64). */
int nrgpu_batch_rhs_eval(nrgpu_batch *batch, const void *in_gfs, void *rhs_gfs);
/* Boundary conditions of every instance; kind 0: float, 1: double, 2: float2 pairs. */
int nrgpu_batch_apply_bcs(nrgpu_batch *batch, void *gfs, int kind);
/* One RK4 step of every instance; gfs->precision must equal the batch's.
 * MIXED: FP32 RHS and FP32 stage buffers, FP64 y_n and running total;
 * COMPENSATED: stage buffers of FP32 pairs (2 floats per value), as in
 * MoL_step_forward_in_time.
 * Neither allocates nor synchronises (graph-capturable). */
int nrgpu_batch_step(nrgpu_batch *batch, MoL_gridfunctions *gfs);
/* Tile autotuner: times the RHS launch for each built tile shape (TX along
 * i0 x TY rows of i1) and persistent grid size, keeps the fastest.  Writes
 * rhs_scratch; synchronises; call outside stream capture. */
int nrgpu_batch_autotune(nrgpu_batch *batch, const void *in_gfs, void *rhs_scratch, int reps,
                         float *best_ms);
int nrgpu_batch_set_tile(nrgpu_batch *batch, int tx, int ty, int grid);
int nrgpu_batch_get_tile(const nrgpu_batch *batch, int *tx, int *ty, int *grid);

/* ------------------------------------------- tangent-linear BSSN (forward mode) */
/* Derivatives of a BSSN evolution with respect to initial-data parameters
 * by forward mode (no counterpart in the reference): a tangent state Y is
 * (ntan + 1) consecutive FP64 state arrays of NUM_EVOL_GFS *
 * Nxx_plus_2NGHOSTS_tot values -- the state, then its derivative along each
 * of ntan parameters (ntan in {0, 1, 2, 4}; 0 is the plain FP64 evolution
 * through the same code).  FD_order 4 on Cartesian and SinhSpherical(v2)
 * grids, FP64, no source terms or dissipation.
 *   BSSN_tangent_rhs_eval: Ricci_eval then rhs_eval of Y and their
 *       derivatives at interior points; aux holds (ntan+1) x 6 RbarDD arrays,
 *       rhs (ntan+1) state arrays.
 *   BSSN_tangent_step: one RK4 step (the reference's unfused order; BCs on
 *       the state and on every tangent, the det(gammabar) rescale and its
 *       linearisation); scratch holds (ntan+1) x 78 x Nxx_plus_2NGHOSTS_tot
 *       doubles.
 *   BSSN_tangent_initial_data_BrillLindquist: the data of
 *       BSSN_initial_data_BrillLindquist in Y[0] and, in Y[k], its
 *       derivative with respect to parameter param_index[k-1]: 0 m1, 1 m2,
 *       2..4 x1[0..2], 5..7 x2[0..2].
 *   BSSN_tangent_shell_accumulate: on the shell i0 (its Nxx1*Nxx2 interior
 *       (i1, i2) points, q = j1 + Nxx1 * j2) of gridfunction gf:
 *       accum[0] += scale sum_q wts[q] (f_q - offset)^2 and
 *       accum[k] += 2 scale sum_q wts[q] (f_q - offset) df_q/dp_k (device). */
int BSSN_tangent_rhs_eval(const rfm_struct *rfmstruct, const NRGPU_PARAMSTRUCT *params, int ntan,
                          const double *in_Y, double *aux, double *rhs_Y);
int BSSN_tangent_step(const rfm_struct *rfmstruct, const NRGPU_PARAMSTRUCT *params, const bc_struct *bcstruct,
                      int ntan, double *Y, double *scratch, double dt);
int BSSN_tangent_initial_data_BrillLindquist(const NRGPU_PARAMSTRUCT *params, double m1, const double x1[3],
                                             double m2, const double x2[3], int ntan, const int *param_index,
                                             double *Y);
int BSSN_tangent_shell_accumulate(const NRGPU_PARAMSTRUCT *params, int ntan, const double *Y, int gf, int i0,
                                  const double *wts, double scale, double offset, double *accum);

/* ------------------------------------------------------------ adjoint */
/* Discrete adjoints of the linear evolutions: Maxwell System I (FP64,
 * Cartesian) and ScalarWave (FP64, Cartesian and the curvilinear families
 * Spherical/SinhSpherical(v2)/Cylindrical/SinhCylindrical(v2)/SymTP/
 * SinhSymTP).  The reference has no adjoint; these are the transposes of
 * the linear maps above, so that gradients of observables of an evolution
 * with respect to its initial data are exact for the discretised problem.
 *   Maxwell_rhs_eval_adjoint, ScalarWave_rhs_eval_adjoint:  adj_in = L^T
 *       adj_rhs at every point, where L is Maxwell_rhs_eval /
 *       ScalarWave(Curvilinear)_rhs_eval (interior rows only); adj_rhs is
 *       read at interior points only.  rfmstruct: as for
 *       ScalarWaveCurvilinear_rhs_eval (NULL on Cartesian grids).
 *   apply_bcs_curvilinear_adjoint:  in place, the transpose of
 *       apply_bcs_curvilinear: ghost adjoints are added onto the points they
 *       were computed from (phases in reverse order) and zeroed.
 *   MoL_adjoint_step_backward:  lam_out = (dy_{n+1}/dy_n)^T lam_in for one
 *       MoL_step_forward_in_time step of `system` (NRGPU_SYS_MAXWELL or
 *       NRGPU_SYS_SCALARWAVE) with extrapolation/parity boundary conditions;
 *       lam_in is overwritten; scratch holds 4 * NUM_EVOL_GFS *
 *       Nxx_plus_2NGHOSTS_tot doubles. */
int Maxwell_rhs_eval_adjoint(const NRGPU_PARAMSTRUCT *params, const double *adj_rhs_gfs, double *adj_in_gfs);
int ScalarWave_rhs_eval_adjoint(const rfm_struct *rfmstruct, const NRGPU_PARAMSTRUCT *params,
                                const double *adj_rhs_gfs, double *adj_in_gfs);
int apply_bcs_curvilinear_adjoint(const NRGPU_PARAMSTRUCT *params, const bc_struct *bcstruct, int NUM_GFS,
                                  const int8_t *gfs_parity, double *adj_gfs);
int MoL_adjoint_step_backward(int system, const rfm_struct *rfmstruct, const NRGPU_PARAMSTRUCT *params,
                              const bc_struct *bcstruct, double *lam_in, double *lam_out, double *scratch,
                              double dt);
/* Toroidal-dipole initial data (Maxwell/InitialData.py:41-104) at all
 * points, and its derivatives with respect to amp and lam (any of the three
 * outputs may be NULL). */
int Maxwell_initial_data_toroidal_dipole(const NRGPU_PARAMSTRUCT *params, double amp, double lam, double time,
                                         double *in_gfs, double *d_in_d_amp, double *d_in_d_lam);
/* Gaussian pulse for ScalarWave at all points of any CoordSystem:
 * uu = A exp(-(r - r0)^2 / w^2), vv = 0, r the Cartesian radius of the point;
 * and its derivatives with respect to A, r0 and w (each output may be NULL;
 * all are 2-gridfunction FP64 arrays). */
int ScalarWave_initial_data_gaussian(const NRGPU_PARAMSTRUCT *params, double A, double r0, double w,
                                     double *in_gfs, double *d_in_d_A, double *d_in_d_r0, double *d_in_d_w);
/* Radial shell of a curvilinear grid: the Nxx1*Nxx2 interior (i1, i2)
 * points of gridfunction gf on the i0 = const shell (i0 an interior index):
 * samples[q] = f(i0, NGHOSTS + q % Nxx1, NGHOSTS + q / Nxx1), and
 * accum[0] += scale * sum_q wts[q] samples[q]^2 (device arrays).
 * nrgpu_shell_sample_adjoint adds the gradient of J = sqrt(accum[0]) for one
 * sample set: adj_gfs[gf] += (scale/J) wts[q] samples[q] at the shell points. */
int nrgpu_shell_sample(const NRGPU_PARAMSTRUCT *params, const double *gfs, int gf, int i0, const double *wts,
                       double scale, double *samples, double *accum);
int nrgpu_shell_sample_adjoint(const NRGPU_PARAMSTRUCT *params, const double *samples, int gf, int i0,
                               const double *wts, double scale, const double *accum, double *adj_gfs);
/* Extraction sphere: tricubic Lagrange interpolation of gridfunctions
 * gf0..gf0+ngf-1 at npts Cartesian points (device array pts[3*npts]) into
 * samples[npts*ngf], and accum[0] += scale * sum_p wts[p] |f(x_p)|^2 (device
 * scalars).  Points whose 4x4x4 stencil leaves the grid set a flag that
 * nrgpu_sphere_check reads (and that the next call clears).
 * nrgpu_sphere_sample_adjoint adds the gradient of J = sqrt(accum[0]) with
 * respect to the sampled gridfunctions for one sample set:
 * adj_gfs += (scale/J) sum_p wts[p] samples[p] (x) interpolation weights. */
int nrgpu_sphere_sample(const NRGPU_PARAMSTRUCT *params, const double *gfs, int gf0, int ngf, const double *pts,
                        const double *wts, int npts, double scale, double *samples, double *accum);
int nrgpu_sphere_sample_adjoint(const NRGPU_PARAMSTRUCT *params, const double *samples, int gf0, int ngf,
                                const double *pts, const double *wts, int npts, double scale,
                                const double *accum, double *adj_gfs);
int nrgpu_sphere_check(const NRGPU_PARAMSTRUCT *params, int *outside);
/* result[0] = sum_i a[i] b[i] (device arrays, FP64, fixed summation order). */
int nrgpu_dot(const double *a, const double *b, long long n, double *scratch, int scratch_len, double *result);

/* --------------------------------------------------------- diagnostics */
/* Sum over interior points of f^2 (and of 1) for gridfunction `gf` of an
 * FP64 array, FP64 accumulation; result[0] = sum f^2, result[1] = count.
 * `result` is a DEVICE pointer to 2 doubles.  Used for the RMS L2 norms of
 * the constraint diagnostics (Tutorial-Start_to_Finish-Solving_Maxwells_
 * Equations_in_Vacuum-Cartesian.ipynb:1089-1106). */
int nrgpu_l2_norm_sq(const NRGPU_PARAMSTRUCT *params, const double *gfs, int gf,
                     double *scratch, int scratch_len, double *result);
/* The same reduction for callers that cannot allocate device memory: host
 * codes that pass this library only the arrays they own and allow no device
 * allocation inside their time loop, and C/Fortran drivers with no device
 * allocator of their own.  No counterpart in the reference.  Its partial sums
 * live in a fixed 2048-double (16 KB) device array inside the library, held
 * by every GPU that loads it until the process exits; a call that would need
 * more partials fails with NRGPU_ERR_SIZE.  The first call on a device looks
 * up that array's device address (cudaGetSymbolAddress) with the device
 * current, so make the first call before any stream capture.  The cached
 * address is that context's: after cudaDeviceReset (or any teardown of the
 * device's primary context) it is stale, so do not call this entry point
 * again in that process.  All calls share the array, so calls that overlap
 * on the GPU race; no cudaMalloc/cudaFree. */
int nrgpu_l2_norm_sq_static(const NRGPU_PARAMSTRUCT *params, const double *gfs, int gf, double *result);

#ifdef __cplusplus
}
#endif
#endif /* NRGPU_H */
