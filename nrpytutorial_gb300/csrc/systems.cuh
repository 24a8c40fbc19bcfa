// systems.cuh -- internal interface between the MoL driver and the per-system
// RHS launchers.
#pragma once
#include <type_traits>

#include "common.cuh"
#include "fd.cuh"

namespace nrgpu {

// One RHS evaluation, with either a plain store (stage < 0) or the fused RK4
// update of substep `stage` as its epilogue.
struct StageArgs {
  int stage;          // -1 plain rhs_eval, 0..3 RK4 substep
  double dt;
  int prec;           // NRGPU_PREC_FP64, or FP32 arithmetic (MIXED, COMPENSATED;
                      // COMPENSATED: *in and *out are float2 pair arrays)
  const void *in;     // stage input gfs
  bool in_is_f64;     // type of *in
  double *y_n;        // FP64 state (fused stages)
  double *rt;         // FP64 running total (fused stages)
  void *out;          // output: FP64 if prec==FP64 else FP32
  void *auxevol;      // BSSN: RbarDD (same type as out)
};

// The kernel-side input of a stage (a float2 pair array for Pair32).
template <typename Tin> inline typename InRef<Tin>::type stage_input(const StageArgs &a) {
  if constexpr (std::is_same<Tin, Pair32>::value) return (const float2 *)a.in;
  else return (const Tin *)a.in;
}

int scalarwave_launch(const rfm_struct *rfm, const paramstruct *p, const StageArgs &a);
int maxwell_launch(const paramstruct *p, const StageArgs &a);
int maxwell_curvi_launch(const rfm_struct *rfm, const paramstruct *p, const StageArgs &a);
int bssn_ricci_launch(const rfm_struct *rfm, const paramstruct *p, const void *in, bool in_is_f64,
                      int prec, void *auxevol);
int bssn_rhs_launch(const rfm_struct *rfm, const paramstruct *p, const StageArgs &a);
int bssn_stage_launch(const rfm_struct *rfm, const paramstruct *p, const StageArgs &a);
// Whether a BSSN step stores the RHS and runs the RK update as a separate
// interior kernel instead of the RHS kernel's epilogue.
bool bssn_split_update(const paramstruct *p, int prec);
// The BSSN kernel selection (nrgpu_set_bssn_kernels).
int bssn_kernels_mode();
// is_f64: double array; otherwise float, or float2 pairs when pair is set
// ff_f64: FP64 data rescaled in float-float arithmetic (the FP32-stage steps' state)
// f64_pair: pair data rescaled in FP64 arithmetic (COMPENSATED_FP64RK stages)
int bssn_enforce_launch(const rfm_struct *rfm, const paramstruct *p, void *gfs, bool is_f64, bool pair = false,
                        bool ff_f64 = false, bool f64_pair = false);

// Evolved-gridfunction counts and parity types (alphabetical gf order;
// parity types from CurviBoundaryConditions.py:122-213).
int system_num_gfs(int system);
const int8_t *system_parity(int system);

// Boundary conditions on FP32 pair gridfunctions: ghost values computed in
// FP64 from the pairs and stored back as pairs.
int apply_bcs_pair_impl(const paramstruct *p, const bc_struct *bc, int NUM_GFS, const int8_t *gfs_parity,
                        float2 *gfs);
// Sommerfeld radiation condition on rhs from the state gfs (FP64); xx may be
// NULL (cell-centred coordinates from params).
int apply_sommerfeld_impl(const paramstruct *p, double *const xx[3], const bc_struct *bc, int NUM_GFS,
                          const int8_t *gfs_parity, const double *gfs, double *rhs);
// Transpose of the boundary conditions (FP64), in place: ghost adjoints are
// moved onto their sources and zeroed.
int apply_bcs_adjoint_impl(const paramstruct *p, const bc_struct *bc, int NUM_GFS, const int8_t *gfs_parity,
                           double *gfs);

}  // namespace nrgpu
