// systems.cuh -- internal interface between the MoL driver and the per-system
// RHS launchers.
#pragma once
#include "common.cuh"

namespace nrgpu {

// One RHS evaluation, with either a plain store (stage < 0) or the fused RK4
// update of substep `stage` as its epilogue.
struct StageArgs {
  int stage;          // -1 plain rhs_eval, 0..3 RK4 substep
  double dt;
  int prec;           // NRGPU_PREC_FP64 or NRGPU_PREC_MIXED (FP32 arithmetic)
  const void *in;     // stage input gfs
  bool in_is_f64;     // type of *in
  double *y_n;        // FP64 state (fused stages)
  double *rt;         // FP64 running total (fused stages)
  void *out;          // output: FP64 if prec==FP64 else FP32
  void *auxevol;      // BSSN: RbarDD (same type as out)
};

int scalarwave_launch(const rfm_struct *rfm, const paramstruct *p, const StageArgs &a);
int maxwell_launch(const paramstruct *p, const StageArgs &a);
int bssn_ricci_launch(const rfm_struct *rfm, const paramstruct *p, const void *in, bool in_is_f64,
                      int prec, void *auxevol);
int bssn_rhs_launch(const rfm_struct *rfm, const paramstruct *p, const StageArgs &a);
int bssn_enforce_launch(const rfm_struct *rfm, const paramstruct *p, void *gfs, bool is_f64);

// Evolved-gridfunction counts and parity types (alphabetical gf order;
// parity types from CurviBoundaryConditions.py:122-213).
int system_num_gfs(int system);
const int8_t *system_parity(int system);

}  // namespace nrgpu
