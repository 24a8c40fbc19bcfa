/* mol_ref.c -- CPU restatement (OpenMP C) of the non-generated parts of the
 * reference's RK4 step, used with the reference-generated kernels for the
 * timed CPU baseline.  TEST INFRASTRUCTURE: only bench.py's reference leg
 * and tests call it.
 *
 *  ref_rk4_update   the LOOP_ALL_GFS_GPS update of RK_MoL.h for "RK4"
 *                   (MoLtimestepping/C_Code_Generation.py:277-329)
 *  ref_apply_bcs    apply_bcs_curvilinear
 *                   (CurviBoundaryConditions/boundary_conditions/
 *                   apply_bcs_curvilinear.h:19-64) over a flattened map:
 *                   per layer, outer points (dest, step) then inner points
 *                   (dest, src, parity bits), OpenMP over gridfunctions.
 */
#include <stdint.h>

void ref_rk4_update(int stage, double dt, long long n, double *y_n, double *rt, double *k) {
#pragma omp parallel for
  for (long long i = 0; i < n; i++) {
    switch (stage) {
      case 0:
        rt[i] = k[i] * dt * (1.0 / 6.0);
        k[i] = y_n[i] + k[i] * dt * (1.0 / 2.0);
        break;
      case 1:
        rt[i] = rt[i] + k[i] * dt * (1.0 / 3.0);
        k[i] = y_n[i] + k[i] * dt * (1.0 / 2.0);
        break;
      case 2:
        rt[i] = rt[i] + k[i] * dt * (1.0 / 3.0);
        k[i] = y_n[i] + k[i] * dt;
        break;
      default:
        y_n[i] = y_n[i] + rt[i] + k[i] * dt * (1.0 / 6.0);
        break;
    }
  }
}

void ref_apply_bcs(int nghosts, const int *ob_start /* [nghosts+1] */, const int *outer_dest,
                   const int *outer_step, const int *ib_start /* [nghosts+1] */, const int *inner_dest,
                   const int *inner_src, const int *inner_parity, int ngfs, const int8_t *gf_parity,
                   long long ntot, double *gfs) {
#pragma omp parallel for
  for (int g = 0; g < ngfs; g++) {
    double *f = gfs + (long long)g * ntot;
    for (int gz = 0; gz < nghosts; gz++) {
      for (int p = ob_start[gz]; p < ob_start[gz + 1]; p++) {
        const long long d = outer_dest[p], s = outer_step[p];
        f[d] = +3.0 * f[d + s] - 3.0 * f[d + 2 * s] + 1.0 * f[d + 3 * s];
      }
      for (int p = ib_start[gz]; p < ib_start[gz + 1]; p++) {
        const int neg = (inner_parity[p] >> gf_parity[g]) & 1;
        f[inner_dest[p]] = (neg ? -1.0 : 1.0) * f[inner_src[p]];
      }
    }
  }
}
