// pairfn.cuh -- the pair plug-in: the counterpart of the reference's
// External :: user_func (SRC/exaMD_forces.f90:532), with its contract
// (:534-549).  Given r^2 of d = x_j - x_i, a pair function returns dg with
// f_i = dg * d and f_j = -f_i, the pair energy e, and a status:
//   0    apply the pair,
//   > 0  skip it (beyond the potential's range; the reference's retval = 1),
//   < 0  error: the kernel records it and the host returns EXAMD_ERR_PAIRFN
//        (the reference prints "Error from user_func" and goes on).
// The potential is chosen per context (examd_params.potential, warp-uniform).
// Its parameters per ordered type pair are filled in examd_gpu_create: the
// LJ family (EXAMD_POT_LJ, _LJ_SHIFTED, _WCA) shares one expression and
// differs in range (rcut2) and energy shift (eshift).  A new functional form
// is a new EXAMD_POT_* value, its parameter row, and a case here in both
// precisions.
#pragma once

#include "common.cuh"

namespace examd {

// Coincident atoms: the force is undefined for every potential.
constexpr float kR2Min32 = 1e-12f;
constexpr double kR2Min64 = 1e-12;

// Mixed form, FP32: user_func.f90:58-69 with a fast reciprocal.
template <bool ENERGY>
__device__ __forceinline__ int pair_fn32(int pot, float d2, const LJ32& P, float& dg, float& e) {
  switch (pot) {
    case EXAMD_POT_LJ:
    case EXAMD_POT_LJ_SHIFTED:
    case EXAMD_POT_WCA: {
      if (!(d2 >= kR2Min32)) return -1;
      if (d2 > P.rcut2) return 1;
      const float ri = rcp_approx(d2);
      const float s2 = P.sig2 * ri;
      const float s6 = s2 * s2 * s2;
      dg = P.m24eps * s6 * fmaf(2.f, s6, -1.f) * ri;
      if (ENERGY) e = P.c4eps * s6 * (s6 - 1.f) - P.eshift;
      return 0;
    }
    default:
      return -2;
  }
}

// FP64 form: the reference's arithmetic and operation order (user_func.f90:
// 52-69): d2i = 1/d2, d6 = (sig2 d2i)^3, d12 = d6^2, dg = -eps24 (2 d12 - d6) d2i.
template <bool ENERGY>
__device__ __forceinline__ int pair_fn64(int pot, double d2, const LJ64& P, double& dg, double& e) {
  switch (pot) {
    case EXAMD_POT_LJ:
    case EXAMD_POT_LJ_SHIFTED:
    case EXAMD_POT_WCA: {
      if (!(d2 >= kR2Min64)) return -1;
      if (d2 > P.rcut2) return 1;  // If (d2 > prmvdw(1,5)**2) retval = 1 (user_func.f90:52-53)
      const double d2i = __drcp_rn(d2);
      const double tt = __dmul_rn(P.sig2, d2i);
      const double d6 = __dmul_rn(__dmul_rn(tt, tt), tt);
      const double d12 = __dmul_rn(d6, d6);
      dg = -__dmul_rn(__dmul_rn(P.eps24, __dsub_rn(__dmul_rn(2.0, d12), d6)), d2i);
      if (ENERGY) e = __dsub_rn(__dmul_rn(P.eps4, __dsub_rn(d12, d6)), P.eshift);
      return 0;
    }
    default:
      return -2;
  }
}

}  // namespace examd
