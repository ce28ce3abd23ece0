// green32.cuh -- one entry of the SCHEFF Green's table in FP32 (the ring's
// E_r, E_z per unit charge before the c1 scale), shared by the FP32 solver's
// table and the field surrogate's spot solve.
#pragma once

#include "common.cuh"

namespace hps {

// UpdateFldTbl1Kernel (space_charge_kernel.cu:39-100) in FP32.  With
// b = (rp + rs)^2, c = (rp - rs)^2 and the complementary parameter
// g = 1 - 4 rs rp / (b + d^2) = (c + d^2) / (b + d^2) (no cancellation), the
// reference's radial term  ek - (rs^2 - rp^2 + d^2) ee / (c + d^2)  equals
// (ek - ee) - ee 2 rp (rs - rp) / (c + d^2).  ek - ee is the difference of
// the two fits re-expanded in m = 1 - g = 4 rs rp / (b + d^2) and
// h = log(g) = log1p(-m):
//   ek - ee = C0 + m (Cm + Cmm m) + h (Ch + m (Chm + Chmm m)),
// with the coefficients formed exactly from the fits' (C0 = 6e-8 is the fits'
// own residual at m = 0), so the far field (ek - ee = O(m)) is not a
// difference of two O(1) values.  Rows rs >= (nr/by)*by are not written, as
// in the reference's grid.
struct GreenTerm { float er, ez; };
__device__ inline GreenTerm green_term(float rs, float rp, float d) {
  const float d2 = d * d;
  const float c = (rp - rs) * (rp - rs), b = (rp + rs) * (rp + rs);
  const float inv = 1.0f / (b + d2);
  const float g = (c + d2) * inv, m = 4.0f * rs * rp * inv;
  const float h = m < 0.5f ? log1pf(-m) : logf(g);
  const float ee = 1.0f + g * (0.4630106f - 0.2452740f * h + g * (0.1077857f - 0.04125321f * h));
  // D0..D5 = ek - ee coefficients of 1, h, g, g h, g^2, g^2 h:
  //   0.38629436, -0.5, -0.3510409, 0.1239254, -0.0352534, 0.01237849
  // C0 = D0+D2+D4, Ch = D1+D3+D5, Cm = -D2-2D4, Chm = -D3-2D5, Cmm = D4, Chmm = D5
  const float dke = 6.0e-8f + m * (0.4215477f - 0.0352534f * m) +
                    h * (-0.36369611f + m * (-0.14868238f + 0.01237849f * m));
  const float a = sqrtf(b + d2);
  GreenTerm t;
  t.er = rp != 0.0f ? (dke - ee * 2.0f * rp * (rs - rp) / (c + d2)) / (2.0f * rp * a) : 0.0f;
  t.ez = d * ee / (a * (c + d2));
  return t;
}


}  // namespace hps
