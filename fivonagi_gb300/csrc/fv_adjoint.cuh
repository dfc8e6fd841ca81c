// fv_adjoint.cuh -- reverse-mode (adjoint) versions of the step's local
// operations, derived by hand from fv_device.cuh.
//
// Each function recomputes its forward values from the same inputs, then
// propagates output adjoints back to input adjoints. Branches are replayed
// from the recomputed forward values: the sign of each wave speed (which of
// amdq/apdq a wave feeds, apps/na/fv.h:148-180), the upwind side and the
// min/max branch of the MC limiter (fv.h:587-662), the interior masks. dt
// is a frozen input (the adjoint follows the forward run's dt schedule), so
// nothing flows through the CFL. The rounding of u1 through (u1 + 1) - 1 in
// the diffusion step (apps/na/source.h:84) has derivative 1.
#pragma once

#include "fv_device.cuh"

namespace fvgb {

// Division of the reverse pass: PTX div.full.f32, a full-range quotient
// within 2 ulp, without the operand-dependent slow path of IEEE division.
// The reverse kernels use the forward values only as the point where the
// step is linearised. The branches they replay (signs of wave speeds,
// limiter branches) can differ from the forward's only where a value lies
// within a few ulps of the branch point, and there both branches give
// nearly the same derivative.
__device__ __forceinline__ float fdiv(float a, float b) {
  float q;
  asm("div.full.f32 %0, %1, %2;" : "=f"(q) : "f"(a), "f"(b));
  return q;
}

// The division policy of fv_device.cuh's riemann() and mc_limit() for
// the reverse pass's recomputation: fdiv everywhere.
struct DivFast {
  static constexpr bool kFlags = false;
  struct Rcp {
    float b;
  };
  __device__ __forceinline__ Rcp recip(float b) { return Rcp{b}; }
  __device__ __forceinline__ float div_r(float a, const Rcp &rb) { return fdiv(a, rb.b); }
  __device__ __forceinline__ float div(float a, float b) { return fdiv(a, b); }
  __device__ __forceinline__ float ratio(float a, float b) { return fdiv(a, b); }
  __device__ __forceinline__ bool unsafe() const { return false; }
};

// Adjoint of one cell in a sweep's local frame: component 1 = u1,
// 2 = normal momentum, 3 = transverse momentum.
struct Adj3 {
  float q1, qn, qt;
};

struct WaveAdj {
  float s1, s2, s3;
  float w11, w21, w31, w12, w22, w32, w33;
};

struct FluctAdj {
  float am1, am2, am3, ap1, ap2, ap3;
};

__device__ __forceinline__ void zero(WaveAdj &a) {
  a.s1 = a.s2 = a.s3 = 0.f;
  a.w11 = a.w21 = a.w31 = a.w12 = a.w22 = a.w32 = a.w33 = 0.f;
}

// Reverse of riemann() for the interface between cell b and cell a (q* are
// the cells' local-frame states, u1 = rho - 1). Adds the input adjoints to
// ga (cell a) and gb (cell b).
__device__ __forceinline__ void riemann_adj(float q1a, float qna, float qta, float q1b, float qnb,
                                            float qtb, float two_bm1, const WaveAdj &gw,
                                            const FluctAdj &gf, Adj3 &ga, Adj3 &gb) {
  // ---- forward
  const float ra = q1a + 1.0f, rb = q1b + 1.0f;
  const float vna = fdiv(qna, ra), vta = fdiv(qta, ra), vnb = fdiv(qnb, rb), vtb = fdiv(qtb, rb);
  const float Z1 = (ra + rb) * 0.5f;
  const float Zn = (vna + vnb) * 0.5f;
  const float Zt = (vta + vtb) * 0.5f;
  const float tmp1 = fdiv(Zn, Z1);
  const float tmp2 = fdiv(Zn * Zn, Z1);
  const float tmp3 = tmp1 * tmp1 - 2.0f * tmp2 + 1.0f + two_bm1 * (Z1 - 1.0f);
  const float sq = sqrtf(tmp3);
  const float L1 = tmp1 + sq, L2 = tmp1 - sq, L3 = tmp1;
  const float N1 = L1 * Zt - 2.0f * Zn * Zt, D1 = L1 * Z1 - Zt;
  const float N2 = L2 * Zt - 2.0f * Zn * Zt, D2 = L2 * Z1 - Zt;
  const float A1 = fdiv(N1, D1), A2 = fdiv(N2, D2);
  const float drho = ra - rb, dun = qna - qnb;
  const float Da = L1 - L2;
  const float a1 = fdiv(dun - drho * L2, Da);
  const float a2 = drho - a1;
  const float N3 = (L1 * A2 - L2 * A1) * drho + (A1 - A2) * dun;
  const float D3 = L2 - L1;
  const float q3 = fdiv(N3, D3);
  const float a3 = q3 + qta - qtb;
  // ---- reverse
  // fluctuations: each wave feeds amdq if its speed is negative, apdq if positive
  const float m11 = L1 < 0.f ? gf.am1 : (L1 > 0.f ? gf.ap1 : 0.f);
  const float m12 = L1 < 0.f ? gf.am2 : (L1 > 0.f ? gf.ap2 : 0.f);
  const float m13 = L1 < 0.f ? gf.am3 : (L1 > 0.f ? gf.ap3 : 0.f);
  const float m21 = L2 < 0.f ? gf.am1 : (L2 > 0.f ? gf.ap1 : 0.f);
  const float m22 = L2 < 0.f ? gf.am2 : (L2 > 0.f ? gf.ap2 : 0.f);
  const float m23 = L2 < 0.f ? gf.am3 : (L2 > 0.f ? gf.ap3 : 0.f);
  const float m33 = L3 < 0.f ? gf.am3 : (L3 > 0.f ? gf.ap3 : 0.f);
  float gL1 = gw.s1 + m11 * a1 + m12 * 2.0f * L1 * a1 + m13 * a1 * A1 + gw.w21 * a1;
  float gL2 = gw.s2 + m21 * a2 + m22 * 2.0f * L2 * a2 + m23 * a2 * A2 + gw.w22 * a2;
  float gL3 = gw.s3 + m33 * a3;
  float ga1 = m11 * L1 + m12 * L1 * L1 + m13 * L1 * A1 + gw.w11 + gw.w21 * L1 + gw.w31 * A1;
  float ga2 = m21 * L2 + m22 * L2 * L2 + m23 * L2 * A2 + gw.w12 + gw.w22 * L2 + gw.w32 * A2;
  float ga3 = m33 * L3 + gw.w33;
  float gA1 = m13 * L1 * a1 + gw.w31 * a1;
  float gA2 = m23 * L2 * a2 + gw.w32 * a2;
  // a3 = N3 / D3 + qta - qtb
  float gqta = ga3, gqtb = -ga3;
  const float gN3 = fdiv(ga3, D3);
  const float gD3 = fdiv(-ga3 * q3, D3);
  gL2 += gD3;
  gL1 -= gD3;
  gL1 += gN3 * A2 * drho;
  gA2 += gN3 * L1 * drho;
  gL2 -= gN3 * A1 * drho;
  gA1 -= gN3 * L2 * drho;
  float gdrho = gN3 * (L1 * A2 - L2 * A1);
  gA1 += gN3 * dun;
  gA2 -= gN3 * dun;
  float gdun = gN3 * (A1 - A2);
  // a2 = drho - a1
  gdrho += ga2;
  ga1 -= ga2;
  // a1 = (dun - drho L2) / (L1 - L2)
  const float gNa = fdiv(ga1, Da);
  const float gDa = fdiv(-ga1 * a1, Da);
  gdun += gNa;
  gdrho -= gNa * L2;
  gL2 -= gNa * drho;
  gL1 += gDa;
  gL2 -= gDa;
  // A1 = N1 / D1, A2 = N2 / D2
  float gZ1 = 0.f, gZn = 0.f, gZt = 0.f;
  {
    const float gN = fdiv(gA1, D1), gD = fdiv(-gA1 * A1, D1);
    gL1 += gN * Zt + gD * Z1;
    gZt += gN * (L1 - 2.0f * Zn) - gD;
    gZn -= gN * 2.0f * Zt;
    gZ1 += gD * L1;
  }
  {
    const float gN = fdiv(gA2, D2), gD = fdiv(-gA2 * A2, D2);
    gL2 += gN * Zt + gD * Z1;
    gZt += gN * (L2 - 2.0f * Zn) - gD;
    gZn -= gN * 2.0f * Zt;
    gZ1 += gD * L2;
  }
  // L1 = tmp1 + sq, L2 = tmp1 - sq, L3 = tmp1
  float gtmp1 = gL1 + gL2 + gL3;
  const float gsq = gL1 - gL2;
  const float gtmp3 = fdiv(gsq, 2.0f * sq);
  gtmp1 += gtmp3 * 2.0f * tmp1;
  const float gtmp2 = -2.0f * gtmp3;
  gZ1 += gtmp3 * two_bm1;
  // tmp2 = Zn^2 / Z1, tmp1 = Zn / Z1
  gZn += fdiv(gtmp2 * 2.0f * Zn, Z1) + fdiv(gtmp1, Z1);
  gZ1 -= fdiv(gtmp2 * tmp2, Z1) + fdiv(gtmp1 * tmp1, Z1);
  // means
  float gra = 0.5f * gZ1, grb = 0.5f * gZ1;
  const float gvna = 0.5f * gZn, gvnb = 0.5f * gZn, gvta = 0.5f * gZt, gvtb = 0.5f * gZt;
  // drho, dun
  gra += gdrho;
  grb -= gdrho;
  float gqna = gdun, gqnb = -gdun;
  // v = q / rho
  gqna += fdiv(gvna, ra);
  gqta += fdiv(gvta, ra);
  gra -= fdiv(gvna * vna + gvta * vta, ra);
  gqnb += fdiv(gvnb, rb);
  gqtb += fdiv(gvtb, rb);
  grb -= fdiv(gvnb * vnb + gvtb * vtb, rb);
  ga.q1 += gra;
  ga.qn += gqna;
  ga.qt += gqta;
  gb.q1 += grb;
  gb.qn += gqnb;
  gb.qt += gqtb;
}

// Derivative of the MC limiter phi(r) of fv.h:587-605 (the branches the
// forward value took; 0 where phi is the constant 1 of a zero wave).
__device__ __forceinline__ float mc_limit_dphi(float r) {
  const float c = (1.0f + r) / 2.0f;
  const float r2 = 2.0f * r;
  const float w1 = gmin(c, 2.0f);
  const float dw1 = (c < 2.0f) ? 0.5f : 0.0f;
  const float w = gmin(w1, r2);
  const float dw = (w1 < r2) ? dw1 : 2.0f;
  return (w > 0.0f) ? dw : 0.0f;
}

// Reverse of correction() at interface k: from the adjoint of its flux
// (gf1..gf3), add adjoints to the waves at k-1 (gm), k (g0), k+1 (gp).
__device__ __forceinline__ void correction_adj(const WaveN &wm, const WaveN &w0, const WaveN &wp,
                                               float dtx, float gf1, float gf2, float gf3,
                                               WaveAdj &gm, WaveAdj &g0, WaveAdj &gp) {
  // forward per wave p: n_p = |W_p|^2, d_p = W_p . W_p(upwind), r = d/n,
  // phi_p, g_p = |s_p|(1 - |s_p| dtx), f_k = 0.5 sum_p g_p W_kp phi_p
  const float s[3] = {w0.s1, w0.s2, w0.s3};
  const float W0[3][3] = {{w0.w11, w0.w12, 0.f}, {w0.w21, w0.w22, 0.f}, {w0.w31, w0.w32, w0.w33}};
  const float WM[3][3] = {{wm.w11, wm.w12, 0.f}, {wm.w21, wm.w22, 0.f}, {wm.w31, wm.w32, wm.w33}};
  const float WP[3][3] = {{wp.w11, wp.w12, 0.f}, {wp.w21, wp.w22, 0.f}, {wp.w31, wp.w32, wp.w33}};
  const float gf[3] = {gf1, gf2, gf3};
  float g0W[3][3] = {{0.f}}, gmW[3][3] = {{0.f}}, gpW[3][3] = {{0.f}};
  float gs[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    const float n = W0[0][p] * W0[0][p] + W0[1][p] * W0[1][p] + W0[2][p] * W0[2][p];
    const bool up = s[p] > 0.0f;  // upwind neighbour: k-1 for positive speed
    const float dl = W0[0][p] * WM[0][p] + W0[1][p] * WM[1][p] + W0[2][p] * WM[2][p];
    const float dr = W0[0][p] * WP[0][p] + W0[1][p] * WP[1][p] + W0[2][p] * WP[2][p];
    const float d = up ? dl : dr;
    const bool nz = n != 0.0f;
    const float r = nz ? fdiv(d, n) : 0.0f;
    DivFast fast;
    const float phi = nz ? mc_limit(n, dl, dr, s[p], fast) : 1.0f;
    const float as = fabsf(s[p]);
    const float g = as * (1.0f - as * dtx);
    // f_k = 0.5 sum_p g_p W_kp phi_p
    float gphi = 0.f, gg = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      g0W[k][p] += 0.5f * gf[k] * g * phi;
      gphi += 0.5f * gf[k] * g * W0[k][p];
      gg += 0.5f * gf[k] * W0[k][p] * phi;
    }
    // g = |s| - |s|^2 dtx
    const float sgn = s[p] > 0.0f ? 1.0f : (s[p] < 0.0f ? -1.0f : 0.0f);
    gs[p] += gg * (1.0f - 2.0f * as * dtx) * sgn;
    if (nz) {
      const float gr = gphi * mc_limit_dphi(r);
      const float gd = fdiv(gr, n);
      const float gn = fdiv(-gr * r, n);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        g0W[k][p] += 2.0f * W0[k][p] * gn;
        if (up) {
          g0W[k][p] += gd * WM[k][p];
          gmW[k][p] += gd * W0[k][p];
        } else {
          g0W[k][p] += gd * WP[k][p];
          gpW[k][p] += gd * W0[k][p];
        }
      }
    }
  }
  g0.s1 += gs[0];
  g0.s2 += gs[1];
  g0.s3 += gs[2];
  g0.w11 += g0W[0][0]; g0.w21 += g0W[1][0]; g0.w31 += g0W[2][0];
  g0.w12 += g0W[0][1]; g0.w22 += g0W[1][1]; g0.w32 += g0W[2][1];
  g0.w33 += g0W[2][2];
  gm.w11 += gmW[0][0]; gm.w21 += gmW[1][0]; gm.w31 += gmW[2][0];
  gm.w12 += gmW[0][1]; gm.w22 += gmW[1][1]; gm.w32 += gmW[2][1];
  gm.w33 += gmW[2][2];
  gp.w11 += gpW[0][0]; gp.w21 += gpW[1][0]; gp.w31 += gpW[2][0];
  gp.w12 += gpW[0][1]; gp.w22 += gpW[1][1]; gp.w32 += gpW[2][1];
  gp.w33 += gpW[2][2];
}

}  // namespace fvgb
