// Split-axis Riemann fluxes and thermodynamics of the density-based path.
//
// T = double compiled without FMA contraction (kernels_exact.cu) rounds
// every operation in the order the reference evaluates it, so the face
// fluxes are bit-identical to the reference's:
//   work/FUNCTION.cpp:3-15            getP / getht (2D momentum only)
//   rhoSolver/SolverAusm.cpp:3-26, :53-63, :105-143   AUSM+
//   rhoSolver/SolverRoe.cpp:3-16, :70-111, :114-123   Roe, |A| = R|L|R^-1
// The same code compiled with FMA (kernels_fast.cu) gives the FP64 and
// FP32 production variants.
#pragma once
#include <cuda_runtime.h>

namespace mst {

template <class T>
struct Gas {
  // gamma = 1.4 is fixed by the reference (CONST.h:41)
  static __host__ __device__ __forceinline__ T gamma() { return T(1.4); }
  static __host__ __device__ __forceinline__ T gm1() { return T(1.4) - T(1); }
  static __host__ __device__ __forceinline__ T gp1() { return T(1.4) + T(1); }
};

template <class T>
__host__ __device__ __forceinline__ T th_p(const T q[4]) {
  T ke = T(0.5) * (q[1] * q[1] + q[2] * q[2]) / q[0];
  return (q[3] - ke) * Gas<T>::gm1();
}
template <class T>
__host__ __device__ __forceinline__ T th_ht(const T q[4]) {
  T p = th_p(q);
  return (q[3] + p) / q[0];
}

// Per-state quantities of the AUSM+ flux that do not depend on the axis
// (SolverAusm.cpp:6-25 set(), :107-113): pressure, total enthalpy, the
// critical-speed interface estimate a*^2/max(a*,|U|), the true sound speed,
// and the convected vector (rho, rho u, rho v, rho H).  Computing them once
// per face state and reusing them for both axes gives the same values as
// the reference's per-axis recomputation.
template <class T>
struct AusmSide {
  T p, a_face, a_true, fc[4];
};

template <class T>
__host__ __device__ __forceinline__ AusmSide<T> ausm_side(const T q[4]) {
  const T g = Gas<T>::gamma(), gm1 = Gas<T>::gm1(), gp1 = Gas<T>::gp1();
  AusmSide<T> s;
  s.p = th_p(q);
  const T h = (q[3] + s.p) / q[0];
  const T as = sqrt(T(2) * h * gm1 / gp1);
  const T U = sqrt((q[1] * q[1] + q[2] * q[2]) / q[0] / q[0]);
  s.a_face = as * as / (as < U ? U : as);
  s.a_true = sqrt(g * s.p / q[0]);
  s.fc[0] = q[0];
  s.fc[1] = q[1];
  s.fc[2] = q[2];
  s.fc[3] = q[3] + s.p;
  return s;
}

// AUSM+ flux along axis d (0 = x, 1 = y) from the two sides' quantities;
// ql, qr are the states themselves (for the Mach numbers).
template <class T>
__host__ __device__ __forceinline__ void ausm_axis(const T ql[4], const AusmSide<T>& L,
                                                   const T qr[4], const AusmSide<T>& R,
                                                   int d, T f[4]) {
  const T aF = (R.a_face < L.a_face) ? R.a_face : L.a_face;
  const T mL = ql[d + 1] / ql[0] / aF;
  const T mR = qr[d + 1] / qr[0] / aF;
  const T pL = L.p, pR = R.p, aL = L.a_true, aR = R.a_true;
  T mp, mm, pp, pm;
  // the reference's abs(mach <= 1) is the plain test mach <= 1
  if (mL <= T(1)) {
    mp = T(0.25) * (mL + T(1)) * (mL + T(1)) +
         T(0.125) * (mL * mL - T(1)) * (mL * mL - T(1));
    pp = pL * T(0.25) * (mL + T(1)) * (mL + T(1)) * (T(2) - mL) +
         T(0.1875) * mL * (mL * mL - T(1)) * (mL * mL - T(1));
  } else {
    mp = T(0.5) * (mL + fabs(mL));
    pp = pL * T(0.5) * (mL + fabs(mL)) / mL;
  }
  if (mR <= T(1)) {
    mm = T(-0.25) * (mR - T(1)) * (mR - T(1)) -
         T(0.125) * (mR * mR - T(1)) * (mR * mR - T(1));
    pm = pR * T(0.25) * (mR - T(1)) * (mR - T(1)) * (T(2) + mR) -
         T(0.1875) * mR * (mR * mR - T(1)) * (mR * mR - T(1));
  } else {
    mm = T(0.5) * (mR - fabs(mR));
    pm = pR * T(0.5) * (mR - fabs(mR)) / mR;
  }
  const T mF = mm + mp;
  const T pF = pm + pp;
  const T amF = fabs(mF);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    T a = mF * (aL * L.fc[k] + aR * R.fc[k]);
    T b = amF * (aR * R.fc[k] - aL * L.fc[k]);
    f[k] = T(0.5) * (a - b);
  }
  f[d + 1] += pF;
}

// The same AUSM+ quantities for the FP32 production path, with each
// state's 1/rho computed once and the supersonic branches in closed form
// ((M + |M|) / (2M) = 1 for M > 1, (M - |M|) = 0): fewer divisions, the
// same formulas as ausm_axis (including the pressure polynomial whose
// second term is not scaled by p) up to rounding.  Not used by the exact
// path.
struct AusmSideF {
  float ir, p, a_face, a_true, fc[4];
};

__host__ __device__ __forceinline__ AusmSideF ausm_side_f(const float q[4]) {
  AusmSideF s;
  const float gm1 = Gas<float>::gm1();
  s.ir = 1.0f / q[0];
  const float m2 = q[1] * q[1] + q[2] * q[2];
  s.p = (q[3] - 0.5f * m2 * s.ir) * gm1;
  const float h = (q[3] + s.p) * s.ir;
  const float as = sqrtf(h * (2.0f * gm1 / Gas<float>::gp1()));
  const float U = sqrtf(m2) * s.ir;
  s.a_face = as * as / fmaxf(as, U);
  s.a_true = sqrtf(Gas<float>::gamma() * s.p * s.ir);
  s.fc[0] = q[0];
  s.fc[1] = q[1];
  s.fc[2] = q[2];
  s.fc[3] = q[3] + s.p;
  return s;
}

__host__ __device__ __forceinline__ void ausm_axis_f(const float ql[4], const AusmSideF& L,
                                                     const float qr[4], const AusmSideF& R, int d,
                                                     float f[4]) {
  const float iaF = 1.0f / fminf(R.a_face, L.a_face);
  const float mL = ql[d + 1] * L.ir * iaF;
  const float mR = qr[d + 1] * R.ir * iaF;
  float mp, mm, pp, pm;
  if (mL <= 1.0f) {
    const float a = (mL + 1.0f) * (mL + 1.0f), b = (mL * mL - 1.0f) * (mL * mL - 1.0f);
    mp = 0.25f * a + 0.125f * b;
    pp = L.p * 0.25f * a * (2.0f - mL) + 0.1875f * mL * b;
  } else {
    mp = mL;
    pp = L.p;
  }
  if (mR <= 1.0f) {
    const float a = (mR - 1.0f) * (mR - 1.0f), b = (mR * mR - 1.0f) * (mR * mR - 1.0f);
    mm = -0.25f * a - 0.125f * b;
    pm = R.p * 0.25f * a * (2.0f + mR) - 0.1875f * mR * b;
  } else {
    mm = 0.0f;
    pm = 0.0f;
  }
  const float mF = mm + mp, pF = pm + pp, amF = fabsf(mF);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float al = L.a_true * L.fc[k], ar = R.a_true * R.fc[k];
    f[k] = 0.5f * (mF * (al + ar) - amF * (ar - al));
  }
  f[d + 1] += pF;
}

// AUSM+ flux of the split-axis scheme along axis d (0 = x, 1 = y).
template <class T>
__host__ __device__ __forceinline__ void ausm_flux(const T ql[4], const T qr[4],
                                                   int d, T f[4]) {
  const AusmSide<T> L = ausm_side(ql), R = ausm_side(qr);
  ausm_axis(ql, L, qr, R, d, f);
}

template <class T>
__host__ __device__ __forceinline__ T entropy_fix(T x) {
  const T e = T(0.125);
  if (x > e) return x;
  return (x * x + e * e) / T(2) / e;
}

template <class T>
__host__ __device__ __forceinline__ T det3(T a, T b, T c, T d, T e, T f, T g,
                                           T h, T i) {
  return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
}

// 4x4 inverse by the adjugate formula (row-major), the algorithm of the
// oracle's Eigen shim: cofactors from 3x3 minors by first-row expansion,
// det along row 0, inverse = adj^T * (1/det).
template <class T>
__host__ __device__ __forceinline__ void inv4(const T m[16], T inv[16]) {
  T cof[16];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int r0 = (i == 0) ? 1 : 0, r1 = (i <= 1) ? 2 : 1, r2 = (i <= 2) ? 3 : 2;
      const int c0 = (j == 0) ? 1 : 0, c1 = (j <= 1) ? 2 : 1, c2 = (j <= 2) ? 3 : 2;
      T v = det3(m[4 * r0 + c0], m[4 * r0 + c1], m[4 * r0 + c2],
                 m[4 * r1 + c0], m[4 * r1 + c1], m[4 * r1 + c2],
                 m[4 * r2 + c0], m[4 * r2 + c1], m[4 * r2 + c2]);
      cof[4 * i + j] = ((i + j) & 1) ? -v : v;
    }
  }
  T det = m[0] * cof[0];
  det += m[1] * cof[1];
  det += m[2] * cof[2];
  det += m[3] * cof[3];
  const T id = T(1) / det;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) inv[4 * i + j] = cof[4 * j + i] * id;
}

// Roe flux along axis d.
template <class T>
__host__ __device__ __forceinline__ void roe_flux(const T ql[4], const T qr[4],
                                                  int d, T f[4]) {
  const T eor = T(1e-10);
  const T D = sqrt(fabs(qr[0] / ql[0]));
  T u[2];
#pragma unroll
  for (int k = 0; k < 2; ++k)
    u[k] = (ql[k + 1] / ql[0] + D * qr[k + 1] / qr[0]) / (T(1) + D);
  const T pL = th_p(ql), pR = th_p(qr);
  const T hL = (ql[3] + pL) / ql[0], hR = (qr[3] + pR) / qr[0];
  const T H = (hL + D * hR) / (T(1) + D);
  const T un = sqrt(u[0] * u[0] + u[1] * u[1]);
  const T a = sqrt(fabs(Gas<T>::gm1() * (H - T(0.5) * (un * un))));
  const T ud = u[d];
  T lam[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) lam[k] = T(0);
  lam[0] = entropy_fix(fabs(ud - a));
  lam[5] = entropy_fix(fabs(ud));
  lam[10] = entropy_fix(fabs(ud));
  lam[15] = entropy_fix(fabs(ud + a));
  const T ke = T(0.5) * (u[0] * u[0] + u[1] * u[1]);
  T R[16], FL[4], FR[4];
  if (d == 0) {
    R[0] = T(1); R[1] = T(1); R[2] = T(0); R[3] = T(1);
    R[4] = u[0] - a; R[5] = u[0]; R[6] = T(0); R[7] = u[0] + a;
    R[8] = u[1]; R[9] = u[1]; R[10] = T(1); R[11] = u[1];
    R[12] = H - u[0] * a; R[13] = ke; R[14] = u[1]; R[15] = H + u[0] * a;
    FL[0] = ql[1];
    FL[1] = ql[1] * ql[1] / (ql[0] + eor) + pL;
    FL[2] = ql[1] * ql[2] / (ql[0] + eor);
    FL[3] = hL * ql[1];
    FR[0] = qr[1];
    FR[1] = qr[1] * qr[1] / (qr[0] + eor) + pR;
    FR[2] = qr[1] * qr[2] / (qr[0] + eor);
    FR[3] = hR * qr[1];
  } else {
    R[0] = T(1); R[1] = T(1); R[2] = T(0); R[3] = T(1);
    R[4] = u[0]; R[5] = u[0]; R[6] = T(1); R[7] = u[0];
    R[8] = u[1] - a; R[9] = u[1]; R[10] = T(0); R[11] = u[1] + a;
    R[12] = H - u[1] * a; R[13] = ke; R[14] = u[0]; R[15] = H + u[1] * a;
    FL[0] = ql[2];
    FL[1] = ql[1] * ql[2] / (ql[0] + eor);
    FL[2] = ql[2] * ql[2] / (ql[0] + eor) + pL;
    FL[3] = hL * ql[2];
    FR[0] = qr[2];
    FR[1] = qr[1] * qr[2] / (qr[0] + eor);
    FR[2] = qr[2] * qr[2] / (qr[0] + eor) + pR;
    FR[3] = hR * qr[2];
  }
  T Ri[16];
  inv4(R, Ri);
  // (R * Lambda) * R^-1 with the shim's left-to-right sums
  T RL[16], A[16];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      T s = R[4 * i] * lam[j];
#pragma unroll
      for (int k = 1; k < 4; ++k) s += R[4 * i + k] * lam[4 * k + j];
      RL[4 * i + j] = s;
    }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      T s = RL[4 * i] * Ri[j];
#pragma unroll
      for (int k = 1; k < 4; ++k) s += RL[4 * i + k] * Ri[4 * k + j];
      A[4 * i + j] = s;
    }
  T dU[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) dU[k] = qr[k] - ql[k];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    T s = (T(0.5) * A[4 * k]) * dU[0];
#pragma unroll
    for (int j = 1; j < 4; ++j) s += (T(0.5) * A[4 * k + j]) * dU[j];
    f[k] = T(0.5) * (FL[k] + FR[k]) - s;
  }
}

// The same Roe flux for the production paths: |A| dQ in closed form as the
// sum over the waves of |lambda_k| alpha_k r_k, with the wave strengths
// from the primitive jumps and the Roe-averaged state (equal to
// R |Lambda| R^-1 dQ of roe_flux for that state, without the 4x4 inverse
// and the two 4x4 products); the same entropy-fixed eigenvalues, physical
// fluxes and EOR denominators.  Not used by the exact path.
template <class T>
__host__ __device__ __forceinline__ void roe_flux_fast(const T ql[4], const T qr[4], int d,
                                                       T f[4]) {
  const T eor = T(1e-10);
  const int t = 1 - d;
  const T irL = T(1) / ql[0], irR = T(1) / qr[0];
  const T D = sqrt(fabs(qr[0] * irL));
  const T iD = T(1) / (T(1) + D);
  const T uL[2] = {ql[1] * irL, ql[2] * irL}, uR[2] = {qr[1] * irR, qr[2] * irR};
  const T u[2] = {(uL[0] + D * uR[0]) * iD, (uL[1] + D * uR[1]) * iD};
  const T pL = th_p(ql), pR = th_p(qr);
  const T hL = (ql[3] + pL) * irL, hR = (qr[3] + pR) * irR;
  const T H = (hL + D * hR) * iD;
  const T ke = T(0.5) * (u[0] * u[0] + u[1] * u[1]);
  const T a2 = fabs(Gas<T>::gm1() * (H - ke));
  const T a = sqrt(a2);
  const T ud = u[d], ut = u[t];
  const T l1 = entropy_fix(fabs(ud - a)), l2 = entropy_fix(fabs(ud)),
          l4 = entropy_fix(fabs(ud + a));
  const T rt = D * ql[0];
  const T dp = pR - pL, dud = uR[d] - uL[d], dut = uR[t] - uL[t];
  const T ia2 = T(1) / a2;
  const T w1 = l1 * (T(0.5) * (dp - rt * a * dud) * ia2);
  const T w4 = l4 * (T(0.5) * (dp + rt * a * dud) * ia2);
  const T w2 = l2 * ((qr[0] - ql[0]) - dp * ia2);
  const T w3 = l2 * (rt * dut);
  T dis[4];
  dis[0] = w1 + w2 + w4;
  dis[1 + d] = w1 * (ud - a) + w2 * ud + w4 * (ud + a);
  dis[1 + t] = (w1 + w2 + w4) * ut + w3;
  dis[3] = w1 * (H - ud * a) + w2 * ke + w4 * (H + ud * a) + w3 * ut;
  const T iL = T(1) / (ql[0] + eor), iR = T(1) / (qr[0] + eor);
  T FL[4], FR[4];
  FL[0] = ql[1 + d];
  FR[0] = qr[1 + d];
  FL[1 + d] = ql[1 + d] * ql[1 + d] * iL + pL;
  FR[1 + d] = qr[1 + d] * qr[1 + d] * iR + pR;
  FL[1 + t] = ql[1] * ql[2] * iL;
  FR[1 + t] = qr[1] * qr[2] * iR;
  FL[3] = hL * ql[1 + d];
  FR[3] = hR * qr[1 + d];
#pragma unroll
  for (int k = 0; k < 4; ++k) f[k] = T(0.5) * (FL[k] + FR[k]) - T(0.5) * dis[k];
}

}  // namespace mst
