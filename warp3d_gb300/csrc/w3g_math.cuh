// w3g_math.cuh -- per-Gauss-point FP64 kinematics and the mm01 material
// update, written for one thread per (element, Gauss point). Each routine
// states the WARP3D routine whose arithmetic it reproduces; results agree
// with the reference to rounding (the kernels use fused multiply-add and
// one reciprocal instead of repeated divisions).
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include "w3g_internal.cuh"

namespace w3g {

// Voigt order used throughout WARP3D: xx, yy, zz, xy, yz, xz.
// 3x3 matrices are column-major: m[r + 3c].

// jacob1 (src/gtmat1.f:300-507): [J] = sum_a dN_a (x) x_a, det, inverse.
// x, y, z: nodal coordinates (length NN), dnx/dne/dnz: dN/dxi.. at the GP.
template <int NN, class T>
__device__ __forceinline__ void jacobian_inverse(const T* dnx, const T* dne, const T* dnz, const T* x,
                                                 const T* y, const T* z, T* gama, T& dj) {
  T j11 = 0, j12 = 0, j13 = 0, j21 = 0, j22 = 0, j23 = 0, j31 = 0, j32 = 0, j33 = 0;
#pragma unroll
  for (int a = 0; a < NN; ++a) {
    T xa = x[a], ya = y[a], za = z[a];
    T p = dnx[a], q = dne[a], r = dnz[a];
    j11 += p * xa; j12 += p * ya; j13 += p * za;
    j21 += q * xa; j22 += q * ya; j23 += q * za;
    j31 += r * xa; j32 += r * ya; j33 += r * za;
  }
  T c1 = j22 * j33 - j23 * j32;
  T c2 = j21 * j33 - j23 * j31;
  T c3 = j21 * j32 - j22 * j31;
  dj = j11 * c1 - j12 * c2 + j13 * c3;
  T rdj = T(1) / dj;
  gama[0] = c1 * rdj;                       // (1,1)
  gama[1] = -c2 * rdj;                      // (2,1)
  gama[2] = c3 * rdj;                       // (3,1)
  gama[3] = (j32 * j13 - j12 * j33) * rdj;  // (1,2)
  gama[4] = (j11 * j33 - j31 * j13) * rdj;  // (2,2)
  gama[5] = (j12 * j31 - j11 * j32) * rdj;  // (3,2)
  gama[6] = (j12 * j23 - j13 * j22) * rdj;  // (1,3)
  gama[7] = (j13 * j21 - j11 * j23) * rdj;  // (2,3)
  gama[8] = (j11 * j22 - j12 * j21) * rdj;  // (3,3)
}

// spatial gradient of N_a: g = [Gamma] dN_a  (blcmp1 btemp, src/blcmp1.f:41-49)
template <class T>
__device__ __forceinline__ void shape_gradient(const T* gama, T p, T q, T r, T& gx, T& gy, T& gz) {
  gx = gama[0] * p + gama[3] * q + gama[6] * r;
  gy = gama[1] * p + gama[4] * q + gama[7] * r;
  gz = gama[2] * p + gama[5] * q + gama[8] * r;
}

// getrm1 opt 2 (src/gtmat1.f:803-846): Cauchy {T} = [q]{t}, q row-major
// here: q[6*r + c]. R column-major.
template <class T>
__device__ __forceinline__ void rotation_q2(const T* R, T* q) {
#define RR(a, b) R[(a - 1) + 3 * (b - 1)]
  q[0] = RR(1, 1) * RR(1, 1); q[1] = RR(1, 2) * RR(1, 2); q[2] = RR(1, 3) * RR(1, 3);
  q[3] = T(2) * RR(1, 1) * RR(1, 2); q[4] = T(2) * RR(1, 3) * RR(1, 2); q[5] = T(2) * RR(1, 1) * RR(1, 3);
  q[6] = RR(2, 1) * RR(2, 1); q[7] = RR(2, 2) * RR(2, 2); q[8] = RR(2, 3) * RR(2, 3);
  q[9] = T(2) * RR(2, 1) * RR(2, 2); q[10] = T(2) * RR(2, 3) * RR(2, 2); q[11] = T(2) * RR(2, 1) * RR(2, 3);
  q[12] = RR(3, 1) * RR(3, 1); q[13] = RR(3, 2) * RR(3, 2); q[14] = RR(3, 3) * RR(3, 3);
  q[15] = T(2) * RR(3, 1) * RR(3, 2); q[16] = T(2) * RR(3, 3) * RR(3, 2); q[17] = T(2) * RR(3, 1) * RR(3, 3);
  q[18] = RR(1, 1) * RR(2, 1); q[19] = RR(1, 2) * RR(2, 2); q[20] = RR(1, 3) * RR(2, 3);
  q[21] = RR(1, 1) * RR(2, 2) + RR(2, 1) * RR(1, 2);
  q[22] = RR(1, 2) * RR(2, 3) + RR(1, 3) * RR(2, 2);
  q[23] = RR(1, 1) * RR(2, 3) + RR(1, 3) * RR(2, 1);
  q[24] = RR(2, 1) * RR(3, 1); q[25] = RR(3, 2) * RR(2, 2); q[26] = RR(2, 3) * RR(3, 3);
  q[27] = RR(2, 1) * RR(3, 2) + RR(2, 2) * RR(3, 1);
  q[28] = RR(2, 2) * RR(3, 3) + RR(3, 2) * RR(2, 3);
  q[29] = RR(2, 1) * RR(3, 3) + RR(2, 3) * RR(3, 1);
  q[30] = RR(1, 1) * RR(3, 1); q[31] = RR(1, 2) * RR(3, 2); q[32] = RR(1, 3) * RR(3, 3);
  q[33] = RR(1, 1) * RR(3, 2) + RR(1, 2) * RR(3, 1);
  q[34] = RR(1, 2) * RR(3, 3) + RR(1, 3) * RR(3, 2);
  q[35] = RR(1, 1) * RR(3, 3) + RR(3, 1) * RR(1, 3);
#undef RR
}

// getrm1 opt 1 (src/gtmat1.f:765-801): unrotated {d} = [q]{D}, row-major.
__device__ __forceinline__ void rotation_q1(const double* R, double* q) {
#define RR(a, b) R[(a - 1) + 3 * (b - 1)]
  q[0] = RR(1, 1) * RR(1, 1); q[1] = RR(2, 1) * RR(2, 1); q[2] = RR(3, 1) * RR(3, 1);
  q[3] = RR(1, 1) * RR(2, 1); q[4] = RR(3, 1) * RR(2, 1); q[5] = RR(1, 1) * RR(3, 1);
  q[6] = RR(1, 2) * RR(1, 2); q[7] = RR(2, 2) * RR(2, 2); q[8] = RR(3, 2) * RR(3, 2);
  q[9] = RR(1, 2) * RR(2, 2); q[10] = RR(3, 2) * RR(2, 2); q[11] = RR(1, 2) * RR(3, 2);
  q[12] = RR(1, 3) * RR(1, 3); q[13] = RR(2, 3) * RR(2, 3); q[14] = RR(3, 3) * RR(3, 3);
  q[15] = RR(1, 3) * RR(2, 3); q[16] = RR(3, 3) * RR(2, 3); q[17] = RR(1, 3) * RR(3, 3);
  q[18] = 2.0 * RR(1, 1) * RR(1, 2); q[19] = 2.0 * RR(2, 1) * RR(2, 2); q[20] = 2.0 * RR(3, 1) * RR(3, 2);
  q[21] = RR(1, 1) * RR(2, 2) + RR(1, 2) * RR(2, 1);
  q[22] = RR(2, 1) * RR(3, 2) + RR(3, 1) * RR(2, 2);
  q[23] = RR(1, 1) * RR(3, 2) + RR(3, 1) * RR(1, 2);
  q[24] = 2.0 * RR(1, 2) * RR(1, 3); q[25] = 2.0 * RR(2, 3) * RR(2, 2); q[26] = 2.0 * RR(3, 2) * RR(3, 3);
  q[27] = RR(1, 2) * RR(2, 3) + RR(2, 2) * RR(1, 3);
  q[28] = RR(2, 2) * RR(3, 3) + RR(2, 3) * RR(3, 2);
  q[29] = RR(1, 2) * RR(3, 3) + RR(3, 2) * RR(1, 3);
  q[30] = 2.0 * RR(1, 1) * RR(1, 3); q[31] = 2.0 * RR(2, 1) * RR(2, 3); q[32] = 2.0 * RR(3, 1) * RR(3, 3);
  q[33] = RR(1, 1) * RR(2, 3) + RR(2, 1) * RR(1, 3);
  q[34] = RR(2, 1) * RR(3, 3) + RR(3, 1) * RR(2, 3);
  q[35] = RR(1, 1) * RR(3, 3) + RR(1, 3) * RR(3, 1);
#undef RR
}

// qmply1 (src/qmply1.f:15-36): m2 = q m1
template <class T>
__device__ __forceinline__ void qmply(const T* q, const T* m1, T* m2) {
#pragma unroll
  for (int j = 0; j < 6; ++j)
    m2[j] = q[6 * j + 0] * m1[0] + q[6 * j + 1] * m1[1] + q[6 * j + 2] * m1[2] + q[6 * j + 3] * m1[3] +
            q[6 * j + 4] * m1[4] + q[6 * j + 5] * m1[5];
}

// Polar decomposition [F] = [R][U]: rtcmp1 + irscp1 + ivcmp1 + evcmp1_new
// (src/gtmat1.f:691-735, 961-1210). U^-1 from the invariants of U, whose
// principal values come from Cardano's closed form for C = F^T F.
__device__ __forceinline__ void polar_rotation(const double* F, double* R) {
#define FF(a, b) F[(a - 1) + 3 * (b - 1)]
  double c[6], cc[6];
  c[0] = FF(1, 1) * FF(1, 1) + FF(2, 1) * FF(2, 1) + FF(3, 1) * FF(3, 1);
  c[1] = FF(1, 1) * FF(1, 2) + FF(2, 1) * FF(2, 2) + FF(3, 1) * FF(3, 2);
  c[2] = FF(1, 2) * FF(1, 2) + FF(2, 2) * FF(2, 2) + FF(3, 2) * FF(3, 2);
  c[3] = FF(1, 1) * FF(1, 3) + FF(2, 1) * FF(2, 3) + FF(3, 1) * FF(3, 3);
  c[4] = FF(1, 2) * FF(1, 3) + FF(2, 2) * FF(2, 3) + FF(3, 2) * FF(3, 3);
  c[5] = FF(1, 3) * FF(1, 3) + FF(2, 3) * FF(2, 3) + FF(3, 3) * FF(3, 3);
  cc[0] = c[0] * c[0] + c[1] * c[1] + c[3] * c[3];
  cc[1] = c[0] * c[1] + c[1] * c[2] + c[3] * c[4];
  cc[2] = c[1] * c[1] + c[2] * c[2] + c[4] * c[4];
  cc[3] = c[0] * c[3] + c[1] * c[4] + c[3] * c[5];
  cc[4] = c[1] * c[3] + c[2] * c[4] + c[4] * c[5];
  cc[5] = c[3] * c[3] + c[4] * c[4] + c[5] * c[5];
  // evcmp1_new: Cardano's closed form
  const double third = 1.0 / 3.0;
  double m11 = c[0], m12 = c[1], m13 = c[3], m22 = c[2], m23 = c[4], m33 = c[5];
  double de = m12 * m23, dd = m12 * m12, ee = m23 * m23, ff = m13 * m13;
  double m = m11 + m22 + m33;
  double c1 = (m11 * m22 + m11 * m33 + m22 * m33) - (dd + ee + ff);
  double c0 = m33 * dd + m11 * ee + m22 * ff - m11 * m22 * m33 - 2.0 * m13 * de;
  double p = m * m - 3.0 * c1;
  double q = m * (p - 1.5 * c1) - 13.5 * c0;
  double sqrtp = sqrt(fabs(p));
  double phi = 27.0 * (0.25 * c1 * c1 * (p - c1) + c0 * (q + 6.75 * c0));
  phi = third * atan2(sqrt(fabs(phi)), q);
  double sphi0, cphi0;
  sincos(phi, &sphi0, &cphi0);
  const double iroot3 = 0.5773502691896258;    // 1/sqrt(3) rounded to double
  double cphi = sqrtp * cphi0;
  double sphi = iroot3 * sqrtp * sphi0;
  double e2 = third * (m - cphi);
  double e3 = e2 + sphi;
  double e1 = e2 + cphi;
  e2 = e2 - sphi;
  // increasing order as evcmp1_new returns them (the sums below are
  // order-sensitive in the last bit)
  if (e2 < e1) { double t = e1; e1 = e2; e2 = t; }
  if (e3 < e1) { double t = e1; e1 = e3; e3 = t; }
  if (e3 < e2) { double t = e2; e2 = e3; e3 = t; }
  double v1 = sqrt(e1), v2 = sqrt(e2), v3 = sqrt(e3);
  double iu = v1 + v2 + v3;
  double iiu = v1 * v2 + v2 * v3 + v1 * v3;
  double iiiu = v1 * v2 * v3;
  double a2 = 1.0 / (iiiu * (iu * iiu - iiiu));
  double b2 = iu * iiu * iiu - iiiu * (iu * iu + iiu);
  double c2 = -iiiu - iu * (iu * iu - 2.0 * iiu);
  double d2 = iu;
  double ui0 = a2 * (b2 + c2 * c[0] + d2 * cc[0]);
  double ui1 = a2 * (c2 * c[1] + d2 * cc[1]);
  double ui2 = a2 * (b2 + c2 * c[2] + d2 * cc[2]);
  double ui3 = a2 * (c2 * c[3] + d2 * cc[3]);
  double ui4 = a2 * (c2 * c[4] + d2 * cc[4]);
  double ui5 = a2 * (b2 + c2 * c[5] + d2 * cc[5]);
  R[0] = FF(1, 1) * ui0 + FF(1, 2) * ui1 + FF(1, 3) * ui3;
  R[3] = FF(1, 1) * ui1 + FF(1, 2) * ui2 + FF(1, 3) * ui4;
  R[6] = FF(1, 1) * ui3 + FF(1, 2) * ui4 + FF(1, 3) * ui5;
  R[1] = FF(2, 1) * ui0 + FF(2, 2) * ui1 + FF(2, 3) * ui3;
  R[4] = FF(2, 1) * ui1 + FF(2, 2) * ui2 + FF(2, 3) * ui4;
  R[7] = FF(2, 1) * ui3 + FF(2, 2) * ui4 + FF(2, 3) * ui5;
  R[2] = FF(3, 1) * ui0 + FF(3, 2) * ui1 + FF(3, 3) * ui3;
  R[5] = FF(3, 1) * ui1 + FF(3, 2) * ui2 + FF(3, 3) * ui4;
  R[8] = FF(3, 1) * ui3 + FF(3, 2) * ui4 + FF(3, 3) * ui5;
#undef FF
}

// double -> float, rounded to nearest even, on the integer pipes. GB300's
// FP64 pipe (which also executes the F2F conversion) retires 2 lanes per
// clock and SM, a warp-wide conversion costs ~64 issue cycles of its SM
// sub-partition; this sequence of ~12 integer operations costs ~1. From
// the IEEE 754 binary64 / binary32 layouts: the float keeps the top 23 of
// the 52 mantissa bits, the 29 dropped bits decide the rounding (ties to
// even), a carry out of the mantissa moves into the exponent. Magnitudes
// below the smallest normal float become 0 and above the largest become
// infinity (also for infinite and NaN inputs), which the element inputs
// (stresses, rotations, material matrices) never reach.
__device__ __forceinline__ float d2f_rn(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const int e = (int)((hi >> 20) & 0x7FFu) - (1023 - 127);
  const unsigned m = __funnelshift_l(lo, hi, 3) & 0x7FFFFFu;
  const unsigned rest = lo & 0x1FFFFFFFu;
  unsigned r = ((unsigned)e << 23) + m;
  r += (rest > 0x10000000u) | ((rest == 0x10000000u) & (m & 1u));
  r = e <= 0 ? 0u : (e >= 255 || r >= 0x7F800000u ? 0x7F800000u : r);
  return __uint_as_float((hi & 0x80000000u) | r);
}

// a double input in the arithmetic type of a kernel: unchanged for double,
// d2f_rn for float (the same value as a float conversion in the normal
// range, without the FP64 pipe)
template <class T> __device__ __forceinline__ T from_f64(double x);
template <> __device__ __forceinline__ double from_f64<double>(double x) { return x; }
template <> __device__ __forceinline__ float from_f64<float>(double x) { return d2f_rn(x); }

// ---------------------------------------------------------------------
// Fixed-order arithmetic for the finite-strain kinematics chain.
//
// WARP3D's polar decomposition (Cardano eigenvalues of C = F^T F, then
// U^-1 from the invariants of U) is ill-conditioned when F is close to a
// rotation: p = m^2 - 3 c1 cancels, and two evaluation orders of the same
// formulas give rotations that differ by ~1e-9. To reproduce the oracle's
// rotations and strain increments to 1e-12, jacob1 (at t=0), tcomp1,
// fcomp1 and the polar decomposition below evaluate every expression in
// one fixed order with explicitly rounded operations, the same order as
// the oracle: jacob1 at t = 0 without fused multiply-add (computed once
// and cached), the per-call chain with the reference's product sums fused
// left to right (a*b + c*d + e*f -> fma(e, f, fma(c, d, a*b)), x - a*b ->
// fma(-a, b, x)) -- what an FMA-contracting build of the Fortran executes
// and two FP64 instructions in three fewer. Divisions stay where the
// reference divides. The transcendental calls (atan2, cos, sin) are
// CUDA's.
// ---------------------------------------------------------------------
__device__ __forceinline__ double rm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ra(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rs(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rd(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double fm(double a, double b, double c) { return __fma_rn(a, b, c); }
// a*b + c*d + e*f, fused left to right
__device__ __forceinline__ double dot3f(double a, double b, double c, double d, double e, double f) {
  return fm(e, f, fm(c, d, rm(a, b)));
}
// one node's term of tcomp1 for both configurations: th += t * u (fused)
__device__ __forceinline__ void tcomp1_node(double* th, double tx, double ty, double tz, double ux, double uy,
                                            double uz) {
  th[0] = fm(tx, ux, th[0]); th[1] = fm(tx, uy, th[1]); th[2] = fm(tx, uz, th[2]);
  th[3] = fm(ty, ux, th[3]); th[4] = fm(ty, uy, th[4]); th[5] = fm(ty, uz, th[5]);
  th[6] = fm(tz, ux, th[6]); th[7] = fm(tz, uy, th[7]); th[8] = fm(tz, uz, th[8]);
}

// jacob1 (src/gtmat1.f:382-480) in reference order; gama column-major.
template <int NN>
__device__ __forceinline__ void jacob1_ref(const double* dnx, const double* dne, const double* dnz,
                                           const double* x, const double* y, const double* z, double* gama,
                                           double& dj) {
  double j11 = 0, j12 = 0, j13 = 0, j21 = 0, j22 = 0, j23 = 0, j31 = 0, j32 = 0, j33 = 0;
#pragma unroll
  for (int a = 0; a < NN; ++a) {
    j11 = ra(j11, rm(dnx[a], x[a])); j12 = ra(j12, rm(dnx[a], y[a])); j13 = ra(j13, rm(dnx[a], z[a]));
    j21 = ra(j21, rm(dne[a], x[a])); j22 = ra(j22, rm(dne[a], y[a])); j23 = ra(j23, rm(dne[a], z[a]));
    j31 = ra(j31, rm(dnz[a], x[a])); j32 = ra(j32, rm(dnz[a], y[a])); j33 = ra(j33, rm(dnz[a], z[a]));
  }
  double c1 = rs(rm(j22, j33), rm(j23, j32));
  double c2 = rs(rm(j21, j33), rm(j23, j31));
  double c3 = rs(rm(j21, j32), rm(j22, j31));
  dj = ra(rs(rm(j11, c1), rm(j12, c2)), rm(j13, c3));
  gama[0] = rd(c1, dj);
  gama[1] = rd(-c2, dj);
  gama[2] = rd(c3, dj);
  gama[3] = rd(rs(rm(j32, j13), rm(j12, j33)), dj);
  gama[4] = rd(rs(rm(j11, j33), rm(j31, j13)), dj);
  gama[5] = rd(rs(rm(j12, j31), rm(j11, j32)), dj);
  gama[6] = rd(rs(rm(j12, j23), rm(j13, j22)), dj);
  gama[7] = rd(rs(rm(j13, j21), rm(j11, j23)), dj);
  gama[8] = rd(rs(rm(j11, j22), rm(j12, j21)), dj);
}

// thtemp of tcomp1 (src/gtmat1.f:545-556): Gamma dN_a in reference order
__device__ __forceinline__ void grad_ref(const double* g, double p, double q, double r, double& tx, double& ty,
                                         double& tz) {
  tx = ra(ra(rm(g[0], p), rm(g[3], q)), rm(g[6], r));
  ty = ra(ra(rm(g[1], p), rm(g[4], q)), rm(g[7], r));
  tz = ra(ra(rm(g[2], p), rm(g[5], q)), rm(g[8], r));
}

// fcomp1 determinant (src/gtmat1.f:640-652), fused as in the oracle
__device__ __forceinline__ double det_ref(const double* F) {
  double f1 = fm(F[4], F[8], -rm(F[7], F[5]));
  double f2 = fm(F[1], F[8], -rm(F[7], F[2]));
  double f3 = fm(F[1], F[5], -rm(F[4], F[2]));
  return fm(F[6], f3, fm(F[0], f1, -rm(F[3], f2)));
}

// rtcmp1 + irscp1 + ivcmp1 + evcmp1_new (src/gtmat1.f:691-735, 961-1210),
// the reference's expressions with the product sums fused as in the oracle
__device__ __forceinline__ void polar_rotation_ref(const double* F, double* R) {
#define FF(a, b) F[(a - 1) + 3 * (b - 1)]
  double c[6], cc[6];
  c[0] = dot3f(FF(1, 1), FF(1, 1), FF(2, 1), FF(2, 1), FF(3, 1), FF(3, 1));
  c[1] = dot3f(FF(1, 1), FF(1, 2), FF(2, 1), FF(2, 2), FF(3, 1), FF(3, 2));
  c[2] = dot3f(FF(1, 2), FF(1, 2), FF(2, 2), FF(2, 2), FF(3, 2), FF(3, 2));
  c[3] = dot3f(FF(1, 1), FF(1, 3), FF(2, 1), FF(2, 3), FF(3, 1), FF(3, 3));
  c[4] = dot3f(FF(1, 2), FF(1, 3), FF(2, 2), FF(2, 3), FF(3, 2), FF(3, 3));
  c[5] = dot3f(FF(1, 3), FF(1, 3), FF(2, 3), FF(2, 3), FF(3, 3), FF(3, 3));
  cc[0] = dot3f(c[0], c[0], c[1], c[1], c[3], c[3]);
  cc[1] = dot3f(c[0], c[1], c[1], c[2], c[3], c[4]);
  cc[2] = dot3f(c[1], c[1], c[2], c[2], c[4], c[4]);
  cc[3] = dot3f(c[0], c[3], c[1], c[4], c[3], c[5]);
  cc[4] = dot3f(c[1], c[3], c[2], c[4], c[4], c[5]);
  cc[5] = dot3f(c[3], c[3], c[4], c[4], c[5], c[5]);
  const double third = 1.0 / 3.0;
  double m11 = c[0], m12 = c[1], m13 = c[3], m22 = c[2], m23 = c[4], m33 = c[5];
  double de = rm(m12, m23), dd = rm(m12, m12), ee = rm(m23, m23), ff = rm(m13, m13);
  double m = ra(ra(m11, m22), m33);
  double c1 = rs(fm(m22, m33, fm(m11, m33, rm(m11, m22))), ra(ra(dd, ee), ff));
  double c0 = fm(-rm(2.0, m13), de, fm(-rm(m11, m22), m33, fm(m22, ff, fm(m11, ee, rm(m33, dd)))));
  double p = fm(m, m, -rm(3.0, c1));
  double q = fm(m, rs(p, rm(1.5, c1)), -rm(13.5, c0));
  double sqrtp = sqrt(fabs(p));
  double phi = rm(27.0, fm(rm(rm(0.25, c1), c1), rs(p, c1), rm(c0, fm(6.75, c0, q))));
  phi = rm(third, atan2(sqrt(fabs(phi)), q));
  const double iroot3 = 0.5773502691896258;    // 1/sqrt(3) rounded to double
  double cphi = rm(sqrtp, cos(phi));
  double sphi = rm(rm(iroot3, sqrtp), sin(phi));
  double e2 = rm(third, rs(m, cphi));
  double e3 = ra(e2, sphi);
  double e1 = ra(e2, cphi);
  e2 = rs(e2, sphi);
  if (e2 < e1) { double t = e1; e1 = e2; e2 = t; }
  if (e3 < e1) { double t = e1; e1 = e3; e3 = t; }
  if (e3 < e2) { double t = e2; e2 = e3; e3 = t; }
  double v1 = sqrt(e1), v2 = sqrt(e2), v3 = sqrt(e3);
  double iu = ra(ra(v1, v2), v3);
  double iiu = fm(v1, v3, fm(v2, v3, rm(v1, v2)));
  double iiiu = rm(rm(v1, v2), v3);
  double a2 = rd(1.0, rm(iiiu, fm(iu, iiu, -iiiu)));
  double b2 = fm(rm(iu, iiu), iiu, -rm(iiiu, fm(iu, iu, iiu)));
  double c2 = fm(-iu, fm(iu, iu, -rm(2.0, iiu)), -iiiu);
  double d2 = iu;
  double ui0 = rm(a2, fm(d2, cc[0], fm(c2, c[0], b2)));
  double ui1 = rm(a2, fm(d2, cc[1], rm(c2, c[1])));
  double ui2 = rm(a2, fm(d2, cc[2], fm(c2, c[2], b2)));
  double ui3 = rm(a2, fm(d2, cc[3], rm(c2, c[3])));
  double ui4 = rm(a2, fm(d2, cc[4], rm(c2, c[4])));
  double ui5 = rm(a2, fm(d2, cc[5], fm(c2, c[5], b2)));
  R[0] = dot3f(FF(1, 1), ui0, FF(1, 2), ui1, FF(1, 3), ui3);
  R[3] = dot3f(FF(1, 1), ui1, FF(1, 2), ui2, FF(1, 3), ui4);
  R[6] = dot3f(FF(1, 1), ui3, FF(1, 2), ui4, FF(1, 3), ui5);
  R[1] = dot3f(FF(2, 1), ui0, FF(2, 2), ui1, FF(2, 3), ui3);
  R[4] = dot3f(FF(2, 1), ui1, FF(2, 2), ui2, FF(2, 3), ui4);
  R[7] = dot3f(FF(2, 1), ui3, FF(2, 2), ui4, FF(2, 3), ui5);
  R[2] = dot3f(FF(3, 1), ui0, FF(3, 2), ui1, FF(3, 3), ui3);
  R[5] = dot3f(FF(3, 1), ui1, FF(3, 2), ui2, FF(3, 3), ui4);
  R[8] = dot3f(FF(3, 1), ui3, FF(3, 2), ui4, FF(3, 3), ui5);
#undef FF
}

// mm01 history word 4 stores an integer state in the low 32 bits of a
// double (src/mm01.f:251-284, :651-652).
__device__ __forceinline__ int mm01_state(double d) {
  return (int)(uint32_t)((unsigned long long)__double_as_longlong(d) & 0xffffffffull);
}
__device__ __forceinline__ double mm01_state_word(int s) {
  return __longlong_as_double((long long)(unsigned long long)(uint32_t)s);
}

// One Gauss point of mm01 (src/mm01.f:24-233): mm01_set_history (step 1),
// mm01_init, mm01_general, the elastic branch, mm01_sig_final,
// mm01_wrapup; then cnst1 (src/mm01.f:1196-1348) for the lower triangle
// of [D] (rstgp1_store_cep order). hist is modified at step 1 exactly as
// the reference modifies its local copy. alpha11_first: history word 11
// of the block's first element at this Gauss point, which mm01_general
// reads for every element (src/mm01.f:843-845).
//
// Per-element constants come precomputed (MatProps, evaluated on the host
// with the reference's expressions); the remaining divisions by
// per-point values use one reciprocal each.
__device__ __forceinline__ void mm01_point(const MatProps& mp, int step, double* cgn /*9, modified at step 1*/,
                                           const double* deps, double* hist /*11*/, double alpha11_first,
                                           double* cgn1 /*9*/, double* hist1 /*11*/, double* cep21) {
  const double one = 1.0, two = 2.0, half = 0.5;
  const double third = 1.0 / 3.0;
  const double root2 = 1.4142135623730951, inv_root3 = 0.5773502691896258, inv_root2 = 0.7071067811865476;
  const bool lnelas = mp.lnelas != 0.0;
  if (step == 1) {   // mm01_set_history
    hist[0] = 0.0; hist[1] = mp.yld_root3; hist[2] = 0.0; hist[3] = mm01_state_word(3); hist[4] = mp.h;
#pragma unroll
    for (int k = 5; k < 11; ++k) hist[k] = 0.0;
    cgn[7] = 0.0; cgn[8] = 0.0;
    alpha11_first = 0.0;
  }
  // mm01_init
  const double deps_vol = deps[0] + deps[1] + deps[2];
  const double eps_mean = deps_vol * third;
  const double een1 = (cgn[0] - mp.nu * (cgn[1] + cgn[2])) * mp.inv_e;
  const double een2 = (cgn[1] - mp.nu * (cgn[0] + cgn[2])) * mp.inv_e;
  const double een3 = (cgn[2] - mp.nu * (cgn[0] + cgn[1])) * mp.inv_e;
  const double eps_vol_n1 = een1 + een2 + een3 + deps_vol;
  const double eps_mean_n = (een1 + een2 + een3) * third;
  const double g2 = two * mp.shear;
  double dev[6];
  dev[0] = g2 * ((een1 - eps_mean_n) + (deps[0] - eps_mean));
  dev[1] = g2 * ((een2 - eps_mean_n) + (deps[1] - eps_mean));
  dev[2] = g2 * ((een3 - eps_mean_n) + (deps[2] - eps_mean));
  dev[3] = mp.shear * (cgn[3] * mp.inv_gn + deps[3]);
  dev[4] = mp.shear * (cgn[4] * mp.inv_gn + deps[4]);
  dev[5] = mp.shear * (cgn[5] * mp.inv_gn + deps[5]);
  const double hbark_n = (one - mp.beta) * hist[4];
  const double kbar = (mp.yld + mp.hbari * hist[2]) * inv_root3;
  double lk = one;
  if (fabs(hbark_n) > 0.000001) lk = mp.hbark / hbark_n;
  double rtse[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) rtse[k] = dev[k] - hist[5 + k] * lk;
  double mrts = sqrt(rtse[0] * rtse[0] + rtse[1] * rtse[1] + rtse[2] * rtse[2] +
                     two * (rtse[3] * rtse[3] + rtse[4] * rtse[4] + rtse[5] * rtse[5]));
  const double yf = mrts - root2 * kbar;
#pragma unroll
  for (int k = 0; k < 6; ++k) rtse[k] = dev[k] - hist[5 + k];
  const double mrtsq = rtse[0] * rtse[0] + rtse[1] * rtse[1] + rtse[2] * rtse[2] +
                       two * (rtse[3] * rtse[3] + rtse[4] * rtse[4] + rtse[5] * rtse[5]);
  mrts = sqrt(mrtsq);
  const bool yield = !lnelas && yf >= 0.0000001 * root2 * kbar;
  const int instat = yield ? 1 : 3;

  double devn1[6];
  if (yield) {   // mm01_general
    const double root2c = 1.414213562373095, twthrd = 0.666666666666667, root23 = 0.816496580927,
                 root2o3 = 0.4714045207910;
    const double rmrts = one / mrts;
    const double a = (g2 + twthrd * mp.hbark) * rmrts;
    const double b = one - lk;
    const double d = root2o3 * mp.hbari;
    const double vbar = mrts * mrts;
    const double wbar = hist[5] * hist[5] + hist[6] * hist[6] + hist[7] * hist[7] +
                        two * (hist[8] * hist[8] + hist[9] * hist[9] + alpha11_first * alpha11_first);
    const double vwbar = rtse[0] * hist[5] + rtse[1] * hist[6] + rtse[2] * hist[7] +
                         two * (rtse[3] * hist[8] + rtse[4] * hist[9] + rtse[5] * hist[10]);
    const double t1 = a * a * vbar - two * d * d;
    const double t2 = -4.0 * d * kbar - two * a * vbar - two * a * b * vwbar;
    const double t3 = b * b * wbar + two * b * vwbar + vbar - two * kbar * kbar;
    const double discr = t2 * t2 - 4.0 * t1 * t3;
    double lambda_deltat = 0.0;
    if (!(discr < 0.0)) {
      const double sd = sqrt(discr), r2t1 = half / t1;
      lambda_deltat = fmin((-t2 + sd) * r2t1, (-t2 - sd) * r2t1);
    }
    hist1[0] = lambda_deltat;
    hist1[1] = kbar + (root2c / 3.0) * mp.hbari * lambda_deltat;
    hist1[2] = hist[2] + lambda_deltat * root23;
    hist1[4] = mp.h;
    const double const1 = twthrd * mp.hbark * lambda_deltat * rmrts;
    const double const2 = one - lambda_deltat * (twthrd * mp.hbark + g2) * rmrts;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      hist1[5 + k] = lk * hist[5 + k] + const1 * rtse[k];
      devn1[k] = hist1[5 + k] + b * hist[5 + k] + const2 * rtse[k];
    }
  } else {
    hist1[0] = 0.0;
    hist1[1] = lnelas ? 0.0 : kbar;
    hist1[2] = hist[2];
    hist1[4] = mp.h;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      hist1[5 + k] = hist[5 + k] * lk;
      devn1[k] = rtse[k] + hist[5 + k];
    }
  }
  // mm01_sig_final
  const double sig_mean_np1 = eps_vol_n1 * mp.k3 * third;
  cgn1[0] = devn1[0] + sig_mean_np1;
  cgn1[1] = devn1[1] + sig_mean_np1;
  cgn1[2] = devn1[2] + sig_mean_np1;
  cgn1[3] = devn1[3]; cgn1[4] = devn1[4]; cgn1[5] = devn1[5];
  cgn1[6] = cgn[6] + half * (deps[0] * (cgn1[0] + cgn[0]) + deps[1] * (cgn1[1] + cgn[1]) +
                             deps[2] * (cgn1[2] + cgn[2]) + deps[3] * (cgn1[3] + cgn[3]) +
                             deps[4] * (cgn1[4] + cgn[4]) + deps[5] * (cgn1[5] + cgn[5]));
  hist1[3] = mm01_state_word(instat);
  // mm01_wrapup
  cgn1[7] = cgn[7];
  cgn1[8] = cgn[8];
  if (yield) {
    const double six = 6.0;
    const double sbar_n = sqrt((cgn[0] - cgn[1]) * (cgn[0] - cgn[1]) + (cgn[1] - cgn[2]) * (cgn[1] - cgn[2]) +
                               (cgn[0] - cgn[2]) * (cgn[0] - cgn[2]) +
                               six * (cgn[3] * cgn[3] + cgn[4] * cgn[4] + cgn[5] * cgn[5])) * inv_root2;
    const double sbar_n1 = sqrt((cgn1[0] - cgn1[1]) * (cgn1[0] - cgn1[1]) + (cgn1[1] - cgn1[2]) * (cgn1[1] - cgn1[2]) +
                                (cgn1[0] - cgn1[2]) * (cgn1[0] - cgn1[2]) +
                                six * (cgn1[3] * cgn1[3] + cgn1[4] * cgn1[4] + cgn1[5] * cgn1[5])) * inv_root2;
    const double depbar = hist1[2] - hist[2];
    cgn1[7] = cgn[7] + half * (sbar_n1 + sbar_n) * depbar;
    cgn1[8] = cgn[8] + depbar;
  }
  // cnst1: lower triangle, order (1,1) (2,1) (2,2) (3,1) (3,2) (3,3) (4,1)..(6,6)
  if (!yield) {
    cep21[0] = mp.c2; cep21[1] = mp.c4; cep21[2] = mp.c2; cep21[3] = mp.c4; cep21[4] = mp.c4; cep21[5] = mp.c2;
#pragma unroll
    for (int k = 6; k < 21; ++k) cep21[k] = 0.0;
    cep21[9] = mp.c3; cep21[14] = mp.c3; cep21[20] = mp.c3;
  } else {
    const double root2t = 1.414213562;   // cnst1 uses a truncated sqrt(2)
    const double kn1 = hist1[1], ldt = hist1[0];
    const double rm = one / mrtsq;
    const double bb = (root2t * kn1 + (two / 3.0) * (one - mp.beta) * mp.h * ldt) / mrts;
    const double gambar = mp.gamma - one + bb;
    const double gbar = mp.shear * bb;
    const double albar = mp.kbulk - two * gbar * third;
    const double thbar = two * mp.shear * gambar * rm;
    const double* r = rtse;
    const double a2g = albar + two * gbar;
    cep21[0] = a2g - thbar * (r[0] * r[0]);
    cep21[1] = albar - thbar * r[0] * r[1];
    cep21[2] = a2g - thbar * (r[1] * r[1]);
    cep21[3] = albar - thbar * r[0] * r[2];
    cep21[4] = albar - thbar * r[2] * r[1];
    cep21[5] = a2g - thbar * (r[2] * r[2]);
    cep21[6] = -(thbar * r[0] * r[3]);
    cep21[7] = -(thbar * r[1] * r[3]);
    cep21[8] = -(thbar * r[2] * r[3]);
    cep21[9] = gbar - thbar * (r[3] * r[3]);
    cep21[10] = -(thbar * r[0] * r[4]);
    cep21[11] = -(thbar * r[1] * r[4]);
    cep21[12] = -(thbar * r[2] * r[4]);
    cep21[13] = -(thbar * r[3] * r[4]);
    cep21[14] = gbar - thbar * (r[4] * r[4]);
    cep21[15] = -(thbar * r[0] * r[5]);
    cep21[16] = -(thbar * r[1] * r[5]);
    cep21[17] = -(thbar * r[2] * r[5]);
    cep21[18] = -(thbar * r[3] * r[5]);
    cep21[19] = -(thbar * r[4] * r[5]);
    cep21[20] = gbar - thbar * (r[5] * r[5]);
  }
}

// {t} = [R]{T}[R]^T-type rotations of a symmetric tensor in Voigt form
// (xx, yy, zz, xy, yz, xz). rotate_to_spatial: S = R s R^T (getrm1 opt 2 +
// qmply1, src/gtmat1.f:803-846); rotate_to_unrotated for a rate of
// deformation with engineering shears: d = R^T D R (getrm1 opt 1).
__device__ __forceinline__ void rotate_to_spatial(const double* R, const double* s, double* S) {
  // A = R s (3x3), S = A R^T, symmetric tensor s
  const double t[9] = {s[0], s[3], s[5], s[3], s[1], s[4], s[5], s[4], s[2]};   // column-major
  double A[9];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int r = 0; r < 3; ++r) A[r + 3 * c] = R[r] * t[3 * c] + R[r + 3] * t[1 + 3 * c] + R[r + 6] * t[2 + 3 * c];
  // S_ij = sum_k A_ik R_jk
  S[0] = A[0] * R[0] + A[3] * R[3] + A[6] * R[6];
  S[1] = A[1] * R[1] + A[4] * R[4] + A[7] * R[7];
  S[2] = A[2] * R[2] + A[5] * R[5] + A[8] * R[8];
  S[3] = A[0] * R[1] + A[3] * R[4] + A[6] * R[7];
  S[4] = A[1] * R[2] + A[4] * R[5] + A[7] * R[8];
  S[5] = A[0] * R[2] + A[3] * R[5] + A[6] * R[8];
}

__device__ __forceinline__ void rotate_to_unrotated(const double* R, const double* d, double* u) {
  // tensor D with half shears; A = R^T D, u = A R
  const double t[9] = {d[0], 0.5 * d[3], 0.5 * d[5], 0.5 * d[3], d[1], 0.5 * d[4], 0.5 * d[5], 0.5 * d[4], d[2]};
  double A[9];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int r = 0; r < 3; ++r)
      A[r + 3 * c] = R[3 * r] * t[3 * c] + R[1 + 3 * r] * t[1 + 3 * c] + R[2 + 3 * r] * t[2 + 3 * c];
  // u_ij = sum_k A_ik R_kj
  u[0] = A[0] * R[0] + A[3] * R[1] + A[6] * R[2];
  u[1] = A[1] * R[3] + A[4] * R[4] + A[7] * R[5];
  u[2] = A[2] * R[6] + A[5] * R[7] + A[8] * R[8];
  u[3] = 2.0 * (A[0] * R[3] + A[3] * R[4] + A[6] * R[5]);
  u[4] = 2.0 * (A[1] * R[6] + A[4] * R[7] + A[7] * R[8]);
  u[5] = 2.0 * (A[0] * R[6] + A[3] * R[7] + A[6] * R[8]);
}

}  // namespace w3g
