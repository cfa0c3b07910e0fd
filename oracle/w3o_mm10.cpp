// w3o_mm10.cpp -- the oracle's restatement of WARP3D's mm10 crystal
// plasticity for one Gauss point with one fcc or bcc (12-system) crystal, isotropic
// elasticity and Voce hardening. TEST INFRASTRUCTURE ONLY.
//
// Follows, statement by statement:
//   mm10 / mm10_a_do_crystal / mm10_a_crystal_avgs / mm10_a_store_crystal
//     (src/mm10_a.f:29-362), mm10_tangent (:664-840), mm10_setup
//     (:852-986), mm10_store_cryhist (:998-1089), mm10_solve_crystal
//     (:1102-1181), mm10_update_euler_angles (:1195-1245), mm10_atan2,
//     mm10_rotation_matrix (:1310-1387), mm10_rt2rve/rvw, et2ev, wt2wv,
//     mm10_setup_np1 (:1689-1765), mm10_init_*_hist, mm10_init_voche,
//     mm10_setup_voche (:2071-2117), mm10_copy_cc_hist (:2493-2600),
//     mm10_solve_strup (:2657-2897), mm10_solve (:2901-3360),
//     mm10_update_rotation, mm10_expmw3x3, mm10_output (:3362-3740);
//   mm10_formR2 / formJ11 / formJ12 / formJ21 / formJ22 / formJ / formR /
//     formR1 / form_dbarp / form_wbarp / form_wp / symsw / symswmat / iw /
//     slipinc / rs and the Voce functions (src/mm10_b.f:63-2082);
//   setup_mm10_rknstr (src/rknstr.f:1568-2027) and the fcc / bcc slip systems of
//     finalize_new_crystal (src/mod_crystals.f:440-596).
//
// LAPACK/BLAS calls of the reference (MKL, not part of the sources) are
// restated with the reference-BLAS/LAPACK algorithms: DGESV = unblocked
// partial-pivot LU (first max |a| pivot, reciprocal column scaling) +
// unit-lower and upper triangular solves; DPOSV = unblocked upper
// Cholesky + the two triangular solves; DGER and DGEMM in column order.
// The isotropic stiffness is formed in closed form (lambda, mu) rather
// than by the DSYTRF/DSYTRI inverse of the flexibility.
#include "w3o_mm10.h"

#include <cmath>
#include <cstring>

namespace w3o {

namespace {

const double zero = 0.0, one = 1.0, two = 2.0, three = 3.0, half = 0.5;
const double pi = 3.141592653589793, one_eighty = 180.0, onept5 = 1.5, pt1 = 0.1;
const double twothirds = 2.0 / 3.0;
constexpr int NS = MM10_NSLIP;

inline double& M6(double* a, int r, int c) { return a[r + 6 * c]; }
inline double M6(const double* a, int r, int c) { return a[r + 6 * c]; }
inline double& M3(double* a, int r, int c) { return a[r + 3 * c]; }
inline double M3(const double* a, int r, int c) { return a[r + 3 * c]; }
inline double sign1(double b) { return b >= 0.0 ? 1.0 : -1.0; }   // Fortran sign(one, b)

// x^y for y a non-negative integer up to 64 (the slip-rate exponents n,
// n - 1, n - 2 and the Voce exponent m of the usual data): binary
// powering, the same multiplications in the oracle and on the device, a
// few roundings instead of pow's log/exp sequence, which costs ~100 FP64
// instructions on GB300's narrow FP64 pipe; any other y: pow
inline double powr(double x, double y) {
  const int k = (int)y;
  if ((double)k == y && k >= 0 && k <= 64) {
    double r = 1.0, b = x;
    for (int e = k;;) {
      if (e & 1) r = r * b;
      e >>= 1;
      if (!e) break;
      b = b * b;
    }
    return r;
  }
  return std::pow(x, y);
}

// ---- history locations (mm10_set_history_locs, 1 crystal, 0-based) ----
constexpr int H_TAN = 0, H_GRADFE = 36, H_R = 63, H_WORK = 72, H_SLIP = 75;
constexpr int C0 = 87;
constexpr int C_STRESS = C0, C_EULER = C0 + 6, C_RP = C0 + 9, C_D = C0 + 18, C_EPS = C0 + 24,
              C_SLIP = C0 + 30, C_TT = C0 + 42, C_U = C0 + 43, C_TTRATE = C0 + 58, C_EP = C0 + 59,
              C_ED = C0 + 65;
static_assert(C_ED + 6 == MM10_HIST, "history layout");

struct State {   // crystal_state (the members this scope uses)
  double R[9], Rp[9], D[6], stress[6], eps[6], euler[3];
  double tau_tilde, tt_rate, u[15], slip_incs[NS], gradFeinv[27], tangent[36];
  double ms[NS][6], qs[NS][3], qc[NS][3], tau_l[NS], ep[6], ed[6];
  double temp, tinc, dg, mu_harden, work_inc, p_work_inc, p_strain_inc;
  int step, elem, iter, gp;
};

// ---- small BLAS/LAPACK restatements ----------------------------------
// DGESV for n x n, nrhs right-hand sides (b column-major, ldb = n)
int dgesv(int n, int nrhs, double* a, double* b) {
  int ipiv[16];
  int info = 0;
  for (int j = 0; j < n; ++j) {
    int jp = j;
    double amax = std::fabs(a[j + n * j]);
    for (int i = j + 1; i < n; ++i)
      if (std::fabs(a[i + n * j]) > amax) { amax = std::fabs(a[i + n * j]); jp = i; }
    ipiv[j] = jp;
    if (a[jp + n * j] != zero) {
      if (jp != j)
        for (int k = 0; k < n; ++k) { double t = a[j + n * k]; a[j + n * k] = a[jp + n * k]; a[jp + n * k] = t; }
      if (j < n - 1) {
        const double r = one / a[j + n * j];
        for (int i = j + 1; i < n; ++i) a[i + n * j] = r * a[i + n * j];
      }
    } else if (info == 0) {
      info = j + 1;
    }
    for (int k = j + 1; k < n; ++k) {   // DGER, column k
      const double temp = -a[j + n * k];
      if (temp != zero)
        for (int i = j + 1; i < n; ++i) a[i + n * k] = std::fma(a[i + n * j], temp, a[i + n * k]);
    }
  }
  if (info) return info;
  for (int c = 0; c < nrhs; ++c) {
    double* x = b + (size_t)n * c;
    for (int i = 0; i < n; ++i)
      if (ipiv[i] != i) { double t = x[i]; x[i] = x[ipiv[i]]; x[ipiv[i]] = t; }
    for (int k = 0; k < n; ++k)
      if (x[k] != zero)
        for (int i = k + 1; i < n; ++i) x[i] = std::fma(-x[k], a[i + n * k], x[i]);
    for (int k = n - 1; k >= 0; --k)
      if (x[k] != zero) {
        x[k] = x[k] / a[k + n * k];
        for (int i = 0; i < k; ++i) x[i] = std::fma(-x[k], a[i + n * k], x[i]);
      }
  }
  return 0;
}

// DPOSV('U', 6, 1): Cholesky a = U^T U, solve for b
int dposv6(double* a, double* b) {
  const int n = 6;
  for (int j = 0; j < n; ++j) {
    double dot = zero;
    for (int k = 0; k < j; ++k) dot = dot + a[k + n * j] * a[k + n * j];
    double ajj = a[j + n * j] - dot;
    if (ajj <= zero) return j + 1;
    ajj = std::sqrt(ajj);
    a[j + n * j] = ajj;
    for (int jj = j + 1; jj < n; ++jj) {   // DGEMV('T'), alpha = -1
      double temp = zero;
      for (int k = 0; k < j; ++k) temp = temp + a[k + n * jj] * a[k + n * j];
      a[j + n * jj] = a[j + n * jj] + (-one) * temp;
    }
    const double r = one / ajj;
    for (int jj = j + 1; jj < n; ++jj) a[j + n * jj] = r * a[j + n * jj];
  }
  for (int i = 0; i < n; ++i) {   // U^T y = b
    double temp = b[i];
    for (int k = 0; k < i; ++k) temp = temp - a[k + n * i] * b[k];
    b[i] = temp / a[i + n * i];
  }
  for (int k = n - 1; k >= 0; --k)   // U x = y
    if (b[k] != zero) {
      b[k] = b[k] / a[k + n * k];
      for (int i = 0; i < k; ++i) b[i] = b[i] - b[k] * a[i + n * k];
    }
  return 0;
}

// ---- tensor helpers ---------------------------------------------------
void rt2rve(const double* rt, double* rv) {   // mm10_rt2rve
#define RT(a, b) M3(rt, a - 1, b - 1)
#define RV(a, b) M6(rv, a - 1, b - 1)
  RV(1, 1) = RT(1, 1) * RT(1, 1); RV(1, 2) = RT(1, 2) * RT(1, 2); RV(1, 3) = RT(1, 3) * RT(1, 3);
  RV(1, 4) = two * RT(1, 1) * RT(1, 2); RV(1, 5) = two * RT(1, 3) * RT(1, 2); RV(1, 6) = two * RT(1, 1) * RT(1, 3);
  RV(2, 1) = RT(2, 1) * RT(2, 1); RV(2, 2) = RT(2, 2) * RT(2, 2); RV(2, 3) = RT(2, 3) * RT(2, 3);
  RV(2, 4) = two * RT(2, 1) * RT(2, 2); RV(2, 5) = two * RT(2, 3) * RT(2, 2); RV(2, 6) = two * RT(2, 1) * RT(2, 3);
  RV(3, 1) = RT(3, 1) * RT(3, 1); RV(3, 2) = RT(3, 2) * RT(3, 2); RV(3, 3) = RT(3, 3) * RT(3, 3);
  RV(3, 4) = two * RT(3, 1) * RT(3, 2); RV(3, 5) = two * RT(3, 3) * RT(3, 2); RV(3, 6) = two * RT(3, 1) * RT(3, 3);
  RV(4, 1) = RT(1, 1) * RT(2, 1); RV(4, 2) = RT(1, 2) * RT(2, 2); RV(4, 3) = RT(1, 3) * RT(2, 3);
  RV(4, 4) = RT(1, 1) * RT(2, 2) + RT(2, 1) * RT(1, 2); RV(4, 5) = RT(1, 2) * RT(2, 3) + RT(1, 3) * RT(2, 2);
  RV(4, 6) = RT(1, 1) * RT(2, 3) + RT(1, 3) * RT(2, 1);
  RV(5, 1) = RT(2, 1) * RT(3, 1); RV(5, 2) = RT(3, 2) * RT(2, 2); RV(5, 3) = RT(2, 3) * RT(3, 3);
  RV(5, 4) = RT(2, 1) * RT(3, 2) + RT(2, 2) * RT(3, 1); RV(5, 5) = RT(2, 2) * RT(3, 3) + RT(3, 2) * RT(2, 3);
  RV(5, 6) = RT(2, 1) * RT(3, 3) + RT(2, 3) * RT(3, 1);
  RV(6, 1) = RT(1, 1) * RT(3, 1); RV(6, 2) = RT(1, 2) * RT(3, 2); RV(6, 3) = RT(1, 3) * RT(3, 3);
  RV(6, 4) = RT(1, 1) * RT(3, 2) + RT(1, 2) * RT(3, 1); RV(6, 5) = RT(1, 2) * RT(3, 3) + RT(1, 3) * RT(3, 2);
  RV(6, 6) = RT(1, 1) * RT(3, 3) + RT(3, 1) * RT(1, 3);
#undef RV
}

void rt2rvw(const double* rt, double* rv) {   // mm10_rt2rvw
#define RW(a, b) M3(rv, a - 1, b - 1)
  RW(1, 1) = RT(2, 2) * RT(3, 3) - RT(2, 3) * RT(3, 2);
  RW(1, 2) = RT(2, 1) * RT(3, 3) - RT(2, 3) * RT(3, 1);
  RW(1, 3) = RT(2, 1) * RT(3, 2) - RT(2, 2) * RT(3, 1);
  RW(2, 1) = RT(1, 2) * RT(3, 3) - RT(1, 3) * RT(3, 2);
  RW(2, 2) = RT(1, 1) * RT(3, 3) - RT(1, 3) * RT(3, 1);
  RW(2, 3) = RT(1, 1) * RT(3, 2) - RT(1, 2) * RT(3, 1);
  RW(3, 1) = RT(1, 2) * RT(2, 3) - RT(1, 3) * RT(2, 2);
  RW(3, 2) = RT(1, 1) * RT(2, 3) - RT(1, 3) * RT(2, 1);
  RW(3, 3) = RT(1, 1) * RT(2, 2) - RT(1, 2) * RT(2, 1);
#undef RW
#undef RT
}

void mult_type_1(double* a, const double* b, const double* c) {   // [a] = [b][c]
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) M3(a, i, j) = M3(b, i, 0) * M3(c, 0, j) + M3(b, i, 1) * M3(c, 1, j) + M3(b, i, 2) * M3(c, 2, j);
}
void mult_type_2(double* a, const double* b, const double* c) {   // a = [b] c (6x6)
  for (int r = 0; r < 6; ++r) a[r] = M6(b, r, 0) * c[0];
  for (int j = 1; j < 6; ++j)
    for (int r = 0; r < 6; ++r) a[r] = a[r] + M6(b, r, j) * c[j];
}
void mult_type_3(double* a, const double* b, const double* c) {   // a = [b] c (3x3)
  for (int r = 0; r < 3; ++r) a[r] = M3(b, r, 0) * c[0] + M3(b, r, 1) * c[1] + M3(b, r, 2) * c[2];
}
void mult_type_3t(double* a, const double* b, const double* c) {   // [a] = [b][c]^T
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) M3(a, i, j) = M3(b, i, 0) * M3(c, j, 0) + M3(b, i, 1) * M3(c, j, 1) + M3(b, i, 2) * M3(c, j, 2);
}
void mult_type_4(double* a, const double* b, const double* c, const double* d, double cst) {   // a = [b]c + cst d
  for (int r = 0; r < 6; ++r) a[r] = cst * d[r];
  for (int j = 0; j < 6; ++j)
    for (int r = 0; r < 6; ++r) a[r] = a[r] + M6(b, r, j) * c[j];
}

// The products of the local solve's inner loops (resolved shears, plastic
// strain rate and spin, [C] times a vector, the Jacobian's outer products,
// the LU updates) are fused multiply-adds in a fixed order, as on the
// device (on FMA hardware the reference's compiler contracts them as
// well); everything else stays unfused (-ffp-contract=off).
void mult_type_2f(double* a, const double* b, const double* c) {   // a = [b] c, fused
  for (int r = 0; r < 6; ++r) a[r] = M6(b, r, 0) * c[0];
  for (int j = 1; j < 6; ++j)
    for (int r = 0; r < 6; ++r) a[r] = std::fma(M6(b, r, j), c[j], a[r]);
}
void mult_type_4f(double* a, const double* b, const double* c, const double* d, double cst) {   // fused
  for (int r = 0; r < 6; ++r) a[r] = cst * d[r];
  for (int j = 0; j < 6; ++j)
    for (int r = 0; r < 6; ++r) a[r] = std::fma(M6(b, r, j), c[j], a[r]);
}

void symsw(const double* s, const double* w, double* sw) {   // mm10_symsw
  sw[0] = s[3] * w[2] - s[5] * w[1];
  sw[1] = s[3] * w[2] - s[4] * w[0];
  sw[2] = s[5] * w[1] + s[4] * w[0];
  sw[3] = half * (w[2] * (s[0] - s[1]) + w[0] * s[5] - w[1] * s[4]);
  sw[4] = half * (w[0] * (s[1] - s[2]) + w[1] * s[3] + w[2] * s[5]);
  sw[5] = half * (w[1] * (s[0] - s[2]) + w[0] * s[3] - w[2] * s[4]);
}

void iw_mat(const double* w, double* iw) {   // mm10_iw
  for (int k = 0; k < 36; ++k) iw[k] = zero;
#define IW(a, b) M6(iw, a - 1, b - 1)
  IW(1, 4) = two * w[2]; IW(1, 6) = -two * w[1]; IW(2, 4) = two * w[2]; IW(2, 5) = -two * w[0];
  IW(3, 5) = two * w[0]; IW(3, 6) = two * w[1];
  IW(4, 1) = w[2]; IW(4, 2) = -w[2]; IW(4, 5) = -w[1]; IW(4, 6) = w[0];
  IW(5, 2) = w[0]; IW(5, 3) = -w[0]; IW(5, 4) = w[1]; IW(5, 6) = w[2];
  IW(6, 1) = w[1]; IW(6, 3) = -w[1]; IW(6, 4) = w[0]; IW(6, 5) = -w[2];
#undef IW
}

// ---- Voce slip law (mm10_b.f:1813-2082) -------------------------------
double rs_of(const State& np1, const double* stress, int i) {
  double r = stress[0] * np1.ms[i][0];
  for (int k = 1; k < 6; ++k) r = std::fma(stress[k], np1.ms[i][k], r);
  return r;
}
double slipinc_of(const CrystalProps& p, const State& np1, const double* stress, double tt, int i) {
  const double rs = rs_of(np1, stress, i);
  return np1.dg / tt * powr(std::fabs(rs / tt), p.rate_n - one) * rs;
}

void form_dbarp(const CrystalProps& p, const State& np1, const double* stress, double tt, double* dbar) {
  for (int k = 0; k < 6; ++k) dbar[k] = zero;
  for (int i = 0; i < NS; ++i) {
    const double slipinc = slipinc_of(p, np1, stress, tt, i);
    const double rs = rs_of(np1, stress, i);
    const double f = rs * np1.tinc * p.iD_v + slipinc;
    for (int k = 0; k < 6; ++k) dbar[k] = std::fma(f, np1.ms[i][k], dbar[k]);
  }
}
void form_wbarp(const CrystalProps& p, const State& np1, const double* stress, double tt, double* w) {
  for (int k = 0; k < 3; ++k) w[k] = zero;
  for (int i = 0; i < NS; ++i) {
    const double slipinc = slipinc_of(p, np1, stress, tt, i);
    for (int k = 0; k < 3; ++k) w[k] = w[k] + slipinc * np1.qs[i][k];
    const double rs = rs_of(np1, stress, i);
    for (int k = 0; k < 3; ++k) w[k] = w[k] + rs * np1.tinc * p.iD_v * np1.qs[i][k];
  }
}
void form_wp(const CrystalProps& p, const State& np1, const double* stress, double tt, double* w) {
  for (int k = 0; k < 3; ++k) w[k] = zero;
  for (int i = 0; i < NS; ++i) {
    const double slipinc = slipinc_of(p, np1, stress, tt, i);
    for (int k = 0; k < 3; ++k) w[k] = std::fma(slipinc, np1.qc[i][k], w[k]);
    const double rs = rs_of(np1, stress, i);
    for (int k = 0; k < 3; ++k) w[k] = std::fma(rs * np1.tinc * p.iD_v, np1.qc[i][k], w[k]);
  }
}

void formR1(const CrystalProps& p, const State& np1, const State& n, const double* stress, double tt, double* R1) {
  double dbarp[6], wp[3], symTW[6], wv1[6], wv2[6];
  form_dbarp(p, np1, stress, tt, dbarp);
  form_wp(p, np1, stress, tt, wp);
  symsw(stress, wp, symTW);
  for (int k = 0; k < 6; ++k) wv1[k] = np1.D[k] - dbarp[k];
  mult_type_2f(wv2, p.stiffness, wv1);
  for (int k = 0; k < 6; ++k) R1[k] = stress[k] - n.stress[k] - wv2[k] + two * symTW[k];
}

// formR2 with mm10_h_voche; stores np1.tt_rate
double formR2(const CrystalProps& p, State& np1, const State& n, const double* stress, double tt) {
  double h = zero;
  for (int i = 0; i < NS; ++i) {
    const double slipinc = slipinc_of(p, np1, stress, tt, i);
    const double h_term = one - (tt - p.tau_y) / p.tau_v + np1.tau_l[i] / (tt - p.tau_y);
    h = std::fma(powr(std::fabs(h_term), p.voche_m) * sign1(h_term), std::fabs(slipinc), h);
  }
  h = n.tau_tilde + p.theta_0 * h;
  np1.tt_rate = (h - n.tau_tilde) / np1.tinc;
  return tt - h;
}

void formR(const CrystalProps& p, State& np1, const State& n, const double* x, double* R) {
  formR1(p, np1, n, x, x[6], R);
  R[6] = formR2(p, np1, n, x, x[6]);
}

void symswmat(const double* s, const State& np1, double sw[NS][6]) {
  for (int i = 0; i < NS; ++i) {
    const double* w = np1.qc[i];
    sw[i][0] = s[3] * w[2] - s[5] * w[1];
    sw[i][1] = s[3] * w[2] - s[4] * w[0];
    sw[i][2] = s[5] * w[1] + s[4] * w[0];
    sw[i][3] = half * (w[2] * (s[0] - s[1]) + w[0] * s[5] - w[1] * s[4]);
    sw[i][4] = half * (w[0] * (s[1] - s[2]) + w[1] * s[3] + w[2] * s[5]);
    sw[i][5] = half * (w[1] * (s[0] - s[2]) + w[0] * s[3] - w[2] * s[4]);
  }
}

void dgdt_voche(const CrystalProps& p, const State& np1, const double* stress, double tt, double* dgdt) {
  for (int s = 0; s < NS; ++s) {
    const double rs = rs_of(np1, stress, s);
    double d = powr(std::fabs(rs), p.rate_n - one);
    d = np1.dg * p.rate_n / powr(tt, p.rate_n) * d;
    d = d + np1.tinc * p.iD_v;
    dgdt[s] = d;
  }
}

void formJ11(const CrystalProps& p, const State& np1, const double* stress, double tt, double* J11) {
  double symtq[NS][6], dgdt[NS], wv[6], wp[3], Iw[36];
  for (int k = 0; k < 36; ++k) J11[k] = zero;
  symswmat(stress, np1, symtq);
  dgdt_voche(p, np1, stress, tt, dgdt);
  for (int i = 0; i < NS; ++i) {
    mult_type_4f(wv, p.stiffness, np1.ms[i], symtq[i], two);
    for (int c = 0; c < 6; ++c) {   // DGER
      const double temp = dgdt[i] * np1.ms[i][c];
      if (temp != zero)
        for (int r = 0; r < 6; ++r) M6(J11, r, c) = std::fma(wv[r], temp, M6(J11, r, c));
    }
  }
  form_wp(p, np1, stress, tt, wp);
  iw_mat(wp, Iw);
  for (int k = 0; k < 36; ++k) J11[k] = J11[k] + Iw[k];
  for (int i = 0; i < 6; ++i) M6(J11, i, i) = M6(J11, i, i) + one;
}

void formJ(const CrystalProps& p, const State& np1, const double* x, double* J /* 7x7 column-major */) {
  const double* stress = x;
  const double tt = x[6];
  double J11[36], J12[6], J21[6], J22;
  formJ11(p, np1, stress, tt, J11);
  // J12 (mm10_formJ12 with mm10_dgdh_voche)
  {
    double symtq[NS][6], tempmat[6];
    for (int k = 0; k < 6; ++k) J12[k] = zero;
    symswmat(stress, np1, symtq);
    for (int i = 0; i < NS; ++i) {
      const double dgam = slipinc_of(p, np1, stress, tt, i);
      const double dgdtt = -p.rate_n / tt * dgam;
      mult_type_4f(tempmat, p.stiffness, np1.ms[i], symtq[i], two);
      const double temp = one * dgdtt;
      if (temp != zero)
        for (int r = 0; r < 6; ++r) J12[r] = std::fma(tempmat[r], temp, J12[r]);
    }
  }
  // J21 = -estress_voche
  {
    double et[6] = {zero, zero, zero, zero, zero, zero};
    for (int i = 0; i < NS; ++i) {
      const double rs = rs_of(np1, stress, i);
      const double h_term = one - (tt - p.tau_y) / p.tau_v + np1.tau_l[i] / (tt - p.tau_y);
      const double f = powr(std::fabs(h_term), p.voche_m) * sign1(h_term) * powr(std::fabs(rs), p.rate_n - two) * rs;
      for (int k = 0; k < 6; ++k) et[k] = std::fma(f, np1.ms[i][k], et[k]);
    }
    const double f = p.theta_0 * np1.dg * p.rate_n / powr(tt, p.rate_n);
    for (int k = 0; k < 6; ++k) J21[k] = -(f * et[k]);
  }
  // J22 = ehard_voche, restated with the reference's sign(one, slipinc)
  // factor in the rate term: the derivative of |slipinc| with respect to
  // tau_tilde carries no such factor, so J22 differs from dR2/dtau_tilde
  // wherever slips are negative and the local Newton iteration converges
  // linearly there (as the reference's does)
  {
    double etau = zero;
    for (int i = 0; i < NS; ++i) {
      const double slipinc = slipinc_of(p, np1, stress, tt, i);
      const double h_term = one - (tt - p.tau_y) / p.tau_v + np1.tau_l[i] / (tt - p.tau_y);
      const double d = tt - p.tau_y;
      etau = etau + (p.voche_m * (-one / p.tau_v - np1.tau_l[i] / (d * d)) * std::fabs(slipinc) / std::fabs(h_term) -
                     std::fabs(slipinc) * p.rate_n / tt * sign1(h_term) * sign1(slipinc)) *
                        powr(std::fabs(h_term), p.voche_m);
    }
    etau = p.theta_0 * etau;
    J22 = one - etau;
  }
  for (int c = 0; c < 6; ++c)
    for (int r = 0; r < 6; ++r) J[r + 7 * c] = M6(J11, r, c);
  for (int r = 0; r < 6; ++r) J[r + 7 * 6] = J12[r];
  for (int c = 0; c < 6; ++c) J[6 + 7 * c] = J21[c];
  J[6 + 7 * 6] = J22;
}

// ---- state set-up -------------------------------------------------------
void setup_np1(const double* Rur, const double* dstrain, double dt, double T, int step, int elem, int iter, int gp,
               State& np1) {
  np1.temp = T; np1.tinc = dt; np1.step = step; np1.elem = elem; np1.iter = iter; np1.gp = gp;
  np1.dg = zero; np1.mu_harden = zero; np1.work_inc = zero; np1.p_work_inc = zero; np1.p_strain_inc = zero;
  for (int i = 0; i < 6; ++i) { np1.D[i] = dstrain[i]; np1.stress[i] = zero; np1.eps[i] = zero; }
  for (int i = 0; i < 3; ++i) np1.euler[i] = zero;
  for (int i = 0; i < NS; ++i) { np1.tau_l[i] = zero; np1.slip_incs[i] = zero; }
  np1.tau_tilde = zero; np1.tt_rate = zero;
  for (int i = 0; i < 15; ++i) np1.u[i] = zero;
  for (int k = 0; k < 9; ++k) { np1.R[k] = Rur[k]; np1.Rp[k] = zero; }
  for (int k = 0; k < 27; ++k) np1.gradFeinv[k] = zero;
  for (int k = 0; k < 36; ++k) np1.tangent[k] = zero;
  std::memset(np1.ms, 0, sizeof(np1.ms));
  std::memset(np1.qs, 0, sizeof(np1.qs));
  std::memset(np1.qc, 0, sizeof(np1.qc));
  for (int i = 0; i < 6; ++i) { np1.ep[i] = zero; np1.ed[i] = zero; }
}

void setup(const CrystalProps& p, State& np1, const State& n) {   // mm10_setup
  const double t1 = np1.D[0] * np1.D[0] + np1.D[1] * np1.D[1] + np1.D[2] * np1.D[2];
  const double t2 = np1.D[3] * np1.D[3] + np1.D[4] * np1.D[4] + np1.D[5] * np1.D[5];
  np1.dg = std::sqrt(twothirds * (t1 + half * t2));
  double trans_nRp[9], RE[36], RW[9], work[9], RWC[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) M3(trans_nRp, i, j) = M3(n.Rp, j, i);
  rt2rve(trans_nRp, RE);
  rt2rvw(trans_nRp, RW);
  mult_type_1(work, np1.R, trans_nRp);
  rt2rvw(work, RWC);
  for (int i = 0; i < NS; ++i) {
    mult_type_2(np1.ms[i], RE, p.ms[i]);
    mult_type_3(np1.qs[i], RW, p.qs[i]);
    mult_type_3(np1.qc[i], RWC, p.qs[i]);
  }
  np1.mu_harden = M6(p.stiffness, 5, 5);   // mm10_setup_voche
  // geometric hardening (mm10_a.f:921-984): lattice curvature of n
#define GF(i, j, k) n.gradFeinv[(i) + 3 * (j) + 9 * (k)]
  double curv[3][3][3];
  for (int i = 0; i < 3; ++i) {
    curv[i][0][0] = GF(i, 0, 0) - GF(i, 0, 0);
    curv[i][0][1] = GF(i, 0, 1) - GF(i, 1, 0);
    curv[i][0][2] = GF(i, 0, 2) - GF(i, 2, 0);
    curv[i][1][0] = GF(i, 1, 0) - GF(i, 0, 1);
    curv[i][1][1] = GF(i, 1, 1) - GF(i, 1, 1);
    curv[i][1][2] = GF(i, 1, 2) - GF(i, 2, 1);
    curv[i][2][0] = GF(i, 2, 0) - GF(i, 0, 2);
    curv[i][2][1] = GF(i, 2, 1) - GF(i, 1, 2);
    curv[i][2][2] = GF(i, 2, 2) - GF(i, 2, 2);
  }
#undef GF
  const double alpha = 1.0 / 3.0;
  const double cst = p.k_0 * p.burgers * alpha * alpha * np1.mu_harden * np1.mu_harden / two / p.theta_0;
  for (int t = 0; t < NS; ++t) {
    double wv[3], cn[3], tm[3] = {zero, zero, zero};
    mult_type_3(wv, trans_nRp, p.ns[t]);
    mult_type_3(cn, n.R, wv);
    for (int i = 0; i < 3; ++i)
      tm[i] = tm[i] + half * (-curv[i][0][1] * cn[2] + curv[i][0][2] * cn[1] + curv[i][1][0] * cn[2] -
                              curv[i][1][2] * cn[0] - curv[i][2][0] * cn[1] + curv[i][2][1] * cn[0]);
    np1.tau_l[t] = cst * std::sqrt(tm[0] * tm[0] + tm[1] * tm[1] + tm[2] * tm[2]);
  }
}

// mm10_solve: predictor on the stress with extrapolated hardening, then
// Newton on (stress, tau_tilde) with line search. J receives the last
// Jacobian (mm10_tangent reads it).
void solve(const CrystalProps& p, State& np1, const State& n, double* stress, double& tt, bool& fail, double dtinc,
           double* J) {
  const double c = 1.0e-4, red = 0.5;
  const int mls = 10, mmin = 1;
  double x[7];
  for (int k = 0; k < 6; ++k) x[k] = stress[k];
  x[6] = tt;
  double inR1;
  // ---- mm10_solve_predict ----
  {
    int iter = 0;
    double x1[6], x2, d1[6], d2[6], R1[6], J11[36], mJ11[36], dx1[6], xnew1[6], wv[6];
    for (int k = 0; k < 6; ++k) x1[k] = x[k];
    const double dt = dtinc;
    for (int k = 0; k < 6; ++k) d1[k] = np1.D[k];
    double dtrace = (d1[0] + d1[1] + d1[2]) / three;
    d1[0] = d1[0] - dtrace; d1[1] = d1[1] - dtrace; d1[2] = d1[2] - dtrace;
    double t1 = d1[0] * d1[0] + d1[1] * d1[1] + d1[2] * d1[2];
    double t2 = d1[3] * d1[3] + d1[4] * d1[4] + d1[5] * d1[5];
    if (t1 + t2 == zero) for (int k = 0; k < 6; ++k) d1[k] = zero;
    else { const double s = std::sqrt(t1 + t2); for (int k = 0; k < 6; ++k) d1[k] = d1[k] / s; }
    for (int k = 0; k < 6; ++k) d2[k] = n.D[k];
    dtrace = (d2[0] + d2[1] + d2[2]) / three;
    d2[0] = d2[0] - dtrace; d2[1] = d2[1] - dtrace; d2[2] = d2[2] - dtrace;
    t1 = d2[0] * d2[0] + d2[1] * d2[1] + d2[2] * d2[2];
    t2 = d2[3] * d2[3] + d2[4] * d2[4] + d2[5] * d2[5];
    if (t1 + t2 == zero) for (int k = 0; k < 6; ++k) d2[k] = zero;
    else { const double s = std::sqrt(t1 + t2); for (int k = 0; k < 6; ++k) d2[k] = d2[k] / s; }
    t1 = d1[0] * d2[0] + d1[1] * d2[1] + d1[2] * d2[2];
    t2 = d1[3] * d2[3] + d1[4] * d2[4] + d1[5] * d2[5];
    const double cos_ang = std::fmax(t1 + t2, zero);
    x2 = x[6] + cos_ang * n.tt_rate * dt;
    formR1(p, np1, n, x1, x2, R1);
    double nR1 = std::sqrt(R1[0] * R1[0] + R1[1] * R1[1] + R1[2] * R1[2] + R1[3] * R1[3] + R1[4] * R1[4] + R1[5] * R1[5]);
    inR1 = nR1;
    while (nR1 > p.atol1 && nR1 / inR1 > p.rtol1) {
      formJ11(p, np1, x1, x2, J11);
      for (int k = 0; k < 6; ++k) dx1[k] = R1[k];
      for (int k = 0; k < 36; ++k) mJ11[k] = -J11[k];
      dgesv(6, 1, mJ11, dx1);
      double alpha = one;
      double dotR1 = R1[0] * R1[0] + R1[1] * R1[1] + R1[2] * R1[2] + R1[3] * R1[3] + R1[4] * R1[4] + R1[5] * R1[5];
      const double ls1 = half * dotR1;
      for (int j = 0; j < 6; ++j)   // mult_type_2t: trans(J11) R1
        wv[j] = M6(J11, 0, j) * R1[0] + M6(J11, 1, j) * R1[1] + M6(J11, 2, j) * R1[2] + M6(J11, 3, j) * R1[3] +
                M6(J11, 4, j) * R1[4] + M6(J11, 5, j) * R1[5];
      const double ls2 = c * (dx1[0] * wv[0] + dx1[1] * wv[1] + dx1[2] * wv[2] + dx1[3] * wv[3] + dx1[4] * wv[4] +
                              dx1[5] * wv[5]);
      int ls = 0;
      for (;;) {
        const double nlsx = ls1 + ls2 * alpha;
        for (int k = 0; k < 6; ++k) xnew1[k] = x1[k] + alpha * dx1[k];
        formR1(p, np1, n, xnew1, x2, R1);
        dotR1 = R1[0] * R1[0] + R1[1] * R1[1] + R1[2] * R1[2] + R1[3] * R1[3] + R1[4] * R1[4] + R1[5] * R1[5];
        nR1 = std::sqrt(dotR1);
        const double nRs = half * dotR1;
        if (nRs <= nlsx || ls > mls) {
          for (int k = 0; k < 6; ++k) x1[k] = xnew1[k];
          break;
        }
        alpha = red * alpha;
        ++ls;
      }
      ++iter;
      bool nan = false;
      for (int k = 0; k < 6; ++k) nan = nan || std::isnan(x1[k]);
      if (iter > p.miter || nan) { fail = true; return; }
    }
    for (int k = 0; k < 6; ++k) x[k] = x1[k];
    x[6] = x2;
  }
  // ---- mm10_solve_update ----
  {
    int iter = 0;
    double R[7], dx[7], mJ[49], xnew[7], wv[7];
    formR(p, np1, n, x, R);
    double dotR = zero;
    for (int k = 0; k < 7; ++k) dotR = dotR + R[k] * R[k];
    double nR = std::sqrt(dotR);
    double inR = nR;
    if (inR == zero) inR = inR1;
    while ((nR > p.atol && nR / inR > p.rtol) || iter < mmin) {
      formJ(p, np1, x, J);
      for (int k = 0; k < 7; ++k) dx[k] = R[k];
      for (int k = 0; k < 49; ++k) mJ[k] = -J[k];
      dgesv(7, 1, mJ, dx);
      double alpha = one;
      dotR = zero;
      for (int k = 0; k < 7; ++k) dotR = dotR + R[k] * R[k];
      const double ls1 = half * dotR;
      for (int i = 0; i < 7; ++i) {   // DGEMM('T','N'): J^T R
        double temp = zero;
        for (int l = 0; l < 7; ++l) temp = temp + J[l + 7 * i] * R[l];
        wv[i] = one * temp;
      }
      double dxw = zero;
      for (int k = 0; k < 7; ++k) dxw = dxw + dx[k] * wv[k];
      const double ls2 = c * dxw;
      int ls = 0;
      for (;;) {
        const double nlsx = ls1 + ls2 * alpha;
        for (int k = 0; k < 7; ++k) xnew[k] = x[k] + alpha * dx[k];
        formR(p, np1, n, xnew, R);
        dotR = zero;
        for (int k = 0; k < 7; ++k) dotR = dotR + R[k] * R[k];
        nR = std::sqrt(dotR);
        const double nRs = half * dotR;
        if (nRs <= nlsx || ls > mls) {
          for (int k = 0; k < 7; ++k) x[k] = xnew[k];
          break;
        }
        alpha = red * alpha;
        ++ls;
      }
      ++iter;
      bool nan = false;
      for (int k = 0; k < 7; ++k) nan = nan || std::isnan(x[k]);
      if (iter > p.miter || nan) { fail = true; return; }
    }
  }
  for (int k = 0; k < 6; ++k) stress[k] = x[k];
  tt = x[6];
}

// mm10_solve_strup; returns fail
bool solve_strup(const CrystalProps& p, State& np1, const State& n, bool iter0off, bool& no_load, double* J) {
  const double mult = 0.5;
  const int mcuts = 4;
  double frac = zero, step = one;
  int cuts = 0;
  double stress[6], ostress[6], tt, ott;
  for (int k = 0; k < 6; ++k) { stress[k] = n.stress[k]; ostress[k] = stress[k]; }
  tt = n.tau_tilde; ott = tt;
  setup(p, np1, n);
  bool fail = false;
  const double temp1 = np1.D[0] * np1.D[0] + np1.D[1] * np1.D[1] + np1.D[2] * np1.D[2] + np1.D[3] * np1.D[3] +
                       np1.D[4] * np1.D[4] + np1.D[5] * np1.D[5];
  const double temp2 = stress[0] * stress[0] + stress[1] * stress[1] + stress[2] * stress[2] +
                       stress[3] * stress[3] + stress[4] * stress[4] + stress[5] * stress[5];
  no_load = (temp2 == zero) && (temp1 == zero);
  double curr_tt_rate = zero;
  if (iter0off || no_load) {   // mm10_solve_strup_a
    for (int k = 0; k < 36; ++k) np1.tangent[k] = p.stiffness[k];
    if (!no_load) {
      double R1[6];
      formR1(p, np1, n, stress, tt, R1);
      for (int k = 0; k < 6; ++k) stress[k] = stress[k] - R1[k];
    }
    curr_tt_rate = zero;
  } else {   // mm10_solve_strup_iterate
    State curr;
    while (frac < one) {
      double D_work[6];
      for (int k = 0; k < 6; ++k) D_work[k] = np1.D[k] * (step + frac);
      const double tinc_work = np1.tinc * (step + frac);
      const double temp_work = (np1.temp - n.temp) * (step + frac) + n.temp;
      setup_np1(np1.R, D_work, tinc_work, temp_work, np1.step, np1.elem, np1.iter, np1.gp, curr);
      setup(p, curr, n);
      tt = n.tau_tilde;
      solve(p, curr, n, stress, tt, fail, np1.tinc * step, J);
      if (fail) {
        for (int k = 0; k < 6; ++k) stress[k] = ostress[k];
        tt = ott;
        step = step * mult;
        ++cuts;
        if (cuts > mcuts) break;
        fail = false;
      } else {
        for (int k = 0; k < 6; ++k) ostress[k] = stress[k];
        ott = tt;
        frac = frac + step;
      }
    }
    bool bad = fail || std::isnan(tt);
    for (int k = 0; k < 6; ++k) bad = bad || std::isnan(stress[k]);
    if (bad) {
      for (int k = 0; k < 6; ++k) np1.stress[k] = n.stress[k];
      np1.tau_tilde = n.tau_tilde;
      return true;
    }
    curr_tt_rate = curr.tt_rate;
  }
  for (int k = 0; k < 6; ++k) np1.stress[k] = stress[k];
  np1.tau_tilde = tt;
  np1.tt_rate = curr_tt_rate;
  return false;
}

void tangent(const CrystalProps& p, State& np1, const double* Jmat) {   // mm10_tangent
  double J11[36], J12[6], J21[6], J22, JJ[36], JR[36], beta[12];
  for (int c = 0; c < 6; ++c)
    for (int r = 0; r < 6; ++r) M6(J11, r, c) = Jmat[r + 7 * c];
  for (int r = 0; r < 6; ++r) J12[r] = Jmat[r + 7 * 6];
  for (int c = 0; c < 6; ++c) J21[c] = Jmat[6 + 7 * c];
  J22 = Jmat[6 + 7 * 6];
  // ed = 0 and dgammadd = 0 (Voce): JA = 0, JB = 0, JR = stiffness
  for (int k = 0; k < 36; ++k) JJ[k] = J11[k];
  double alpha = J22;
  for (int c = 0; c < 6; ++c) beta[c] = J21[c];
  for (int c = 6; c < 12; ++c) beta[c] = zero;
  dgesv(1, 12, &alpha, beta);
  for (int j = 0; j < 6; ++j) {   // DGEMM: JJ = JJ - J12 beta(:,1:6)
    const double temp = -one * beta[j];
    if (temp != zero)
      for (int i = 0; i < 6; ++i) M6(JJ, i, j) = M6(JJ, i, j) + temp * J12[i];
  }
  for (int k = 0; k < 36; ++k) JR[k] = p.stiffness[k];
  dgesv(6, 6, JJ, JR);
  for (int k = 0; k < 36; ++k) np1.tangent[k] = JR[k];
}

void update_rotation(const CrystalProps& p, State& np1, const State& n) {
  double w[3], wt[9], a[9];
  form_wbarp(p, np1, np1.stress, np1.tau_tilde, w);
  // mm10_wv2wt
  M3(wt, 0, 0) = zero; M3(wt, 0, 1) = w[2]; M3(wt, 0, 2) = w[1];
  M3(wt, 1, 0) = -w[2]; M3(wt, 1, 1) = zero; M3(wt, 1, 2) = w[0];
  M3(wt, 2, 0) = -w[1]; M3(wt, 2, 1) = -w[0]; M3(wt, 2, 2) = zero;
  // mm10_expmw3x3
  const double alpha = std::sqrt(M3(wt, 1, 2) * M3(wt, 1, 2) + M3(wt, 0, 2) * M3(wt, 0, 2) + M3(wt, 0, 1) * M3(wt, 0, 1));
  if (alpha < 1.0e-16) {
    for (int k = 0; k < 9; ++k) a[k] = zero;
  } else {
    const double ca = (one - std::cos(alpha)) / (alpha * alpha);
    const double cb = std::sin(alpha) / alpha;
    for (int j = 0; j < 3; ++j) {   // DGEMM: a = ca w w + cb a
      for (int i = 0; i < 3; ++i) a[i + 3 * j] = cb * wt[i + 3 * j];
      for (int l = 0; l < 3; ++l) {
        const double temp = ca * wt[l + 3 * j];
        if (temp != zero)
          for (int i = 0; i < 3; ++i) a[i + 3 * j] = a[i + 3 * j] + temp * wt[i + 3 * l];
      }
    }
  }
  a[0] = a[0] + one; a[4] = a[4] + one; a[8] = a[8] + one;
  mult_type_1(np1.Rp, a, n.Rp);
}

double atan2_2pi(double a, double b) {   // mm10_atan2
  double r = std::atan2(a, b);
  if (r < zero) r = r + two * pi;
  return r;
}

void output(const CrystalProps& p, State& np1, const State& n, double* p_strain_ten_c) {   // mm10_output
  for (int i = 0; i < NS; ++i) np1.slip_incs[i] = slipinc_of(p, np1, np1.stress, np1.tau_tilde, i);
  {   // mm10_update_euler_angles (Kocks, degrees)
    double work1[9], full_rot[9];
    mult_type_3t(work1, np1.Rp, np1.R);
    mult_type_1(full_rot, p.g, work1);
    const double psiK = atan2_2pi(M3(full_rot, 2, 1), M3(full_rot, 2, 0));
    const double phiK = atan2_2pi(M3(full_rot, 1, 2), M3(full_rot, 0, 2));
    if (M3(full_rot, 2, 2) > one) M3(full_rot, 2, 2) = one;
    const double thetaK = std::acos(M3(full_rot, 2, 2));
    np1.euler[0] = one_eighty / pi * psiK;
    np1.euler[1] = one_eighty / pi * thetaK;
    np1.euler[2] = one_eighty / pi * phiK;
  }
  double dif_slp[NS], ed[6], t1, t2;
  for (int i = 0; i < NS; ++i) {
    const double rs = rs_of(np1, np1.stress, i);
    dif_slp[i] = rs * np1.tinc * p.iD_v;
  }
  for (int k = 0; k < 6; ++k) ed[k] = zero;
  for (int i = 0; i < NS; ++i)
    for (int k = 0; k < 6; ++k) ed[k] = ed[k] + dif_slp[i] * np1.ms[i][k];
  for (int k = 0; k < 6; ++k) np1.ed[k] = ed[k] / np1.tinc;
  t1 = ed[0] * ed[0] + ed[1] * ed[1] + ed[2] * ed[2];
  t2 = ed[3] * ed[3] + ed[4] * ed[4] + ed[5] * ed[5];
  double ed_dot = std::sqrt(two / three * (t1 + half * t2));
  ed_dot = ed_dot / np1.tinc;
  np1.u[14] = ed_dot;
  np1.work_inc = np1.stress[0] * np1.D[0] + np1.stress[1] * np1.D[1] + np1.stress[2] * np1.D[2] +
                 np1.stress[3] * np1.D[3] + np1.stress[4] * np1.D[4] + np1.stress[5] * np1.D[5];
  double S[36], eeunrot[6], erot[36], ee[6], dbarp[6], wp[3], ewwe[6], ep[6];
  for (int k = 0; k < 36; ++k) S[k] = p.stiffness[k];
  for (int k = 0; k < 6; ++k) eeunrot[k] = np1.stress[k];
  dposv6(S, eeunrot);
  rt2rve(np1.R, erot);
  mult_type_2(ee, erot, eeunrot);
  for (int k = 0; k < 6; ++k) dbarp[k] = zero;
  for (int i = 0; i < NS; ++i)
    for (int k = 0; k < 6; ++k) dbarp[k] = dbarp[k] + np1.slip_incs[i] * np1.ms[i][k];
  form_wp(p, np1, np1.stress, np1.tau_tilde, wp);
  symsw(ee, wp, ewwe);
  for (int k = 0; k < 6; ++k) ep[k] = dbarp[k] + ewwe[k];
  for (int k = 0; k < 6; ++k) np1.ep[k] = ep[k] / np1.tinc;
  t1 = ep[0] * ep[0] + ep[1] * ep[1] + ep[2] * ep[2];
  t2 = ep[3] * ep[3] + ep[4] * ep[4] + ep[5] * ep[5];
  double ep_dot = std::sqrt(two / three * (t1 + half * t2));
  ep_dot = ep_dot / np1.tinc;
  np1.u[10] = ep_dot;
  for (int k = 0; k < 6; ++k) ep[k] = ep[k] + ed[k];
  for (int k = 0; k < 6; ++k) p_strain_ten_c[k] = ep[k];
  t1 = ep[0] * ep[0] + ep[1] * ep[1] + ep[2] * ep[2];
  t2 = ep[3] * ep[3] + ep[4] * ep[4] + ep[5] * ep[5];
  np1.p_strain_inc = std::sqrt(two / three * (t1 + half * t2));
  np1.p_work_inc = np1.stress[0] * ep[0] + np1.stress[1] * ep[1] + np1.stress[2] * ep[2] + np1.stress[3] * ep[3] +
                   np1.stress[4] * ep[4] + np1.stress[5] * ep[5];
  for (int k = 0; k < 6; ++k) np1.eps[k] = ee[k];
  const double ec_dot = np1.p_strain_inc / np1.tinc;
  double n_eff;
  if (ec_dot > zero) {
    for (int k = 0; k < 6; ++k) ep[k] = ep[k] / np1.tinc;
    double dgdt[NS];
    dgdt_voche(p, np1, np1.stress, np1.tau_tilde, dgdt);
    n_eff = zero;
    for (int i = 0; i < NS; ++i) {
      const double rs = rs_of(np1, np1.stress, i);
      t1 = np1.ms[i][0] * ep[0] + np1.ms[i][1] * ep[1] + np1.ms[i][2] * ep[2];
      t2 = np1.ms[i][3] * ep[3] + np1.ms[i][4] * ep[4] + np1.ms[i][5] * ep[5];
      const double ec_slip = t1 + half * t2;
      t1 = rs * dgdt[i] / ec_dot;
      t2 = ec_slip / ec_dot / np1.tinc;
      n_eff = n_eff + (two / three) * t1 * t2;
    }
  } else {
    n_eff = 1.0e10;
  }
  np1.u[11] = n_eff;
  double s_trace = (np1.stress[0] + np1.stress[1] + np1.stress[2]) / three;
  double se[6];
  for (int k = 0; k < 6; ++k) se[k] = np1.stress[k];
  se[0] = se[0] - s_trace; se[1] = se[1] - s_trace; se[2] = se[2] - s_trace;
  t1 = se[0] * se[0] + se[1] * se[1] + se[2] * se[2];
  t2 = se[3] * se[3] + se[4] * se[4] + se[5] * se[5];
  s_trace = std::sqrt(onept5 * (t1 + two * t2));
  np1.u[12] = s_trace;
  double B_eff;
  if (ec_dot < 1.0e-100) B_eff = zero;
  else if (n_eff > 100.0) B_eff = -one;
  else B_eff = ec_dot / std::pow(s_trace, n_eff);
  np1.u[13] = B_eff;
  for (int i = 0; i < NS; ++i) np1.slip_incs[i] = np1.slip_incs[i] + dif_slp[i];
  double maxslip = zero;
  int sysID = 0;
  for (int i = 0; i < NS; ++i) {
    const double curslip = std::fabs(np1.slip_incs[i]);
    if (curslip > maxslip) { maxslip = curslip; sysID = i + 1; }
  }
  np1.u[5] = maxslip / np1.tinc;
  np1.u[6] = (double)sysID;
  int numAct = 0;
  maxslip = pt1 * maxslip;
  for (int i = 0; i < NS; ++i)
    if (std::fabs(np1.slip_incs[i]) >= maxslip) ++numAct;
  np1.u[7] = (double)numAct;
}

// slip systems of finalize_new_crystal: fcc, slip_type 1
// (src/mod_crystals.f:440-518), directions b and normals n; bcc, slip_type
// 2 (:519-596), the same two tables with the roles exchanged
void slip_systems(int slip_type, double bi[NS][3], double ni[NS][3]) {
  const double f = 1.0 / std::sqrt(2.0);
  const double v110[NS][3] = {{0, -f, f}, {f, 0, -f}, {-f, f, 0}, {0, f, f}, {f, 0, f}, {f, -f, 0},
                              {0, -f, f}, {-f, 0, -f}, {f, f, 0}, {0, f, f}, {f, 0, -f}, {-f, -f, 0}};
  const double g = 1.0 / std::sqrt(3.0);
  const double v111[NS][3] = {{g, g, g}, {g, g, g}, {g, g, g}, {-g, -g, g}, {-g, -g, g}, {-g, -g, g},
                              {-g, g, g}, {-g, g, g}, {-g, g, g}, {g, -g, g}, {g, -g, g}, {g, -g, g}};
  const bool bcc = slip_type == 2;
  std::memcpy(bi, bcc ? v111 : v110, sizeof(v110));
  std::memcpy(ni, bcc ? v110 : v111, sizeof(v111));
}

}  // namespace

void mm10_element_props(const w3g_crystal& cr, const double* angles, CrystalProps& p) {
  // isotropic stiffness (elastic_type 1), closed form
  const double e = cr.e, nu = cr.nu;
  const double lam = e * nu / ((one + nu) * (one - two * nu));
  const double mu = e / (two * (one + nu));
  double C[36];
  for (int k = 0; k < 36; ++k) C[k] = zero;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) M6(C, i, j) = lam;
  for (int i = 0; i < 3; ++i) M6(C, i, i) = lam + two * mu;
  for (int i = 3; i < 6; ++i) M6(C, i, i) = mu;
  // mm10_rotation_matrix (Kocks, degrees)
  const double a = angles[0] * pi / one_eighty, b = angles[1] * pi / one_eighty, c = angles[2] * pi / one_eighty;
  const double psi = a, theta = b, phi = c;
  double* r = p.g;
  M3(r, 0, 0) = -std::sin(psi) * std::sin(phi) - std::cos(psi) * std::cos(phi) * std::cos(theta);
  M3(r, 0, 1) = std::cos(psi) * std::sin(phi) - std::sin(psi) * std::cos(phi) * std::cos(theta);
  M3(r, 0, 2) = std::cos(phi) * std::sin(theta);
  M3(r, 1, 0) = std::sin(psi) * std::cos(phi) - std::cos(psi) * std::sin(phi) * std::cos(theta);
  M3(r, 1, 1) = -std::cos(psi) * std::cos(phi) - std::sin(psi) * std::sin(phi) * std::cos(theta);
  M3(r, 1, 2) = std::sin(phi) * std::sin(theta);
  M3(r, 2, 0) = std::cos(psi) * std::sin(theta);
  M3(r, 2, 1) = std::sin(psi) * std::sin(theta);
  M3(r, 2, 2) = std::cos(theta);
  for (int k = 0; k < 3; ++k) p.angles[k] = angles[k];
  double trans_rot[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) M3(trans_rot, i, j) = M3(r, j, i);
  double bi[NS][3], ni[NS][3];
  slip_systems(cr.slip_type, bi, ni);
  for (int s = 0; s < NS; ++s) {
    double bs[3], ns[3], A[9];
    mult_type_3(bs, trans_rot, bi[s]);
    mult_type_3(ns, trans_rot, ni[s]);
    for (int k = 0; k < 3; ++k) p.ns[s][k] = ns[k];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) M3(A, i, j) = bs[i] * ns[j];
    double As[9], Aa[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        M3(As, i, j) = half * (M3(A, i, j) + M3(A, j, i));
        M3(Aa, i, j) = half * (M3(A, i, j) - M3(A, j, i));
      }
    p.ms[s][0] = M3(As, 0, 0); p.ms[s][1] = M3(As, 1, 1); p.ms[s][2] = M3(As, 2, 2);
    p.ms[s][3] = two * M3(As, 0, 1); p.ms[s][4] = two * M3(As, 1, 2); p.ms[s][5] = two * M3(As, 0, 2);
    p.qs[s][0] = M3(Aa, 1, 2); p.qs[s][1] = M3(Aa, 0, 2); p.qs[s][2] = M3(Aa, 0, 1);
  }
  // rotate the stiffness: Rstiff C Rstiff^T (Rstiff = rt2rve(trans_rot))
  double Rs[36], temp[36];
  rt2rve(trans_rot, Rs);
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      double s = zero;
      for (int k = 0; k < 6; ++k) s = s + M6(C, i, k) * M6(Rs, j, k);
      M6(temp, i, j) = s;
    }
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      double s = zero;
      for (int k = 0; k < 6; ++k) s = s + M6(Rs, i, k) * M6(temp, k, j);
      M6(p.stiffness, i, j) = s;
    }
  p.rate_n = cr.harden_n; p.tau_y = cr.tau_y; p.tau_v = cr.tau_v; p.theta_0 = cr.theta_o;
  p.voche_m = cr.voche_m; p.iD_v = cr.iD_v; p.k_0 = cr.k_o; p.burgers = cr.b;
  p.atol = cr.atol; p.atol1 = cr.atol1; p.rtol = cr.rtol; p.rtol1 = cr.rtol1; p.miter = cr.miter;
}

int mm10_point(const CrystalProps& p, int step, int iter, bool extrapolated_du, double dt, int elem, int gpn,
               double* hn, double* hn1, const double* urcs_n, double* urcs_n1, const double* uddt,
               const double* rot_n1) {
  // drive_10_update: iteration 0 without extrapolation (or step 1) is
  // the linear update (src/rstgp1.f:4450-4455)
  bool iter0off = false;
  if (iter == 0) {
    iter0off = !extrapolated_du;
    if (step == 1) iter0off = true;
  }
  if (step == 1) {   // mm10_init_general_hist / _uout_hist / _slip_hist
    for (int k = 0; k < 36; ++k) hn[H_TAN + k] = zero;
    for (int k = 0; k < 27; ++k) hn[H_GRADFE + k] = zero;
    for (int k = 0; k < 9; ++k) hn[H_R + k] = (k % 4 == 0) ? one : zero;
    for (int k = 0; k < 3; ++k) hn[H_WORK + k] = zero;
    for (int k = 0; k < NS; ++k) hn[H_SLIP + k] = zero;
    // mm10_init_cc_hist0 with user initial stresses = urcs_n(1:6)
    for (int k = 0; k < 6; ++k) hn[C_STRESS + k] = urcs_n[k];
    for (int k = 0; k < 3; ++k) hn[C_EULER + k] = p.angles[k];
    for (int k = 0; k < 9; ++k) hn[C_RP + k] = (k % 4 == 0) ? one : zero;
    for (int k = 0; k < 6; ++k) { hn[C_D + k] = zero; hn[C_EPS + k] = zero; }
    for (int k = 0; k < NS; ++k) hn[C_SLIP + k] = zero;
    hn[C_TT] = p.tau_y + 1.0e-5;                      // mm10_init_voche
    for (int k = 0; k < 15; ++k) hn[C_U + k] = zero;  // left unset by the reference
  }
  // mm10_copy_cc_hist
  State n, np1;
  std::memset(&n, 0, sizeof(n));
  for (int k = 0; k < 9; ++k) n.R[k] = hn[H_R + k];
  for (int k = 0; k < 27; ++k) n.gradFeinv[k] = hn[H_GRADFE + k];
  for (int k = 0; k < 6; ++k) n.stress[k] = hn[C_STRESS + k];
  for (int k = 0; k < 3; ++k) n.euler[k] = hn[C_EULER + k];
  for (int k = 0; k < 9; ++k) n.Rp[k] = hn[C_RP + k];
  for (int k = 0; k < 6; ++k) { n.D[k] = hn[C_D + k]; n.eps[k] = hn[C_EPS + k]; }
  n.tau_tilde = hn[C_TT];
  for (int k = 0; k < 15; ++k) n.u[k] = hn[C_U + k];
  n.tt_rate = hn[C_TTRATE];
  for (int k = 0; k < 6; ++k) { n.ep[k] = hn[C_EP + k]; n.ed[k] = hn[C_ED + k]; }
  setup_np1(rot_n1, uddt, dt, zero, step, elem, iter, gpn, np1);
  // mm10_solve_crystal
  double J[49];
  for (int k = 0; k < 49; ++k) J[k] = zero;
  bool no_load = false;
  if (solve_strup(p, np1, n, iter0off, no_load, J)) return W3G_LOCAL_FAIL;
  double p_strain_ten_c[6] = {zero, zero, zero, zero, zero, zero};
  if (!(iter0off || no_load)) {
    tangent(p, np1, J);
    if (!p.asymmetric) {   // mm10_a_make_symm_1 unless asymmetric assembly (mm10_a.f:1165-1166)
      double w[36];
      for (int j = 0; j < 6; ++j)
        for (int i = 0; i < 6; ++i) M6(w, i, j) = (M6(np1.tangent, i, j) + M6(np1.tangent, j, i)) * half;
      for (int k = 0; k < 36; ++k) np1.tangent[k] = w[k];
    }
    update_rotation(p, np1, n);
    output(p, np1, n, p_strain_ten_c);
  }
  // mm10_store_cryhist
  for (int k = 0; k < 6; ++k) hn1[C_STRESS + k] = np1.stress[k];
  for (int k = 0; k < 3; ++k) hn1[C_EULER + k] = np1.euler[k];
  for (int k = 0; k < 9; ++k) hn1[C_RP + k] = np1.Rp[k];
  for (int k = 0; k < 6; ++k) { hn1[C_D + k] = np1.D[k]; hn1[C_EPS + k] = np1.eps[k]; }
  for (int k = 0; k < NS; ++k) hn1[C_SLIP + k] = np1.slip_incs[k];
  hn1[C_TT] = np1.tau_tilde;
  for (int k = 0; k < 15; ++k) hn1[C_U + k] = np1.u[k];
  hn1[C_TTRATE] = np1.tt_rate;
  for (int k = 0; k < 6; ++k) { hn1[C_EP + k] = np1.ep[k]; hn1[C_ED + k] = np1.ed[k]; }
  // mm10_a_crystal_avgs (one crystal) + mm10_a_store_crystal
  const double rncry = 1.0;
  for (int k = 0; k < 6; ++k) urcs_n1[k] = np1.stress[k] / rncry;
  for (int k = 0; k < 9; ++k) hn1[H_R + k] = rot_n1[k];
  for (int k = 0; k < 36; ++k) hn1[H_TAN + k] = np1.tangent[k] / rncry;
  for (int k = 0; k < NS; ++k) hn1[H_SLIP + k] = hn[H_SLIP + k] + np1.slip_incs[k] / rncry;
  const double t_work = np1.work_inc / rncry, p_work = np1.p_work_inc / rncry, p_strain = np1.p_strain_inc / rncry;
  urcs_n1[6] = urcs_n[6] + t_work;
  urcs_n1[7] = urcs_n[7] + p_work;
  urcs_n1[8] = urcs_n[8] + p_strain;
  hn1[H_WORK + 0] = hn[H_WORK + 0] + t_work;
  hn1[H_WORK + 1] = hn[H_WORK + 1] + p_work;
  hn1[H_WORK + 2] = hn[H_WORK + 2] + p_strain;
  return 0;
}

}  // namespace w3o
