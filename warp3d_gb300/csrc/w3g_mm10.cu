// w3g_mm10.cu -- recovery of 8-node bricks with mm10 crystal plasticity
// (drive_10_update, src/rstgp1.f:4327-4510 -> mm10, src/mm10_a.f:29-362):
// one fcc crystal per Gauss point, isotropic elasticity, Voce hardening.
//
// The local Newton solve of a Gauss point takes from a few to a few dozen
// iterations and the count varies from point to point, so the recovery of
// these blocks runs as three launches:
//   k_mm10_kin     one CTA per 8 elements, one thread per Gauss point: the
//                  reference-order kinematics (F, polar decompositions,
//                  unrotated strain increment uddt), eps_n1, rot_n1; uddt,
//                  R, F and det F to a per-GP scratch
//   k_mm10_update  persistent: each warp takes 32 Gauss points at a time
//                  from a work queue ordered by the iteration counts of the
//                  previous call (largest first, a counting sort on the
//                  device), so that a warp's lanes run similar numbers of
//                  iterations; one thread solves one Gauss point (mm10 with
//                  mm10_solve_strup / mm10_solve / mm10_tangent /
//                  mm10_output) and writes history1, urcs_n1 and its count
//   k_mm10_forces  one CTA per 8 elements: Cauchy stress, element forces
//                  P = w det[J] sigma F^-T applied to dN/dX, volumes, energies
//
// This translation unit is compiled without multiply-add contraction: the
// local Newton iteration stops on residual tests, and evaluating its
// residuals and Jacobians in the reference's operation order keeps the
// iteration paths (and counts) the oracle's.
#include <algorithm>
#include <cmath>
#include "w3g_internal.cuh"
#include "w3g_elem.cuh"
#include "w3g_math.cuh"

namespace w3g {

namespace {

constexpr int NN = Hex8::NN;
constexpr int NG = Hex8::NG;
constexpr int TOT = Hex8::TOTDOF;
constexpr int kDnSize = NG * 3 * NN + NG;
constexpr int kGeo = 3 * NN + 1;
constexpr int NS = kSlip;
constexpr int kBins = 64;          // iteration-count bins of the work-queue sort

// history locations (mm10_set_history_locs, one crystal)
constexpr int H_TAN = 0, H_GRADFE = 36, H_R = 63, H_WORK = 72, H_SLIP = 75;
constexpr int C0 = 87;
constexpr int C_STRESS = C0, C_EULER = C0 + 6, C_RP = C0 + 9, C_D = C0 + 18, C_EPS = C0 + 24,
              C_SLIP = C0 + 30, C_TT = C0 + 42, C_U = C0 + 43, C_TTRATE = C0 + 58, C_EP = C0 + 59,
              C_ED = C0 + 65;
static_assert(C_ED + 6 == kHistMM10, "history layout");

__device__ __forceinline__ double sgn1(double b) { return b >= 0.0 ? 1.0 : -1.0; }

// ---------------------------------------------------------------------
// kinematics (gtmat1, gtlsn1, qmply1, rstgp1_update_strains)
// ---------------------------------------------------------------------
struct KinSmem {
  double dn[kDnSize];
  double ce[8][3 * NN];
  double ue[8][TOT];
  double du[8][TOT];
};

__global__ void __launch_bounds__(kRecoverThreads) k_mm10_kin(RecoverArgs a, int chunk0) {
  __shared__ KinSmem S;
  const IterParams p = *a.params;
  const int tid = threadIdx.x;
  const int ge = tid >> 3, g = tid & 7;
  const Chunk ch = a.chunks[chunk0 + blockIdx.x];
  const BlockDesc bd = a.blocks[ch.blk];
  const bool active = ge < ch.n;
  const int i = ch.i0 + ge;
  const bool dirty = *a.geo_dirty != 0;
  for (int k = tid; k < kDnSize; k += kRecoverThreads) S.dn[k] = a.dn[0][k];
  if (active) {
    const long long dbase = bd.einf_off + (long long)i * TOT;
    for (int d = 0; d < 3; ++d) {
      const int j = d * NN + g;
      if (dirty) S.ce[ge][j] = a.c[a.cdest[dbase + j] - 1];
      const int eidx = a.edest[dbase + j] - 1;
      S.ue[ge][j] = a.u[eidx];
      S.du[ge][j] = a.du[eidx];
    }
  }
  __syncthreads();
  if (!active) return;
  const double* ue = S.ue[ge];
  const double* du = S.du[ge];
  const bool update_coords = bd.geonl && !(p.step == 1 && p.iter == 0);
  const long long gpi = bd.gp_off + (long long)i * NG + g;
  double tg0[3 * NN];
  double* geo = a.geo + bd.geo_off + ((long long)i * NG + g) * kGeo;
  if (dirty) {
    const double* dnx = S.dn + (g * 3 + 0) * NN;
    const double* dne = S.dn + (g * 3 + 1) * NN;
    const double* dnz = S.dn + (g * 3 + 2) * NN;
    double gama0[9], dj0;
    jacob1_ref<NN>(dnx, dne, dnz, S.ce[ge], S.ce[ge] + NN, S.ce[ge] + 2 * NN, gama0, dj0);
    for (int n = 0; n < NN; ++n) grad_ref(gama0, dnx[n], dne[n], dnz[n], tg0[3 * n], tg0[3 * n + 1], tg0[3 * n + 2]);
    for (int k = 0; k < 3 * NN; ++k) geo[k] = tg0[k];
    geo[3 * NN] = dj0;
  } else {
    for (int k = 0; k < 3 * NN; ++k) tg0[k] = geo[k];
  }
  // finite strain: gtmat1 in reference order; small displacement: no
  // deformation gradient, rotations = identity (drive_10_update,
  // rstgp1.f:4415-4432)
  double F1[9], Fh[9], R1[9], Rh[9];
  double dfn1 = 1.0, dfh = 1.0;
  if (bd.geonl) {
    double th1[9], thh[9];
    for (int k = 0; k < 9; ++k) { th1[k] = 0.0; thh[k] = 0.0; }
    for (int n = 0; n < NN; ++n) {
      const double tx = tg0[3 * n], ty = tg0[3 * n + 1], tz = tg0[3 * n + 2];
      const double u1x = ra(ue[n], du[n]), u1y = ra(ue[NN + n], du[NN + n]), u1z = ra(ue[2 * NN + n], du[2 * NN + n]);
      const double uhx = ra(ue[n], rm(0.5, du[n])), uhy = ra(ue[NN + n], rm(0.5, du[NN + n])),
                   uhz = ra(ue[2 * NN + n], rm(0.5, du[2 * NN + n]));
      tcomp1_node(th1, tx, ty, tz, u1x, u1y, u1z);
      tcomp1_node(thh, tx, ty, tz, uhx, uhy, uhz);
    }
    F1[0] = th1[0] + 1.0; F1[1] = th1[1]; F1[2] = th1[2]; F1[3] = th1[3]; F1[4] = th1[4] + 1.0;
    F1[5] = th1[5]; F1[6] = th1[6]; F1[7] = th1[7]; F1[8] = th1[8] + 1.0;
    Fh[0] = thh[0] + 1.0; Fh[1] = thh[1]; Fh[2] = thh[2]; Fh[3] = thh[3]; Fh[4] = thh[4] + 1.0;
    Fh[5] = thh[5]; Fh[6] = thh[6]; Fh[7] = thh[7]; Fh[8] = thh[8] + 1.0;
    dfn1 = det_ref(F1);
    dfh = det_ref(Fh);
    if (dfn1 <= 1.0e-20) atomicMin(a.status, bad_point_key(ch.blk, g, 0, i));
    else if (dfh <= 1.0e-20) atomicMin(a.status, bad_point_key(ch.blk, g, 1, i));
    polar_rotation_ref(F1, R1);
    polar_rotation_ref(Fh, Rh);
  } else {
    for (int k = 0; k < 9; ++k) F1[k] = Fh[k] = R1[k] = Rh[k] = (k % 4 == 0) ? 1.0 : 0.0;
  }
  double dth[9], L[9];
  for (int k = 0; k < 9; ++k) dth[k] = 0.0;
  for (int n = 0; n < NN; ++n) {
    const double dx = du[n], dy = du[NN + n], dz = du[2 * NN + n];
    for (int c = 0; c < 3; ++c) {
      const double t = tg0[3 * n + c];
      dth[3 * c + 0] += dx * t; dth[3 * c + 1] += dy * t; dth[3 * c + 2] += dz * t;
    }
  }
  if (update_coords) {
    const double r = 1.0 / dfh;
    double Fi[9];
    Fi[0] = (Fh[4] * Fh[8] - Fh[7] * Fh[5]) * r; Fi[3] = (Fh[6] * Fh[5] - Fh[3] * Fh[8]) * r;
    Fi[6] = (Fh[3] * Fh[7] - Fh[6] * Fh[4]) * r; Fi[1] = (Fh[7] * Fh[2] - Fh[1] * Fh[8]) * r;
    Fi[4] = (Fh[0] * Fh[8] - Fh[6] * Fh[2]) * r; Fi[7] = (Fh[6] * Fh[1] - Fh[0] * Fh[7]) * r;
    Fi[2] = (Fh[1] * Fh[5] - Fh[4] * Fh[2]) * r; Fi[5] = (Fh[3] * Fh[2] - Fh[0] * Fh[5]) * r;
    Fi[8] = (Fh[0] * Fh[4] - Fh[3] * Fh[1]) * r;
    for (int c = 0; c < 3; ++c)
      for (int rr = 0; rr < 3; ++rr)
        L[rr + 3 * c] = dth[rr] * Fi[3 * c] + dth[rr + 3] * Fi[1 + 3 * c] + dth[rr + 6] * Fi[2 + 3 * c];
  } else {
    for (int k = 0; k < 9; ++k) L[k] = dth[k];
  }
  double ddt[6] = {L[0], L[4], L[8], L[3] + L[1], L[7] + L[5], L[6] + L[2]};
  if (bd.bbar) {
    // b-bar at the mid-step shape (as for mm01): the element's mean
    // dilatation rate over its 8 Gauss-point lanes replaces each point's
    const unsigned gmask = 0xFFu << (tid & 24);
    const double jm = update_coords ? dfh * geo[3 * NN] : geo[3 * NN];
    const double trl = L[0] + L[4] + L[8];
    double s1 = jm * trl, s0 = jm;
    for (int off = 1; off < NG; off <<= 1) {
      s1 += __shfl_xor_sync(gmask, s1, off);
      s0 += __shfl_xor_sync(gmask, s0, off);
    }
    const double cb = a.bbar_beta * (s1 * (1.0 / s0) - trl);
    ddt[0] += cb; ddt[1] += cb; ddt[2] += cb;
  }
  double uddt[6];
  if (bd.geonl) rotate_to_unrotated(Rh, ddt, uddt);
  else for (int k = 0; k < 6; ++k) uddt[k] = ddt[k];   // rstgp2: the increment as it is
  for (int k = 0; k < 6; ++k) a.eps_n1[gpi * 6 + k] = a.eps_n[gpi * 6 + k] + uddt[k];
  if (p.iter > 0 && bd.geonl)
    for (int k = 0; k < 9; ++k) a.rot_n1[gpi * 9 + k] = R1[k];
  double* scr = a.mm10_scr + (long long)(bd.mm10_off + i * NG + g) * kMm10Scratch;
  for (int k = 0; k < 6; ++k) scr[k] = uddt[k];
  for (int k = 0; k < 9; ++k) scr[6 + k] = R1[k];
  for (int k = 0; k < 9; ++k) scr[15 + k] = F1[k];
  scr[24] = dfn1;
}

// ---------------------------------------------------------------------
// the local update of one Gauss point
// ---------------------------------------------------------------------
struct Nstate {   // crystal state n (mm10_copy_cc_hist)
  double R[9], Rp[9], D[6], stress[6], tt, tt_rate;
};

// lattice tensors of the current solve (mm10_setup): Schmid tensors and
// spins rotated by the plastic rotation at n and R(n+1); shared by the
// full-step state and the sub-step states (same R, same n)
struct Geo {
  double ms[NS][6];
  double qc[NS][3];
};

// strain increment and rates of a solve (np1 or a sub-step)
struct Rate {
  double D[6];
  double dg, tinc, tt_rate;
};

// x^y for y a non-negative integer up to 64 (the slip-rate exponents n,
// n - 1, n - 2 and the Voce exponent m of the usual data): binary
// powering, the same multiplications in the oracle and on the device, a
// few roundings instead of pow's log/exp sequence, which costs ~100 FP64
// instructions on GB300's narrow FP64 pipe; any other y: pow
__device__ __forceinline__ double powr(double x, double y) {
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
  return pow(x, y);
}

__device__ void symsw(const double* s, const double* w, double* sw) {
  sw[0] = s[3] * w[2] - s[5] * w[1];
  sw[1] = s[3] * w[2] - s[4] * w[0];
  sw[2] = s[5] * w[1] + s[4] * w[0];
  sw[3] = 0.5 * (w[2] * (s[0] - s[1]) + w[0] * s[5] - w[1] * s[4]);
  sw[4] = 0.5 * (w[0] * (s[1] - s[2]) + w[1] * s[3] + w[2] * s[5]);
  sw[5] = 0.5 * (w[1] * (s[0] - s[2]) + w[0] * s[3] - w[2] * s[4]);
}

// C (column-major 6x6) times c, summed column by column (mm10 mult_type_2)
__device__ __forceinline__ void cmul(const double* C, const double* c, double* a) {
  for (int r = 0; r < 6; ++r) a[r] = C[r] * c[0];
  for (int j = 1; j < 6; ++j)
    for (int r = 0; r < 6; ++r) a[r] = a[r] + C[r + 6 * j] * c[j];
}

// The products of the local solve's inner loops (resolved shears,
// plastic strain rate and spin, C times a vector, the Jacobian's outer
// products, the LU updates) are fused multiply-adds in a fixed order, the
// same in the oracle (on FMA hardware the reference's compiler contracts
// them as well); they are most of the FP64 instructions of a local
// iteration on GB300's narrow FP64 pipe. The translation unit is compiled
// with -fmad=false, so nothing else is contracted.
__device__ __forceinline__ double rs_dot(const double* s, const double* m) {
  double r = s[0] * m[0];
  for (int k = 1; k < 6; ++k) r = fma(s[k], m[k], r);
  return r;
}

// C (column-major 6x6) times c, column by column, fused
__device__ __forceinline__ void cmul_f(const double* C, const double* c, double* a) {
  for (int r = 0; r < 6; ++r) a[r] = C[r] * c[0];
  for (int j = 1; j < 6; ++j)
    for (int r = 0; r < 6; ++r) a[r] = fma(C[r + 6 * j], c[j], a[r]);
}

// resolved shears and slip increments of all systems (mm10_rs,
// mm10_slipinc): computed once per evaluation point and reused by every
// term that the reference evaluates at that point
__device__ __forceinline__ void slip_terms(const CrystalType& t, const Geo& G, const Rate& q, const double* s,
                                           double tt, double* rs, double* sl) {
  for (int i = 0; i < NS; ++i) {
    rs[i] = rs_dot(s, G.ms[i]);
    sl[i] = q.dg / tt * powr(fabs(rs[i] / tt), t.rate_n - 1.0) * rs[i];
  }
}

// spin w_p in the current configuration (mm10_form_wp)
__device__ __forceinline__ void form_wp(const CrystalType& t, const Geo& G, const Rate& q, const double* rs,
                                        const double* sl, double* w) {
  w[0] = 0.0; w[1] = 0.0; w[2] = 0.0;
  for (int i = 0; i < NS; ++i) {
    for (int k = 0; k < 3; ++k) w[k] = fma(sl[i], G.qc[i][k], w[k]);
    for (int k = 0; k < 3; ++k) w[k] = fma(rs[i] * q.tinc * t.iD_v, G.qc[i][k], w[k]);
  }
}

// R1 (mm10_formR1 with mm10_form_dbarp / mm10_form_wp) from slip terms
__device__ void formR1(const CrystalElem& x, const CrystalType& t, const Geo& G, const Rate& q, const Nstate& n,
                       const double* s, const double* rs, const double* sl, double* R1) {
  double dbarp[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, wp[3], symTW[6], wv1[6], wv2[6];
  for (int i = 0; i < NS; ++i) {
    const double f = rs[i] * q.tinc * t.iD_v + sl[i];
    for (int k = 0; k < 6; ++k) dbarp[k] = fma(f, G.ms[i][k], dbarp[k]);
  }
  form_wp(t, G, q, rs, sl, wp);
  symsw(s, wp, symTW);
  for (int k = 0; k < 6; ++k) wv1[k] = q.D[k] - dbarp[k];
  cmul_f(x.C, wv1, wv2);
  for (int k = 0; k < 6; ++k) R1[k] = s[k] - n.stress[k] - wv2[k] + 2.0 * symTW[k];
}

// R2 (mm10_formR2 with mm10_h_voche); sets q.tt_rate. The hardening term
// h_term = 1 - (tt - tau_y)/tau_v + tau_l/(tt - tau_y) is the same for all
// systems (tau_l = 0: no lattice-curvature data in this scope)
__device__ double formR2(const CrystalType& t, Rate& q, const Nstate& n, const double* sl, double tt) {
  const double h_term = 1.0 - (tt - t.tau_y) / t.tau_v + 0.0 / (tt - t.tau_y);
  const double ph = powr(fabs(h_term), t.voche_m) * sgn1(h_term);
  double h = 0.0;
  for (int i = 0; i < NS; ++i) h = fma(ph, fabs(sl[i]), h);
  h = n.tt + t.theta_0 * h;
  q.tt_rate = (h - n.tt) / q.tinc;
  return tt - h;
}

// residual of the predictor (R1 only) and of the coupled update (R1, R2)
__device__ __noinline__ void eval_R1(const CrystalElem& x, const CrystalType& t, const Geo& G, const Rate& q,
                                        const Nstate& n, const double* s, double tt, double* R1) {
  double rs[NS], sl[NS];
  slip_terms(t, G, q, s, tt, rs, sl);
  formR1(x, t, G, q, n, s, rs, sl, R1);
}
__device__ __noinline__ void eval_R(const CrystalElem& x, const CrystalType& t, const Geo& G, Rate& q,
                                       const Nstate& n, const double* xv, double* R) {
  double rs[NS], sl[NS];
  slip_terms(t, G, q, xv, xv[6], rs, sl);
  formR1(x, t, G, q, n, xv, rs, sl, R);
  R[6] = formR2(t, q, n, sl, xv[6]);
}

// J11 (mm10_formJ11 with mm10_dgdt_voche and mm10_iw), optionally with
// J12, J21, J22 of mm10_formJ into the 7x7 J (the reference's J22 keeps
// its sign(one, slipinc) factor in the rate term); ld = 6 or 7
template <bool kFull>
__device__ __noinline__ void formJ(const CrystalElem& x, const CrystalType& t, const Geo& G, const Rate& q, const double* s,
                      double tt, double* J) {
  constexpr int ld = kFull ? 7 : 6;
  double rs[NS], sl[NS];
  slip_terms(t, G, q, s, tt, rs, sl);
  for (int c = 0; c < 6; ++c)
    for (int r = 0; r < 6; ++r) J[r + ld * c] = 0.0;
  const double A = q.dg * t.rate_n / powr(tt, t.rate_n);
  const double B = -t.rate_n / tt;
  double J12[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int i = 0; i < NS; ++i) {
    double sw[6], wv[6];
    symsw(s, G.qc[i], sw);
    double d = powr(fabs(rs[i]), t.rate_n - 1.0);
    d = A * d;
    d = d + q.tinc * t.iD_v;
    for (int r = 0; r < 6; ++r) wv[r] = 2.0 * sw[r];
    for (int j = 0; j < 6; ++j)
      for (int r = 0; r < 6; ++r) wv[r] = fma(x.C[r + 6 * j], G.ms[i][j], wv[r]);
    for (int c = 0; c < 6; ++c) {
      const double temp = d * G.ms[i][c];
      if (temp != 0.0)
        for (int r = 0; r < 6; ++r) J[r + ld * c] = fma(wv[r], temp, J[r + ld * c]);
    }
    if (kFull) {
      const double temp = 1.0 * (B * sl[i]);
      if (temp != 0.0)
        for (int r = 0; r < 6; ++r) J12[r] = fma(wv[r], temp, J12[r]);
    }
  }
  double w[3];
  form_wp(t, G, q, rs, sl, w);
  J[0 + ld * 3] = J[0 + ld * 3] + 2.0 * w[2];
  J[0 + ld * 5] = J[0 + ld * 5] + (-2.0 * w[1]);
  J[1 + ld * 3] = J[1 + ld * 3] + 2.0 * w[2];
  J[1 + ld * 4] = J[1 + ld * 4] + (-2.0 * w[0]);
  J[2 + ld * 4] = J[2 + ld * 4] + 2.0 * w[0];
  J[2 + ld * 5] = J[2 + ld * 5] + 2.0 * w[1];
  J[3 + ld * 0] = J[3 + ld * 0] + w[2];
  J[3 + ld * 1] = J[3 + ld * 1] + (-w[2]);
  J[3 + ld * 4] = J[3 + ld * 4] + (-w[1]);
  J[3 + ld * 5] = J[3 + ld * 5] + w[0];
  J[4 + ld * 1] = J[4 + ld * 1] + w[0];
  J[4 + ld * 2] = J[4 + ld * 2] + (-w[0]);
  J[4 + ld * 3] = J[4 + ld * 3] + w[1];
  J[4 + ld * 5] = J[4 + ld * 5] + w[2];
  J[5 + ld * 0] = J[5 + ld * 0] + w[1];
  J[5 + ld * 2] = J[5 + ld * 2] + (-w[1]);
  J[5 + ld * 3] = J[5 + ld * 3] + w[0];
  J[5 + ld * 4] = J[5 + ld * 4] + (-w[2]);
  for (int k = 0; k < 6; ++k) J[k + ld * k] = J[k + ld * k] + 1.0;
  if (!kFull) return;
  for (int r = 0; r < 6; ++r) J[r + 7 * 6] = J12[r];
  const double h_term = 1.0 - (tt - t.tau_y) / t.tau_v + 0.0 / (tt - t.tau_y);
  const double phm = powr(fabs(h_term), t.voche_m);
  const double ph = phm * sgn1(h_term);
  double et[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int i = 0; i < NS; ++i) {
    const double f = ph * powr(fabs(rs[i]), t.rate_n - 2.0) * rs[i];
    for (int k = 0; k < 6; ++k) et[k] = fma(f, G.ms[i][k], et[k]);
  }
  const double fe = t.theta_0 * q.dg * t.rate_n / powr(tt, t.rate_n);
  for (int c = 0; c < 6; ++c) J[6 + 7 * c] = -(fe * et[c]);
  const double dd = tt - t.tau_y;
  const double dh = t.voche_m * (-1.0 / t.tau_v - 0.0 / (dd * dd));
  double etau = 0.0;
  for (int i = 0; i < NS; ++i)
    etau = etau + (dh * fabs(sl[i]) / fabs(h_term) - fabs(sl[i]) * t.rate_n / tt * sgn1(h_term) * sgn1(sl[i])) * phm;
  etau = t.theta_0 * etau;
  J[6 + 7 * 6] = 1.0 - etau;
}

// partial-pivot LU solve (the oracle's DGESV restatement), n <= 7
__device__ __noinline__ void lu_solve(int n, double* a, double* b, int nrhs) {
  int ipiv[7];
  for (int j = 0; j < n; ++j) {
    int jp = j;
    double amax = fabs(a[j + n * j]);
    for (int i = j + 1; i < n; ++i)
      if (fabs(a[i + n * j]) > amax) { amax = fabs(a[i + n * j]); jp = i; }
    ipiv[j] = jp;
    if (a[jp + n * j] != 0.0) {
      if (jp != j)
        for (int k = 0; k < n; ++k) { const double tt = a[j + n * k]; a[j + n * k] = a[jp + n * k]; a[jp + n * k] = tt; }
      if (j < n - 1) {
        const double r = 1.0 / a[j + n * j];
        for (int i = j + 1; i < n; ++i) a[i + n * j] = r * a[i + n * j];
      }
    }
    for (int k = j + 1; k < n; ++k) {
      const double temp = -a[j + n * k];
      if (temp != 0.0)
        for (int i = j + 1; i < n; ++i) a[i + n * k] = fma(a[i + n * j], temp, a[i + n * k]);
    }
  }
  for (int c = 0; c < nrhs; ++c) {
    double* x = b + n * c;
    for (int i = 0; i < n; ++i)
      if (ipiv[i] != i) { const double tt = x[i]; x[i] = x[ipiv[i]]; x[ipiv[i]] = tt; }
    for (int k = 0; k < n; ++k)
      if (x[k] != 0.0)
        for (int i = k + 1; i < n; ++i) x[i] = fma(-x[k], a[i + n * k], x[i]);
    for (int k = n - 1; k >= 0; --k)
      if (x[k] != 0.0) {
        x[k] = x[k] / a[k + n * k];
        for (int i = 0; i < k; ++i) x[i] = fma(-x[k], a[i + n * k], x[i]);
      }
  }
}

__device__ void rt2rve(const double* rt, double* rv) {   // mm10_rt2rve, column-major in and out
#define RT(a, b) rt[(a - 1) + 3 * (b - 1)]
#define RV(a, b) rv[(a - 1) + 6 * (b - 1)]
  RV(1, 1) = RT(1, 1) * RT(1, 1); RV(1, 2) = RT(1, 2) * RT(1, 2); RV(1, 3) = RT(1, 3) * RT(1, 3);
  RV(1, 4) = 2.0 * RT(1, 1) * RT(1, 2); RV(1, 5) = 2.0 * RT(1, 3) * RT(1, 2); RV(1, 6) = 2.0 * RT(1, 1) * RT(1, 3);
  RV(2, 1) = RT(2, 1) * RT(2, 1); RV(2, 2) = RT(2, 2) * RT(2, 2); RV(2, 3) = RT(2, 3) * RT(2, 3);
  RV(2, 4) = 2.0 * RT(2, 1) * RT(2, 2); RV(2, 5) = 2.0 * RT(2, 3) * RT(2, 2); RV(2, 6) = 2.0 * RT(2, 1) * RT(2, 3);
  RV(3, 1) = RT(3, 1) * RT(3, 1); RV(3, 2) = RT(3, 2) * RT(3, 2); RV(3, 3) = RT(3, 3) * RT(3, 3);
  RV(3, 4) = 2.0 * RT(3, 1) * RT(3, 2); RV(3, 5) = 2.0 * RT(3, 3) * RT(3, 2); RV(3, 6) = 2.0 * RT(3, 1) * RT(3, 3);
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

__device__ void rt2rvw(const double* rt, double* rv) {   // mm10_rt2rvw
#define RW(a, b) rv[(a - 1) + 3 * (b - 1)]
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

__device__ __forceinline__ void m3mul(const double* b, const double* c, double* a) {   // [a] = [b][c]
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) a[i + 3 * j] = b[i] * c[3 * j] + b[i + 3] * c[1 + 3 * j] + b[i + 6] * c[2 + 3 * j];
}
__device__ __forceinline__ void m3vec(const double* b, const double* c, double* a) {   // a = [b] c
  for (int r = 0; r < 3; ++r) a[r] = b[r] * c[0] + b[r + 3] * c[1] + b[r + 6] * c[2];
}

// mm10_setup: lattice tensors for R(n+1) and the plastic rotation at n
__device__ void setup_geo(const CrystalElem& x, const Nstate& n, const double* R, Geo& G) {
  double tr[9], RE[36], RWC[9], work[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) tr[i + 3 * j] = n.Rp[j + 3 * i];
  rt2rve(tr, RE);
  m3mul(R, tr, work);
  rt2rvw(work, RWC);
  for (int i = 0; i < NS; ++i) {
    cmul(RE, x.ms[i], G.ms[i]);
    m3vec(RWC, x.qs[i], G.qc[i]);
  }
}

// mm10_setup_np1 + the effective strain increment of mm10_setup
__device__ __forceinline__ void setup_rate(const double* D, double tinc, Rate& q) {
  for (int k = 0; k < 6; ++k) q.D[k] = D[k];
  q.tinc = tinc;
  q.tt_rate = 0.0;
  const double t1 = q.D[0] * q.D[0] + q.D[1] * q.D[1] + q.D[2] * q.D[2];
  const double t2 = q.D[3] * q.D[3] + q.D[4] * q.D[4] + q.D[5] * q.D[5];
  q.dg = sqrt((2.0 / 3.0) * (t1 + 0.5 * t2));
}

// mm10_solve: predictor (stress with extrapolated hardening) then the
// coupled Newton with line search; J gets the last Jacobian. Returns
// false on failure; *iters accumulates the Newton iterations.
__device__ __noinline__ bool solve(const CrystalElem& x, const CrystalType& t, const Geo& G, Rate& q, const Nstate& n,
                      double* stress, double& tt, double dtinc, double* J, int* iters) {
  const double c = 1.0e-4, red = 0.5;
  const int mls = 10, mmin = 1;
  double xv[7];
  for (int k = 0; k < 6; ++k) xv[k] = stress[k];
  xv[6] = tt;
  double inR1;
  {
    int iter = 0;
    double x1[6], d1[6], d2[6], R1[6];
    for (int k = 0; k < 6; ++k) x1[k] = xv[k];
    for (int k = 0; k < 6; ++k) d1[k] = q.D[k];
    double dtrace = (d1[0] + d1[1] + d1[2]) / 3.0;
    d1[0] = d1[0] - dtrace; d1[1] = d1[1] - dtrace; d1[2] = d1[2] - dtrace;
    double t1 = d1[0] * d1[0] + d1[1] * d1[1] + d1[2] * d1[2];
    double t2 = d1[3] * d1[3] + d1[4] * d1[4] + d1[5] * d1[5];
    if (t1 + t2 == 0.0) for (int k = 0; k < 6; ++k) d1[k] = 0.0;
    else { const double sq = sqrt(t1 + t2); for (int k = 0; k < 6; ++k) d1[k] = d1[k] / sq; }
    for (int k = 0; k < 6; ++k) d2[k] = n.D[k];
    dtrace = (d2[0] + d2[1] + d2[2]) / 3.0;
    d2[0] = d2[0] - dtrace; d2[1] = d2[1] - dtrace; d2[2] = d2[2] - dtrace;
    t1 = d2[0] * d2[0] + d2[1] * d2[1] + d2[2] * d2[2];
    t2 = d2[3] * d2[3] + d2[4] * d2[4] + d2[5] * d2[5];
    if (t1 + t2 == 0.0) for (int k = 0; k < 6; ++k) d2[k] = 0.0;
    else { const double sq = sqrt(t1 + t2); for (int k = 0; k < 6; ++k) d2[k] = d2[k] / sq; }
    t1 = d1[0] * d2[0] + d1[1] * d2[1] + d1[2] * d2[2];
    t2 = d1[3] * d2[3] + d1[4] * d2[4] + d1[5] * d2[5];
    const double cos_ang = fmax(t1 + t2, 0.0);
    const double x2 = xv[6] + cos_ang * n.tt_rate * dtinc;
    eval_R1(x, t, G, q, n, x1, x2, R1);
    double nR1 = sqrt(R1[0] * R1[0] + R1[1] * R1[1] + R1[2] * R1[2] + R1[3] * R1[3] + R1[4] * R1[4] + R1[5] * R1[5]);
    inR1 = nR1;
    while (nR1 > t.atol1 && nR1 / inR1 > t.rtol1) {
      double J11[36], mJ[36], dx1[6], wv[6], xn[6];
      formJ<false>(x, t, G, q, x1, x2, J11);
      for (int k = 0; k < 6; ++k) dx1[k] = R1[k];
      for (int k = 0; k < 36; ++k) mJ[k] = -J11[k];
      lu_solve(6, mJ, dx1, 1);
      double alpha = 1.0;
      double dotR1 = R1[0] * R1[0] + R1[1] * R1[1] + R1[2] * R1[2] + R1[3] * R1[3] + R1[4] * R1[4] + R1[5] * R1[5];
      const double ls1 = 0.5 * dotR1;
      for (int j = 0; j < 6; ++j)
        wv[j] = J11[0 + 6 * j] * R1[0] + J11[1 + 6 * j] * R1[1] + J11[2 + 6 * j] * R1[2] + J11[3 + 6 * j] * R1[3] +
                J11[4 + 6 * j] * R1[4] + J11[5 + 6 * j] * R1[5];
      const double ls2 = c * (dx1[0] * wv[0] + dx1[1] * wv[1] + dx1[2] * wv[2] + dx1[3] * wv[3] + dx1[4] * wv[4] +
                              dx1[5] * wv[5]);
      int ls = 0;
      for (;;) {
        const double nlsx = ls1 + ls2 * alpha;
        for (int k = 0; k < 6; ++k) xn[k] = x1[k] + alpha * dx1[k];
        eval_R1(x, t, G, q, n, xn, x2, R1);
        dotR1 = R1[0] * R1[0] + R1[1] * R1[1] + R1[2] * R1[2] + R1[3] * R1[3] + R1[4] * R1[4] + R1[5] * R1[5];
        nR1 = sqrt(dotR1);
        const double nRs = 0.5 * dotR1;
        if (nRs <= nlsx || ls > mls) {
          for (int k = 0; k < 6; ++k) x1[k] = xn[k];
          break;
        }
        alpha = red * alpha;
        ++ls;
      }
      ++iter;
      ++*iters;
      bool nan = false;
      for (int k = 0; k < 6; ++k) nan = nan || isnan(x1[k]);
      if (iter > t.miter || nan) return false;
    }
    for (int k = 0; k < 6; ++k) xv[k] = x1[k];
    xv[6] = x2;
  }
  {
    int iter = 0;
    double R[7], dx[7], mJ[49], xn[7], wv[7];
    eval_R(x, t, G, q, n, xv, R);
    double dotR = 0.0;
    for (int k = 0; k < 7; ++k) dotR = dotR + R[k] * R[k];
    double nR = sqrt(dotR);
    double inR = nR;
    if (inR == 0.0) inR = inR1;
    while ((nR > t.atol && nR / inR > t.rtol) || iter < mmin) {
      formJ<true>(x, t, G, q, xv, xv[6], J);
      for (int k = 0; k < 7; ++k) dx[k] = R[k];
      for (int k = 0; k < 49; ++k) mJ[k] = -J[k];
      lu_solve(7, mJ, dx, 1);
      double alpha = 1.0;
      dotR = 0.0;
      for (int k = 0; k < 7; ++k) dotR = dotR + R[k] * R[k];
      const double ls1 = 0.5 * dotR;
      for (int i = 0; i < 7; ++i) {
        double temp = 0.0;
        for (int l = 0; l < 7; ++l) temp = temp + J[l + 7 * i] * R[l];
        wv[i] = 1.0 * temp;
      }
      double dxw = 0.0;
      for (int k = 0; k < 7; ++k) dxw = dxw + dx[k] * wv[k];
      const double ls2 = c * dxw;
      int ls = 0;
      for (;;) {
        const double nlsx = ls1 + ls2 * alpha;
        for (int k = 0; k < 7; ++k) xn[k] = xv[k] + alpha * dx[k];
        eval_R(x, t, G, q, n, xn, R);
        dotR = 0.0;
        for (int k = 0; k < 7; ++k) dotR = dotR + R[k] * R[k];
        nR = sqrt(dotR);
        const double nRs = 0.5 * dotR;
        if (nRs <= nlsx || ls > mls) {
          for (int k = 0; k < 7; ++k) xv[k] = xn[k];
          break;
        }
        alpha = red * alpha;
        ++ls;
      }
      ++iter;
      ++*iters;
      bool nan = false;
      for (int k = 0; k < 7; ++k) nan = nan || isnan(xv[k]);
      if (iter > t.miter || nan) return false;
    }
  }
  for (int k = 0; k < 6; ++k) stress[k] = xv[k];
  tt = xv[6];
  return true;
}

__device__ __forceinline__ double atan2_2pi(double a, double b) {
  double r = atan2(a, b);
  if (r < 0.0) r = r + 2.0 * 3.141592653589793;
  return r;
}

// one Gauss point: mm10 for the one crystal (mm10_a_do_crystal ->
// mm10_solve_crystal) and mm10_a_store_crystal. Returns false if the
// local solve failed after all step cuts.
__device__ bool mm10_gp(const RecoverArgs& a, const IterParams& p, int gp_index, int* iters_out) {
  const int code = a.mm10_gp[gp_index];
  const int blk = code >> 12, i = (code >> 3) & 511, g = code & 7;
  const BlockDesc bd = a.blocks[blk];
  const int e = bd.felem + i;
  const CrystalElem& x = a.xtal[e];
  const CrystalType t = a.xtype[x.type];
  const long long gpi = bd.gp_off + (long long)i * NG + g;
  const double* hn = a.hist + bd.hist_off + ((long long)i * NG + g) * kHistMM10;
  double* hn1 = a.hist1 + bd.hist_off + ((long long)i * NG + g) * kHistMM10;
  const double* scr = a.mm10_scr + (long long)(bd.mm10_off + i * NG + g) * kMm10Scratch;
  const double* urcs_n = a.urcs_n + gpi * 9;
  double* urcs_n1 = a.urcs_n1 + gpi * 9;
  const double* uddt = scr;
  const double* R1 = scr + 6;

  bool iter0off = false;
  if (p.iter == 0) {
    iter0off = !p.nonlinear;   // nonlinear = extrapolated_du at iteration 0
    if (p.step == 1) iter0off = true;
  }
  // state n (mm10_copy_cc_hist), with the step-1 initialisation
  // (mm10_init_general_hist, mm10_init_cc_hist0, mm10_init_voche)
  Nstate n;
  double slip_tot[NS], work3[3];
  if (p.step == 1) {
    for (int k = 0; k < 9; ++k) n.R[k] = (k % 4 == 0) ? 1.0 : 0.0;
    for (int k = 0; k < 6; ++k) n.stress[k] = urcs_n[k];
    for (int k = 0; k < 9; ++k) n.Rp[k] = (k % 4 == 0) ? 1.0 : 0.0;
    for (int k = 0; k < 6; ++k) n.D[k] = 0.0;
    n.tt = t.tau_y + 1.0e-5;
    n.tt_rate = hn[C_TTRATE];
    for (int k = 0; k < NS; ++k) slip_tot[k] = 0.0;
    for (int k = 0; k < 3; ++k) work3[k] = 0.0;
  } else {
    for (int k = 0; k < 9; ++k) n.R[k] = hn[H_R + k];
    for (int k = 0; k < 6; ++k) n.stress[k] = hn[C_STRESS + k];
    for (int k = 0; k < 9; ++k) n.Rp[k] = hn[C_RP + k];
    for (int k = 0; k < 6; ++k) n.D[k] = hn[C_D + k];
    n.tt = hn[C_TT];
    n.tt_rate = hn[C_TTRATE];
    for (int k = 0; k < NS; ++k) slip_tot[k] = hn[H_SLIP + k];
    for (int k = 0; k < 3; ++k) work3[k] = hn[H_WORK + k];
  }
  const double dt = a.dt;
  // mm10_solve_strup
  Geo G;
  setup_geo(x, n, R1, G);
  Rate q;
  setup_rate(uddt, dt, q);
  double stress[6], ostress[6], tt = n.tt, ott = n.tt;
  for (int k = 0; k < 6; ++k) { stress[k] = n.stress[k]; ostress[k] = stress[k]; }
  const double temp1 = q.D[0] * q.D[0] + q.D[1] * q.D[1] + q.D[2] * q.D[2] + q.D[3] * q.D[3] + q.D[4] * q.D[4] +
                       q.D[5] * q.D[5];
  const double temp2 = stress[0] * stress[0] + stress[1] * stress[1] + stress[2] * stress[2] +
                       stress[3] * stress[3] + stress[4] * stress[4] + stress[5] * stress[5];
  const bool no_load = (temp2 == 0.0) && (temp1 == 0.0);
  double J[49];
  for (int k = 0; k < 49; ++k) J[k] = 0.0;
  double tt_rate = 0.0;
  int iters = 0;
  if (iter0off || no_load) {
    if (!no_load) {
      double R1v[6];
      eval_R1(x, t, G, q, n, stress, tt, R1v);
      for (int k = 0; k < 6; ++k) stress[k] = stress[k] - R1v[k];
    }
  } else {
    double frac = 0.0, step = 1.0;
    int cuts = 0;
    bool fail = false;
    Rate cq;
    while (frac < 1.0) {
      double Dw[6];
      for (int k = 0; k < 6; ++k) Dw[k] = uddt[k] * (step + frac);
      setup_rate(Dw, dt * (step + frac), cq);
      tt = n.tt;
      fail = !solve(x, t, G, cq, n, stress, tt, dt * step, J, &iters);
      if (fail) {
        for (int k = 0; k < 6; ++k) stress[k] = ostress[k];
        tt = ott;
        step = step * 0.5;
        ++cuts;
        if (cuts > 4) break;
        fail = false;
      } else {
        for (int k = 0; k < 6; ++k) ostress[k] = stress[k];
        ott = tt;
        frac = frac + step;
      }
    }
    bool bad = fail || isnan(tt);
    for (int k = 0; k < 6; ++k) bad = bad || isnan(stress[k]);
    *iters_out = iters;
    if (bad) return false;
    tt_rate = cq.tt_rate;
  }
  *iters_out = iters;
  // np1 results (mm10_store_cryhist layout); zeros where the reference's
  // np1 keeps mm10_setup_np1's values
  double tangent[36], Rp1[9], euler[3] = {0.0, 0.0, 0.0}, eps[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  double slip_incs[NS], u[15], ep6[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, ed6[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  double work_inc = 0.0, p_work_inc = 0.0, p_strain_inc = 0.0;
  for (int k = 0; k < NS; ++k) slip_incs[k] = 0.0;
  for (int k = 0; k < 15; ++k) u[k] = 0.0;
  for (int k = 0; k < 9; ++k) Rp1[k] = 0.0;
  if (iter0off || no_load) {
    for (int k = 0; k < 36; ++k) tangent[k] = x.C[k];
  } else {
    // mm10_tangent: ed = 0, dgammadd = 0 (Voce) -> JR = C
    double JJ[36], beta[12];
    for (int cc = 0; cc < 6; ++cc)
      for (int r = 0; r < 6; ++r) JJ[r + 6 * cc] = J[r + 7 * cc];
    for (int cc = 0; cc < 6; ++cc) beta[cc] = J[6 + 7 * cc] / J[6 + 7 * 6];
    for (int j = 0; j < 6; ++j) {
      const double temp = -1.0 * beta[j];
      if (temp != 0.0)
        for (int r = 0; r < 6; ++r) JJ[r + 6 * j] = JJ[r + 6 * j] + temp * J[r + 7 * 6];
    }
    for (int k = 0; k < 36; ++k) tangent[k] = x.C[k];
    lu_solve(6, JJ, tangent, 6);
    if (!a.asym) {   // mm10_a_make_symm_1 unless asymmetric assembly (mm10_a.f:1165-1166)
      double w[36];
      for (int j = 0; j < 6; ++j)
        for (int r = 0; r < 6; ++r) w[r + 6 * j] = (tangent[r + 6 * j] + tangent[j + 6 * r]) * 0.5;
      for (int k = 0; k < 36; ++k) tangent[k] = w[k];
    }
    // np1 is the full-step solve state (mm10_setup on the whole increment)
    // mm10_update_rotation: wbarp with the lattice spins np1%qs
    double tr[9], RW[9];
    for (int ii = 0; ii < 3; ++ii)
      for (int jj = 0; jj < 3; ++jj) tr[ii + 3 * jj] = n.Rp[jj + 3 * ii];
    rt2rvw(tr, RW);
    double rsc[NS], slc[NS];   // slip terms at the converged state
    slip_terms(t, G, q, stress, tt, rsc, slc);
    double wb[3] = {0.0, 0.0, 0.0};
    for (int s = 0; s < NS; ++s) {
      double qs[3];
      m3vec(RW, x.qs[s], qs);
      for (int k = 0; k < 3; ++k) wb[k] = wb[k] + slc[s] * qs[k];
      for (int k = 0; k < 3; ++k) wb[k] = wb[k] + rsc[s] * q.tinc * t.iD_v * qs[k];
    }
    double wt[9], ex[9];
    wt[0] = 0.0; wt[3] = wb[2]; wt[6] = wb[1];
    wt[1] = -wb[2]; wt[4] = 0.0; wt[7] = wb[0];
    wt[2] = -wb[1]; wt[5] = -wb[0]; wt[8] = 0.0;
    const double al = sqrt(wt[7] * wt[7] + wt[6] * wt[6] + wt[3] * wt[3]);
    if (al < 1.0e-16) {
      for (int k = 0; k < 9; ++k) ex[k] = 0.0;
    } else {
      const double ca = (1.0 - cos(al)) / (al * al);
      const double cb = sin(al) / al;
      for (int j = 0; j < 3; ++j) {
        for (int ii = 0; ii < 3; ++ii) ex[ii + 3 * j] = cb * wt[ii + 3 * j];
        for (int l = 0; l < 3; ++l) {
          const double temp = ca * wt[l + 3 * j];
          if (temp != 0.0)
            for (int ii = 0; ii < 3; ++ii) ex[ii + 3 * j] = ex[ii + 3 * j] + temp * wt[ii + 3 * l];
        }
      }
    }
    ex[0] = ex[0] + 1.0; ex[4] = ex[4] + 1.0; ex[8] = ex[8] + 1.0;
    m3mul(ex, n.Rp, Rp1);
    // mm10_output
    for (int s = 0; s < NS; ++s) slip_incs[s] = slc[s];
    {
      double w1[9], fr[9];
      for (int ii = 0; ii < 3; ++ii)
        for (int jj = 0; jj < 3; ++jj)
          w1[ii + 3 * jj] = Rp1[ii] * R1[jj] + Rp1[ii + 3] * R1[jj + 3] + Rp1[ii + 6] * R1[jj + 6];
      m3mul(x.g, w1, fr);
      const double psiK = atan2_2pi(fr[2 + 3 * 1], fr[2 + 3 * 0]);
      const double phiK = atan2_2pi(fr[1 + 3 * 2], fr[0 + 3 * 2]);
      if (fr[8] > 1.0) fr[8] = 1.0;
      const double thetaK = acos(fr[8]);
      const double c180 = 180.0 / 3.141592653589793;
      euler[0] = c180 * psiK;
      euler[1] = c180 * thetaK;
      euler[2] = c180 * phiK;
    }
    double dif[NS], ed[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, t1, t2;
    for (int s = 0; s < NS; ++s) dif[s] = rsc[s] * q.tinc * t.iD_v;
    for (int s = 0; s < NS; ++s)
      for (int k = 0; k < 6; ++k) ed[k] = ed[k] + dif[s] * G.ms[s][k];
    for (int k = 0; k < 6; ++k) ed6[k] = ed[k] / q.tinc;
    t1 = ed[0] * ed[0] + ed[1] * ed[1] + ed[2] * ed[2];
    t2 = ed[3] * ed[3] + ed[4] * ed[4] + ed[5] * ed[5];
    double ed_dot = sqrt(2.0 / 3.0 * (t1 + 0.5 * t2));
    ed_dot = ed_dot / q.tinc;
    u[14] = ed_dot;
    work_inc = stress[0] * q.D[0] + stress[1] * q.D[1] + stress[2] * q.D[2] + stress[3] * q.D[3] +
               stress[4] * q.D[4] + stress[5] * q.D[5];
    // elastic strain: Cholesky solve C ee = stress (DPOSV 'U')
    double Sm[36], eu[6], erot[36], ee[6];
    for (int k = 0; k < 36; ++k) Sm[k] = x.C[k];
    for (int k = 0; k < 6; ++k) eu[k] = stress[k];
    {
      bool ok = true;
      for (int j = 0; j < 6 && ok; ++j) {
        double dot = 0.0;
        for (int k = 0; k < j; ++k) dot = dot + Sm[k + 6 * j] * Sm[k + 6 * j];
        double ajj = Sm[j + 6 * j] - dot;
        if (ajj <= 0.0) { ok = false; break; }
        ajj = sqrt(ajj);
        Sm[j + 6 * j] = ajj;
        for (int jj = j + 1; jj < 6; ++jj) {
          double temp = 0.0;
          for (int k = 0; k < j; ++k) temp = temp + Sm[k + 6 * jj] * Sm[k + 6 * j];
          Sm[j + 6 * jj] = Sm[j + 6 * jj] + (-1.0) * temp;
        }
        const double r = 1.0 / ajj;
        for (int jj = j + 1; jj < 6; ++jj) Sm[j + 6 * jj] = r * Sm[j + 6 * jj];
      }
      if (ok) {
        for (int ii = 0; ii < 6; ++ii) {
          double temp = eu[ii];
          for (int k = 0; k < ii; ++k) temp = temp - Sm[k + 6 * ii] * eu[k];
          eu[ii] = temp / Sm[ii + 6 * ii];
        }
        for (int k = 5; k >= 0; --k)
          if (eu[k] != 0.0) {
            eu[k] = eu[k] / Sm[k + 6 * k];
            for (int ii = 0; ii < k; ++ii) eu[ii] = eu[ii] - eu[k] * Sm[ii + 6 * k];
          }
      }
    }
    rt2rve(R1, erot);
    cmul(erot, eu, ee);
    double dbarp[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, wp[3], ewwe[6], ep[6];
    for (int s = 0; s < NS; ++s)
      for (int k = 0; k < 6; ++k) dbarp[k] = dbarp[k] + slip_incs[s] * G.ms[s][k];
    form_wp(t, G, q, rsc, slc, wp);
    symsw(ee, wp, ewwe);
    for (int k = 0; k < 6; ++k) ep[k] = dbarp[k] + ewwe[k];
    for (int k = 0; k < 6; ++k) ep6[k] = ep[k] / q.tinc;
    t1 = ep[0] * ep[0] + ep[1] * ep[1] + ep[2] * ep[2];
    t2 = ep[3] * ep[3] + ep[4] * ep[4] + ep[5] * ep[5];
    double ep_dot = sqrt(2.0 / 3.0 * (t1 + 0.5 * t2));
    ep_dot = ep_dot / q.tinc;
    u[10] = ep_dot;
    for (int k = 0; k < 6; ++k) ep[k] = ep[k] + ed[k];
    t1 = ep[0] * ep[0] + ep[1] * ep[1] + ep[2] * ep[2];
    t2 = ep[3] * ep[3] + ep[4] * ep[4] + ep[5] * ep[5];
    p_strain_inc = sqrt(2.0 / 3.0 * (t1 + 0.5 * t2));
    p_work_inc = stress[0] * ep[0] + stress[1] * ep[1] + stress[2] * ep[2] + stress[3] * ep[3] +
                 stress[4] * ep[4] + stress[5] * ep[5];
    for (int k = 0; k < 6; ++k) eps[k] = ee[k];
    const double ec_dot = p_strain_inc / q.tinc;
    double n_eff;
    if (ec_dot > 0.0) {
      for (int k = 0; k < 6; ++k) ep[k] = ep[k] / q.tinc;
      n_eff = 0.0;
      for (int s = 0; s < NS; ++s) {
        const double rs = rsc[s];
        double d = powr(fabs(rs), t.rate_n - 1.0);
        d = q.dg * t.rate_n / powr(tt, t.rate_n) * d;
        d = d + q.tinc * t.iD_v;
        t1 = G.ms[s][0] * ep[0] + G.ms[s][1] * ep[1] + G.ms[s][2] * ep[2];
        t2 = G.ms[s][3] * ep[3] + G.ms[s][4] * ep[4] + G.ms[s][5] * ep[5];
        const double ec_slip = t1 + 0.5 * t2;
        t1 = rs * d / ec_dot;
        t2 = ec_slip / ec_dot / q.tinc;
        n_eff = n_eff + (2.0 / 3.0) * t1 * t2;
      }
    } else {
      n_eff = 1.0e10;
    }
    u[11] = n_eff;
    double s_trace = (stress[0] + stress[1] + stress[2]) / 3.0;
    double se[6];
    for (int k = 0; k < 6; ++k) se[k] = stress[k];
    se[0] = se[0] - s_trace; se[1] = se[1] - s_trace; se[2] = se[2] - s_trace;
    t1 = se[0] * se[0] + se[1] * se[1] + se[2] * se[2];
    t2 = se[3] * se[3] + se[4] * se[4] + se[5] * se[5];
    s_trace = sqrt(1.5 * (t1 + 2.0 * t2));
    u[12] = s_trace;
    double B_eff;
    if (ec_dot < 1.0e-100) B_eff = 0.0;
    else if (n_eff > 100.0) B_eff = -1.0;
    else B_eff = ec_dot / pow(s_trace, n_eff);
    u[13] = B_eff;
    for (int s = 0; s < NS; ++s) slip_incs[s] = slip_incs[s] + dif[s];
    double maxslip = 0.0;
    int sysID = 0;
    for (int s = 0; s < NS; ++s) {
      const double cur = fabs(slip_incs[s]);
      if (cur > maxslip) { maxslip = cur; sysID = s + 1; }
    }
    u[5] = maxslip / q.tinc;
    u[6] = (double)sysID;
    int numAct = 0;
    maxslip = 0.1 * maxslip;
    for (int s = 0; s < NS; ++s)
      if (fabs(slip_incs[s]) >= maxslip) ++numAct;
    u[7] = (double)numAct;
  }
  // mm10_store_cryhist
  for (int k = 0; k < 6; ++k) hn1[C_STRESS + k] = stress[k];
  for (int k = 0; k < 3; ++k) hn1[C_EULER + k] = euler[k];
  for (int k = 0; k < 9; ++k) hn1[C_RP + k] = Rp1[k];
  for (int k = 0; k < 6; ++k) { hn1[C_D + k] = uddt[k]; hn1[C_EPS + k] = eps[k]; }
  for (int k = 0; k < NS; ++k) hn1[C_SLIP + k] = slip_incs[k];
  hn1[C_TT] = tt;
  for (int k = 0; k < 15; ++k) hn1[C_U + k] = u[k];
  hn1[C_TTRATE] = tt_rate;
  for (int k = 0; k < 6; ++k) { hn1[C_EP + k] = ep6[k]; hn1[C_ED + k] = ed6[k]; }
  // mm10_a_crystal_avgs (one crystal) + mm10_a_store_crystal
  const double rncry = 1.0;
  for (int k = 0; k < 6; ++k) urcs_n1[k] = stress[k] / rncry;
  for (int k = 0; k < 9; ++k) hn1[H_R + k] = R1[k];
  for (int k = 0; k < 36; ++k) hn1[H_TAN + k] = tangent[k] / rncry;
  for (int k = 0; k < 27; ++k) hn1[H_GRADFE + k] = 0.0;
  for (int k = 0; k < NS; ++k) hn1[H_SLIP + k] = slip_tot[k] + slip_incs[k] / rncry;
  const double tw = work_inc / rncry, pw = p_work_inc / rncry, ps = p_strain_inc / rncry;
  urcs_n1[6] = urcs_n[6] + tw;
  urcs_n1[7] = urcs_n[7] + pw;
  urcs_n1[8] = urcs_n[8] + ps;
  hn1[H_WORK + 0] = work3[0] + tw;
  hn1[H_WORK + 1] = work3[1] + pw;
  hn1[H_WORK + 2] = work3[2] + ps;
  return true;
}

// CTAs of k_mm10_update resident per SM (registers: 65536 / (128 x this)).
// Measured on the 32^3 polycrystal (recovery, sorted queue): 2 -> 24.4 ms,
// 3 -> 26.2 ms, 4 -> 26.5 ms: the local solve's working set outgrows the
// registers, and the added spills cost more than the added warps hide
#ifndef W3G_MM10_MIN_CTAS
#define W3G_MM10_MIN_CTAS 2
#endif
constexpr int kMm10MinCtas = W3G_MM10_MIN_CTAS;

// persistent: warps take 32 queue entries at a time
__global__ void __launch_bounds__(128, kMm10MinCtas) k_mm10_update(RecoverArgs a, WorkQueue q) {
  const IterParams p = *a.params;
  const int lane = threadIdx.x & 31;
  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(q.counter, 32);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= q.nitems) break;
    const int w = base + lane;
    if (w < q.nitems) {
      const int gpx = q.items[w];
      int iters = 0;
      if (!mm10_gp(a, p, gpx, &iters)) {
        const int code = a.mm10_gp[gpx];
        atomicMin(a.status, bad_point_key(code >> 12, code & 7, 2, (code >> 3) & 511));
      }
      a.mm10_iters[gpx] = iters;
    }
  }
}

// ---- work-queue order: counting sort by last iteration count, largest
// first (bins clamp at kBins - 1) ----
__global__ void k_mm10_bins_zero(int* bins) {
  if (threadIdx.x < 2 * kBins) bins[threadIdx.x] = 0;
}
__global__ void k_mm10_hist(const int* iters, int n, int* bins) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) atomicAdd(&bins[kBins - 1 - min(iters[k], kBins - 1)], 1);
}
__global__ void k_mm10_scan(int* bins) {
  if (threadIdx.x == 0) {
    int s = 0;
    for (int b = 0; b < kBins; ++b) { bins[kBins + b] = s; s += bins[b]; }
  }
}
__global__ void k_mm10_scatter(const int* iters, int n, int* bins, int* order) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) order[atomicAdd(&bins[kBins + kBins - 1 - min(iters[k], kBins - 1)], 1)] = k;
}

// ---------------------------------------------------------------------
// element forces, volumes, energies (rknifv / gpifv1, rstgp1_b)
// ---------------------------------------------------------------------
__global__ void __launch_bounds__(kRecoverThreads) k_mm10_forces(RecoverArgs a, int chunk0) {
  __shared__ double sfe[8][NG][TOT + 1];
  __shared__ double sred[2][2];
  const IterParams p = *a.params;
  const int tid = threadIdx.x;
  const int ge = tid >> 3, g = tid & 7;
  const int cidx = chunk0 + blockIdx.x;
  const Chunk ch = a.chunks[cidx];
  const BlockDesc bd = a.blocks[ch.blk];
  const bool active = ge < ch.n;
  const int i = ch.i0 + ge;
  double vol = 0.0, en = 0.0, pw = 0.0;
  if (active) {
    const long long gpi = bd.gp_off + (long long)i * NG + g;
    const double* geo = a.geo + bd.geo_off + ((long long)i * NG + g) * kGeo;
    const double* scr = a.mm10_scr + (long long)(bd.mm10_off + i * NG + g) * kMm10Scratch;
    const double* R1 = scr + 6;
    const double* F1 = scr + 15;
    const double dfn1 = scr[24];
    const double dj0 = geo[3 * NN];
    const double w = a.dn[0][NG * 3 * NN + g];
    const bool update_coords = bd.geonl && !(p.step == 1 && p.iter == 0);
    double cgn1[9];
    for (int k = 0; k < 9; ++k) cgn1[k] = a.urcs_n1[gpi * 9 + k];
    if (p.iter != 0) {
      const double factor = dfn1 * dj0 * a.beta_fact * w;
      en = cgn1[6] * factor;
      pw = cgn1[7] * factor;
    }
    double S[6];
    if (bd.geonl) rotate_to_spatial(R1, cgn1, S);
    else for (int k = 0; k < 6; ++k) S[k] = cgn1[k];
    const double j1 = update_coords ? dfn1 * dj0 : dj0;
    double pdiag = 0.0;
    if (bd.bbar) {
      // b-bar at n+1 (as for mm01): the element's mean pressure replaces
      // each point's
      const unsigned gmask = 0xFFu << (tid & 24);
      const double trs = S[0] + S[1] + S[2];
      double s1 = w * j1 * trs, s0 = j1;
      for (int off = 1; off < NG; off <<= 1) {
        s1 += __shfl_xor_sync(gmask, s1, off);
        s0 += __shfl_xor_sync(gmask, s0, off);
      }
      const double ptr = a.bbar_beta * trs;
      S[0] = S[0] - ptr; S[1] = S[1] - ptr; S[2] = S[2] - ptr;
      pdiag = a.bbar_beta * (s1 * (1.0 / s0)) * j1;
    }
    double P[9];
    const double wdj = w * j1;
    const double T[9] = {S[0] * wdj + pdiag, S[3] * wdj, S[5] * wdj, S[3] * wdj, S[1] * wdj + pdiag,
                         S[4] * wdj, S[5] * wdj, S[4] * wdj, S[2] * wdj + pdiag};
    if (update_coords) {
      const double r = 1.0 / dfn1;
      double Fi[9];
      Fi[0] = (F1[4] * F1[8] - F1[7] * F1[5]) * r; Fi[3] = (F1[6] * F1[5] - F1[3] * F1[8]) * r;
      Fi[6] = (F1[3] * F1[7] - F1[6] * F1[4]) * r; Fi[1] = (F1[7] * F1[2] - F1[1] * F1[8]) * r;
      Fi[4] = (F1[0] * F1[8] - F1[6] * F1[2]) * r; Fi[7] = (F1[6] * F1[1] - F1[0] * F1[7]) * r;
      Fi[2] = (F1[1] * F1[5] - F1[4] * F1[2]) * r; Fi[5] = (F1[3] * F1[2] - F1[0] * F1[5]) * r;
      Fi[8] = (F1[0] * F1[4] - F1[3] * F1[1]) * r;
      for (int c = 0; c < 3; ++c)
        for (int rr = 0; rr < 3; ++rr) P[rr + 3 * c] = T[rr] * Fi[c] + T[rr + 3] * Fi[c + 3] + T[rr + 6] * Fi[c + 6];
    } else {
      for (int k = 0; k < 9; ++k) P[k] = T[k];
    }
    vol = wdj;
    double* fe = sfe[ge][g];
    for (int n = 0; n < NN; ++n) {
      const double tx = geo[3 * n], ty = geo[3 * n + 1], tz = geo[3 * n + 2];
      fe[n] = P[0] * tx + P[3] * ty + P[6] * tz;
      fe[NN + n] = P[1] * tx + P[4] * ty + P[7] * tz;
      fe[2 * NN + n] = P[2] * tx + P[5] * ty + P[8] * tz;
    }
  }
  __syncthreads();
  if (active) {
    for (int d = 0; d < 3; ++d) {
      const int j = d * NN + g;
      double v = sfe[ge][0][j];
      for (int q = 1; q < NG; ++q) v += sfe[ge][q][j];
      a.einf[bd.einf_off + (long long)j * bd.span + i] = v;
    }
  }
  for (int off = 1; off < NG; off <<= 1) {
    vol += __shfl_xor_sync(0xffffffffu, vol, off);
    en += __shfl_xor_sync(0xffffffffu, en, off);
    pw += __shfl_xor_sync(0xffffffffu, pw, off);
  }
  if (active && g == 0) a.evol[bd.felem + i] = vol;
  en += __shfl_xor_sync(0xffffffffu, en, 8);
  pw += __shfl_xor_sync(0xffffffffu, pw, 8);
  en += __shfl_xor_sync(0xffffffffu, en, 16);
  pw += __shfl_xor_sync(0xffffffffu, pw, 16);
  if ((tid & 31) == 0) { sred[tid >> 5][0] = en; sred[tid >> 5][1] = pw; }
  __syncthreads();
  if (tid == 0) {
    a.partials[2 * cidx + 0] = sred[0][0] + sred[1][0];
    a.partials[2 * cidx + 1] = sred[0][1] + sred[1][1];
  }
}

int g_occ = 0;

}  // namespace

cudaError_t init_mm10_kernels() {
  int n = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mm10_update, 128, 0);
  if (e != cudaSuccess) return e;
  g_occ = std::max(1, n);
  return cudaSuccess;
}

int mm10_kernel_launches(const DeviceModel& m, bool sorted) {
  return m.mm10_chunks > 0 ? (sorted ? 7 : 3) : 0;
}

cudaError_t launch_mm10(const DeviceModel& m, const RecoverArgs& a, cudaStream_t s) {
  int* counter = a.mm10_counter;
  int* order = a.mm10_order;
  int* bins = a.mm10_bins;
  if (m.mm10_chunks == 0) return cudaSuccess;
  k_mm10_kin<<<m.mm10_chunks, kRecoverThreads, 0, s>>>(a, m.mm10_chunk0);
  const int n = m.n_mm10_gp;
  const int nb = (n + 255) / 256;
  if (a.mm10_sorted) {
    k_mm10_bins_zero<<<1, 2 * kBins, 0, s>>>(bins);
    k_mm10_hist<<<nb, 256, 0, s>>>(a.mm10_iters, n, bins);
    k_mm10_scan<<<1, 32, 0, s>>>(bins);
    k_mm10_scatter<<<nb, 256, 0, s>>>(a.mm10_iters, n, bins, order);
  }
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  const int warps = (n + 31) / 32;
  const int grid = std::max(1, std::min(m.nsm * g_occ, (warps + 3) / 4));
  WorkQueue q{a.mm10_sorted ? order : a.mm10_ident, n, 32, counter};
  k_mm10_update<<<grid, 128, 0, s>>>(a, q);
  k_mm10_forces<<<m.mm10_chunks, kRecoverThreads, 0, s>>>(a, m.mm10_chunk0);
  return cudaGetLastError();
}

// setup_mm10_rknstr for one element: the same operations, in the same
// order, as the oracle's restatement (closed-form isotropic stiffness,
// Kocks rotation, fcc slip systems rotated to the reference frame,
// stiffness rotated by rt2rve(g^T))
void build_crystal_elem(const w3g_crystal& cr, int type, const double* angles, CrystalElem& x) {
  const double pi = 3.141592653589793, one_eighty = 180.0;
  const double e = cr.e, nu = cr.nu;
  const double lam = e * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
  const double mu = e / (2.0 * (1.0 + nu));
  double C[36];
  for (int k = 0; k < 36; ++k) C[k] = 0.0;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) C[r + 6 * c] = lam;
  for (int r = 0; r < 3; ++r) C[r + 6 * r] = lam + 2.0 * mu;
  for (int r = 3; r < 6; ++r) C[r + 6 * r] = mu;
  const double psi = angles[0] * pi / one_eighty, theta = angles[1] * pi / one_eighty,
               phi = angles[2] * pi / one_eighty;
  double* g = x.g;
  g[0 + 3 * 0] = -std::sin(psi) * std::sin(phi) - std::cos(psi) * std::cos(phi) * std::cos(theta);
  g[0 + 3 * 1] = std::cos(psi) * std::sin(phi) - std::sin(psi) * std::cos(phi) * std::cos(theta);
  g[0 + 3 * 2] = std::cos(phi) * std::sin(theta);
  g[1 + 3 * 0] = std::sin(psi) * std::cos(phi) - std::cos(psi) * std::sin(phi) * std::cos(theta);
  g[1 + 3 * 1] = -std::cos(psi) * std::cos(phi) - std::sin(psi) * std::sin(phi) * std::cos(theta);
  g[1 + 3 * 2] = std::sin(phi) * std::sin(theta);
  g[2 + 3 * 0] = std::cos(psi) * std::sin(theta);
  g[2 + 3 * 1] = std::sin(psi) * std::sin(theta);
  g[2 + 3 * 2] = std::cos(theta);
  for (int k = 0; k < 3; ++k) x.angles[k] = angles[k];
  double tr[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) tr[r + 3 * c] = g[c + 3 * r];
  // the 12 systems of finalize_new_crystal (src/mod_crystals.f:440-596):
  // fcc {111}<110> (slip_type 1) takes the <110> vectors as directions b
  // and the <111> vectors as normals n; bcc {110}<111> (slip_type 2) the
  // same two tables the other way round
  const double f = 1.0 / std::sqrt(2.0), h = 1.0 / std::sqrt(3.0);
  const double v110[kSlip][3] = {{0, -f, f}, {f, 0, -f}, {-f, f, 0}, {0, f, f}, {f, 0, f}, {f, -f, 0},
                                 {0, -f, f}, {-f, 0, -f}, {f, f, 0}, {0, f, f}, {f, 0, -f}, {-f, -f, 0}};
  const double v111[kSlip][3] = {{h, h, h}, {h, h, h}, {h, h, h}, {-h, -h, h}, {-h, -h, h}, {-h, -h, h},
                                 {-h, h, h}, {-h, h, h}, {-h, h, h}, {h, -h, h}, {h, -h, h}, {h, -h, h}};
  const bool bcc = cr.slip_type == 2;
  const double(*b)[3] = bcc ? v111 : v110;
  const double(*nrm)[3] = bcc ? v110 : v111;
  for (int s = 0; s < kSlip; ++s) {
    double bs[3], ns[3], A[9], As[9], Aa[9];
    for (int r = 0; r < 3; ++r) bs[r] = tr[r] * b[s][0] + tr[r + 3] * b[s][1] + tr[r + 6] * b[s][2];
    for (int r = 0; r < 3; ++r) ns[r] = tr[r] * nrm[s][0] + tr[r + 3] * nrm[s][1] + tr[r + 6] * nrm[s][2];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) A[r + 3 * c] = bs[r] * ns[c];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        As[r + 3 * c] = 0.5 * (A[r + 3 * c] + A[c + 3 * r]);
        Aa[r + 3 * c] = 0.5 * (A[r + 3 * c] - A[c + 3 * r]);
      }
    x.ms[s][0] = As[0]; x.ms[s][1] = As[4]; x.ms[s][2] = As[8];
    x.ms[s][3] = 2.0 * As[0 + 3 * 1]; x.ms[s][4] = 2.0 * As[1 + 3 * 2]; x.ms[s][5] = 2.0 * As[0 + 3 * 2];
    x.qs[s][0] = Aa[1 + 3 * 2]; x.qs[s][1] = Aa[0 + 3 * 2]; x.qs[s][2] = Aa[0 + 3 * 1];
  }
  // C rotated: Rs C Rs^T with Rs = rt2rve(g^T), products summed k = 1..6
  double Rs[36], temp[36];
  {
    const double* rt = tr;
    double* rv = Rs;
#define RT(a, b) rt[(a - 1) + 3 * (b - 1)]
#define RV(a, b) rv[(a - 1) + 6 * (b - 1)]
    RV(1, 1) = RT(1, 1) * RT(1, 1); RV(1, 2) = RT(1, 2) * RT(1, 2); RV(1, 3) = RT(1, 3) * RT(1, 3);
    RV(1, 4) = 2.0 * RT(1, 1) * RT(1, 2); RV(1, 5) = 2.0 * RT(1, 3) * RT(1, 2); RV(1, 6) = 2.0 * RT(1, 1) * RT(1, 3);
    RV(2, 1) = RT(2, 1) * RT(2, 1); RV(2, 2) = RT(2, 2) * RT(2, 2); RV(2, 3) = RT(2, 3) * RT(2, 3);
    RV(2, 4) = 2.0 * RT(2, 1) * RT(2, 2); RV(2, 5) = 2.0 * RT(2, 3) * RT(2, 2); RV(2, 6) = 2.0 * RT(2, 1) * RT(2, 3);
    RV(3, 1) = RT(3, 1) * RT(3, 1); RV(3, 2) = RT(3, 2) * RT(3, 2); RV(3, 3) = RT(3, 3) * RT(3, 3);
    RV(3, 4) = 2.0 * RT(3, 1) * RT(3, 2); RV(3, 5) = 2.0 * RT(3, 3) * RT(3, 2); RV(3, 6) = 2.0 * RT(3, 1) * RT(3, 3);
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
#undef RT
  }
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) {
      double sum = 0.0;
      for (int k = 0; k < 6; ++k) sum = sum + C[r + 6 * k] * Rs[c + 6 * k];
      temp[r + 6 * c] = sum;
    }
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) {
      double sum = 0.0;
      for (int k = 0; k < 6; ++k) sum = sum + Rs[r + 6 * k] * temp[k + 6 * c];
      x.C[r + 6 * c] = sum;
    }
  x.type = type;
  x.pad = 0;
}

}  // namespace w3g
