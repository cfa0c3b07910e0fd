// w3o.cpp -- the oracle: CPU restatement of WARP3D's element-block hot
// path. TEST INFRASTRUCTURE ONLY (parity checker and timed CPU baseline);
// the product path never links or calls this file.
//
// Parity status: WARP3D is Fortran + Intel MKL and no Fortran compiler
// exists on these machines, and the reference's own tests (verification/*)
// are end-to-end decks with no element-level golden vectors. Two of them
// pin this oracle end to end, replayed from their data: verification/test24
// (mm01, finite-strain b-bar bricks, skew constraints, 21 load steps) to
// 3.6e-6 and verification/test82/voche_model (mm10, bcc, Voce, face
// pressures) to 4.0e-5 of the element stress each checker compares (their
// tolerance 1e-4; tests/test_oracle_warp3d_test24.py, _test82.py).
// Everything else is pinned by closed-form known answers
// (tests/test_oracle_*.py): patch tests, rigid-body motions, the analytic
// bilinear uniaxial response and finite-difference checks of the
// consistent tangent.
//
// Every routine follows the cited Fortran statement by statement,
// including its literal constants and evaluation order, so that the
// oracle's arithmetic is the reference's arithmetic. Arrays that the
// reference holds as (mxvl, ...) block-local work arrays are held here as
// column-major [component][element] arrays of the block.
//
// Build: oracle/build.sh (g++ -O2 -fopenmp -ffp-contract=off).

#include "w3o.h"
#include "w3o_mm10.h"
#include "w3o_umat.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int MXVL = W3G_MXVL;
constexpr int MXELPR = W3G_MXELPR;
constexpr int NSTR = 6;
constexpr int NSTRS = 9;
constexpr int MM01_HIST = 11;   // mm01_set_sizes, src/mm01.f:976-979
constexpr int MM10_HIST = w3o::MM10_HIST;
inline int hist_size(int mat_type) {
  return mat_type == W3G_MAT_CRYSTAL ? MM10_HIST : mat_type == W3G_MAT_UMAT ? w3o::UMAT_NSTATV : MM01_HIST;
}

int g_threads = 0;
int g_deterministic = 1;

// ---------------------------------------------------------------------
// module constants, src/mod_main.f:541-622
// ---------------------------------------------------------------------
const double zero = 0.0, one = 1.0, two = 2.0, three = 3.0;
const double half = 0.5, quarter = 0.25, onept5 = 1.5;
const double thirteenpt5 = 13.5, sixpt75 = 6.75, twentyseven = 27.0;
const double third = 1.0 / 3.0;
const double iroot3 = 1.0 / std::sqrt(3.0);

// Fortran logicals arrive as int32, nonzero = .true.
inline bool flog(int v) { return v != 0; }

// history word 4 of mm01 holds an integer through an equivalence with a
// double (src/mm01.f:251-284, :651-652): the low 32 bits are the state.
inline int state_of(double d) {
  uint64_t b; std::memcpy(&b, &d, 8); return (int)(int32_t)(uint32_t)(b & 0xffffffffu);
}
inline double state_word(int s) {
  uint64_t b = (uint64_t)(uint32_t)s; double d; std::memcpy(&d, &b, 8); return d;
}

// ---------------------------------------------------------------------
// element library: getgpts.f / derivs.f
// ---------------------------------------------------------------------

// quad2, src/getgpts.f:642-700: 2x2x2 rule for the 8-node brick.
bool quad2(int order, int gpn, double& xi, double& eta, double& zeta, double& w) {
  if (order != 1) return false;
  const double l1 = 0.5773502691896257645, w1 = 1.0;
  static const int sx[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
  static const int se[8] = {-1, 1, -1, 1, -1, 1, -1, 1};
  static const int sz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
  if (gpn < 1 || gpn > 8) return false;
  xi = sx[gpn - 1] * l1; eta = se[gpn - 1] * l1; zeta = sz[gpn - 1] * l1; w = w1;
  return true;
}

// deriv2, src/derivs.f:283-328: 8-node brick shape-function derivatives.
void deriv2(double xi, double eta, double zeta, double* nxi, double* neta, double* nzeta) {
  const double one25 = 0.125;
  double xp = one + xi, ep = one + eta, zp = one + zeta;
  double xm = one - xi, em = one - eta, zm = one - zeta;
  nxi[0] = -(em * zp * one25); neta[0] = -(xm * zp * one25); nzeta[0] = xm * em * one25;
  nxi[1] = -(em * zm * one25); neta[1] = -(xm * zm * one25); nzeta[1] = -(xm * em * one25);
  nxi[2] = -(ep * zm * one25); neta[2] = xm * zm * one25;    nzeta[2] = -(xm * ep * one25);
  nxi[3] = -(ep * zp * one25); neta[3] = xm * zp * one25;    nzeta[3] = xm * ep * one25;
  nxi[4] = em * zp * one25;    neta[4] = -(xp * zp * one25); nzeta[4] = xp * em * one25;
  nxi[5] = em * zm * one25;    neta[5] = -(xp * zm * one25); nzeta[5] = -(xp * em * one25);
  nxi[6] = ep * zm * one25;    neta[6] = xp * zm * one25;    nzeta[6] = -(xp * ep * one25);
  nxi[7] = ep * zp * one25;    neta[7] = xp * zp * one25;    nzeta[7] = xp * ep * one25;
}

// quad1, src/getgpts.f:177-420: 27-point rule (order 1) of the 20-node
// brick; eta fastest, then xi, then zeta; weights by the number of zero
// coordinates (w1..w4).
bool quad1(int order, int gpn, double& xi, double& eta, double& zeta, double& w) {
  if (order != 1 || gpn < 1 || gpn > 27) return false;
  const double l1 = 0.774596669241483, l2 = 0.0;
  const double w1 = 0.1714677640603571, w2 = 0.2743484224965712, w3 = 0.4389574759945135,
               w4 = 0.7023319615912210;
  const double v[3] = {-l1, l2, l1};
  int g = gpn - 1;
  int ie = g % 3, ix = (g / 3) % 3, iz = g / 9;
  xi = v[ix]; eta = v[ie]; zeta = v[iz];
  int zeros = (ix == 1) + (ie == 1) + (iz == 1);
  const double ws[4] = {w1, w2, w3, w4};
  w = ws[zeros];
  return true;
}

// deriv1, src/derivs.f:182-281: 20-node brick
void deriv1(double r, double s, double t, double* nr, double* ns, double* nt) {
  const double one = 1.0, half = 0.5, fourth = 0.25, eighth = 0.125;
  double rp1 = one + r, rm1 = one - r, sp1 = one + s, sm1 = one - s, tp1 = one + t, tm1 = one - t;
  double rps = r + s, rms = r - s, spt = s + t, smt = s - t;
  nr[0] = sm1 * (rp1 + rps - t) * tp1 * eighth;
  nr[1] = sm1 * (rp1 + rps + t) * tm1 * eighth;
  nr[2] = sp1 * (rp1 + rms + t) * tm1 * eighth;
  nr[3] = sp1 * (rp1 + rms - t) * tp1 * eighth;
  nr[4] = -sm1 * (rm1 - rms - t) * tp1 * eighth;
  nr[5] = -sm1 * (rm1 - rms + t) * tm1 * eighth;
  nr[6] = -sp1 * (rm1 - rps + t) * tm1 * eighth;
  nr[7] = -sp1 * (rm1 - rps - t) * tp1 * eighth;
  nr[8] = -sm1 * tm1 * tp1 * fourth;
  nr[9] = -sm1 * sp1 * tm1 * fourth;
  nr[10] = -sp1 * tm1 * tp1 * fourth;
  nr[11] = -sm1 * sp1 * tp1 * fourth;
  nr[12] = sm1 * tm1 * tp1 * fourth;
  nr[13] = sm1 * sp1 * tm1 * fourth;
  nr[14] = sp1 * tm1 * tp1 * fourth;
  nr[15] = sm1 * sp1 * tp1 * fourth;
  nr[16] = -r * sm1 * tp1 * half;
  nr[17] = -r * sm1 * tm1 * half;
  nr[18] = -r * sp1 * tm1 * half;
  nr[19] = -r * sp1 * tp1 * half;
  ns[0] = rm1 * (rp1 + s + smt) * tp1 * eighth;
  ns[1] = rm1 * (rp1 + s + spt) * tm1 * eighth;
  ns[2] = -rm1 * (rp1 - s - smt) * tm1 * eighth;
  ns[3] = -rm1 * (rp1 - s - spt) * tp1 * eighth;
  ns[4] = rp1 * (rm1 + s + smt) * tp1 * eighth;
  ns[5] = rp1 * (rm1 + s + spt) * tm1 * eighth;
  ns[6] = -rp1 * (rm1 - s - smt) * tm1 * eighth;
  ns[7] = -rp1 * (rm1 - s - spt) * tp1 * eighth;
  ns[8] = -rm1 * tm1 * tp1 * fourth;
  ns[9] = -rm1 * s * tm1 * half;
  ns[10] = rm1 * tm1 * tp1 * fourth;
  ns[11] = -rm1 * s * tp1 * half;
  ns[12] = -rp1 * tm1 * tp1 * fourth;
  ns[13] = -rp1 * s * tm1 * half;
  ns[14] = rp1 * tm1 * tp1 * fourth;
  ns[15] = -rp1 * s * tp1 * half;
  ns[16] = -rm1 * rp1 * tp1 * fourth;
  ns[17] = -rm1 * rp1 * tm1 * fourth;
  ns[18] = rm1 * rp1 * tm1 * fourth;
  ns[19] = rm1 * rp1 * tp1 * fourth;
  nt[0] = -rm1 * sm1 * (rp1 + smt - t) * eighth;
  nt[1] = rm1 * sm1 * (rp1 + spt + t) * eighth;
  nt[2] = rm1 * sp1 * (rp1 - smt + t) * eighth;
  nt[3] = -rm1 * sp1 * (rp1 - spt - t) * eighth;
  nt[4] = -rp1 * sm1 * (rm1 + smt - t) * eighth;
  nt[5] = rp1 * sm1 * (rm1 + spt + t) * eighth;
  nt[6] = rp1 * sp1 * (rm1 - smt + t) * eighth;
  nt[7] = -rp1 * sp1 * (rm1 - spt - t) * eighth;
  nt[8] = -rm1 * sm1 * t * half;
  nt[9] = -rm1 * sm1 * sp1 * fourth;
  nt[10] = -rm1 * sp1 * t * half;
  nt[11] = rm1 * sm1 * sp1 * fourth;
  nt[12] = -rp1 * sm1 * t * half;
  nt[13] = -rp1 * sm1 * sp1 * fourth;
  nt[14] = -rp1 * sp1 * t * half;
  nt[15] = rp1 * sm1 * sp1 * fourth;
  nt[16] = rm1 * rp1 * sm1 * fourth;
  nt[17] = -rm1 * rp1 * sm1 * fourth;
  nt[18] = -rm1 * rp1 * sp1 * fourth;
  nt[19] = rm1 * rp1 * sp1 * fourth;
}

// quad6, src/getgpts.f:771-850: 4-point rule (order 4) of the tetrahedra;
// returns (s2, s3, s4) as (xi, eta, zeta).
bool quad6(int order, int gpn, double& xi, double& eta, double& zeta, double& w) {
  if (order != 4 || gpn < 1 || gpn > 4) return false;
  const double a = 0.58541020, b = 0.13819660;
  w = 0.25;
  xi = gpn == 2 ? a : b;
  eta = gpn == 3 ? a : b;
  zeta = gpn == 4 ? a : b;
  return true;
}

// deriv6, src/derivs.f:606-662: 10-node tetrahedron
void deriv6(double s2, double s3, double s4, double* qs2, double* qs3, double* qs4) {
  const double zero = 0.0, one = 1.0, four = 4.0;
  double s1 = one - s2 - s3 - s4;
  qs2[0] = one - four * s1; qs2[1] = four * s2 - one; qs2[2] = zero; qs2[3] = zero;
  qs2[4] = four * (s1 - s2); qs2[5] = four * s3; qs2[6] = -four * s3; qs2[7] = -four * s4;
  qs2[8] = four * s4; qs2[9] = zero;
  qs3[0] = one - four * s1; qs3[1] = zero; qs3[2] = four * s3 - one; qs3[3] = zero;
  qs3[4] = -four * s2; qs3[5] = four * s2; qs3[6] = four * (s1 - s3); qs3[7] = -four * s4;
  qs3[8] = zero; qs3[9] = four * s4;
  qs4[0] = one - four * s1; qs4[1] = zero; qs4[2] = zero; qs4[3] = four * s4 - one;
  qs4[4] = -four * s2; qs4[5] = zero; qs4[6] = -four * s3; qs4[7] = four * (s1 - s4);
  qs4[8] = four * s2; qs4[9] = four * s3;
}

bool getgpts(int etype, int order, int gpn, double& xi, double& eta, double& zeta, double& w) {
  switch (etype) {
    case W3G_ETYPE_L3DISOP: return quad2(order, gpn, xi, eta, zeta, w);
    case W3G_ETYPE_Q3DISOP: return quad1(order, gpn, xi, eta, zeta, w);
    case W3G_ETYPE_TET10: return quad6(order, gpn, xi, eta, zeta, w);
    default: return false;
  }
}

bool derivs(int etype, double xi, double eta, double zeta, double* nxi, double* neta, double* nzeta) {
  switch (etype) {
    case W3G_ETYPE_L3DISOP: deriv2(xi, eta, zeta, nxi, neta, nzeta); return true;
    case W3G_ETYPE_Q3DISOP: deriv1(xi, eta, zeta, nxi, neta, nzeta); return true;
    case W3G_ETYPE_TET10: deriv6(xi, eta, zeta, nxi, neta, nzeta); return true;
    default: return false;
  }
}

// adjust_scalar_weights, src/initst.f:888-930: tetrahedra integrate with
// weights summing to 1 over the unit parametric tet of volume 1/6
double adjust_scalar(int etype) { return etype == W3G_ETYPE_TET10 ? 1.0 / 6.0 : 1.0; }

// ---------------------------------------------------------------------
// block description
// ---------------------------------------------------------------------
struct Blk {
  int blk, span, felem;      // felem 1-based
  int etype, order, ngp, nnode, ndof, totdof, utsz, mat_type;
  bool geonl, bbar;
};

bool block_info(const w3g_model_desc* m, int blk, Blk& b) {
  b.blk = blk;
  b.span = m->elblks[3 * blk + 0];
  b.felem = m->elblks[3 * blk + 1];
  const int* ip = m->iprops + (size_t)(b.felem - 1) * MXELPR;
  const int* lp = m->lprops + (size_t)(b.felem - 1) * MXELPR;
  b.etype = ip[0]; b.nnode = ip[1]; b.ndof = ip[3]; b.order = ip[4];
  b.ngp = ip[5]; b.mat_type = ip[24];
  b.totdof = b.nnode * b.ndof;
  b.utsz = (b.totdof * b.totdof - b.totdof) / 2 + b.totdof;   // tanstf.f:185
  b.geonl = flog(lp[17]); b.bbar = flog(lp[18]);
  const bool known = (b.etype == W3G_ETYPE_L3DISOP && b.nnode == 8 && b.ngp == 8) ||
                     (b.etype == W3G_ETYPE_Q3DISOP && b.nnode == 20 && b.ngp == 27) ||
                     (b.etype == W3G_ETYPE_TET10 && b.nnode == 10 && b.ngp == 4);
  return b.span >= 1 && b.span <= MXVL && known && b.ndof == 3;
}

// column-major helpers for (span, k) and (span, k, l) work arrays
struct A2 {  // a(i, k): i = 0..MXVL-1 element, k component
  std::vector<double> v; int nk;
  explicit A2(int nk_) : v((size_t)MXVL * nk_, 0.0), nk(nk_) {}
  double& operator()(int i, int k) { return v[(size_t)k * MXVL + i]; }
  double* col(int k) { return &v[(size_t)k * MXVL]; }
  void zero() { std::fill(v.begin(), v.end(), 0.0); }
};

// ---------------------------------------------------------------------
// jacob1, src/gtmat1.f:300-507 (3-D solid branch)
// ce: (span, 3*nnode) x1..xn, y1..yn, z1..zn
// ---------------------------------------------------------------------
void jacob1(int span, int nnode, const double* nxi, const double* neta, const double* nzeta,
            A2& ce, double* dj, A2& gama /* (span, 9): (r,c) -> r + 3c */) {
  double jac[9][MXVL];
  for (int k = 0; k < 9; ++k) for (int i = 0; i < span; ++i) jac[k][i] = zero;
  for (int j = 0; j < nnode; ++j) {
    for (int i = 0; i < span; ++i) {
      double x = ce(i, j), y = ce(i, nnode + j), z = ce(i, 2 * nnode + j);
      jac[0][i] = jac[0][i] + nxi[j] * x;     // (1,1)
      jac[3][i] = jac[3][i] + nxi[j] * y;     // (1,2)
      jac[6][i] = jac[6][i] + nxi[j] * z;     // (1,3)
      jac[1][i] = jac[1][i] + neta[j] * x;    // (2,1)
      jac[4][i] = jac[4][i] + neta[j] * y;    // (2,2)
      jac[7][i] = jac[7][i] + neta[j] * z;    // (2,3)
      jac[2][i] = jac[2][i] + nzeta[j] * x;   // (3,1)
      jac[5][i] = jac[5][i] + nzeta[j] * y;   // (3,2)
      jac[8][i] = jac[8][i] + nzeta[j] * z;   // (3,3)
    }
  }
#define J(r, c) jac[(r - 1) + 3 * (c - 1)][i]
  for (int i = 0; i < span; ++i) {
    double j1 = J(2, 2) * J(3, 3) - J(2, 3) * J(3, 2);
    double j2 = J(2, 1) * J(3, 3) - J(2, 3) * J(3, 1);
    double j3 = J(2, 1) * J(3, 2) - J(2, 2) * J(3, 1);
    dj[i] = J(1, 1) * j1 - J(1, 2) * j2 + J(1, 3) * j3;
    gama(i, 0) = j1 / dj[i];
    gama(i, 1) = -j2 / dj[i];
    gama(i, 2) = j3 / dj[i];
    gama(i, 3) = (J(3, 2) * J(1, 3) - J(1, 2) * J(3, 3)) / dj[i];
    gama(i, 4) = (J(1, 1) * J(3, 3) - J(3, 1) * J(1, 3)) / dj[i];
    gama(i, 5) = (J(1, 2) * J(3, 1) - J(1, 1) * J(3, 2)) / dj[i];
    gama(i, 6) = (J(1, 2) * J(2, 3) - J(1, 3) * J(2, 2)) / dj[i];
    gama(i, 7) = (J(1, 3) * J(2, 1) - J(1, 1) * J(2, 3)) / dj[i];
    gama(i, 8) = (J(1, 1) * J(2, 2) - J(1, 2) * J(2, 1)) / dj[i];
  }
#undef J
}
#define G(r, c) gama(i, (r - 1) + 3 * (c - 1))

// blcmp1, src/blcmp1.f:15-81: linear [B] (span, totdof, 6) at one GP.
// b is stored as b[(k)*totdof + j](i) -> use A2 with nk = totdof*6,
// index j + totdof*k.
void blcmp1(int span, A2& b, int totdof, A2& gama, const double* nxi, const double* neta,
            const double* nzeta, int nnode) {
  int bpos1 = nnode, bpos2 = 2 * nnode;
  for (int j = 0; j < nnode; ++j) {
    for (int i = 0; i < span; ++i) {
      double t1 = G(1, 1) * nxi[j] + G(1, 2) * neta[j] + G(1, 3) * nzeta[j];
      double t2 = G(2, 1) * nxi[j] + G(2, 2) * neta[j] + G(2, 3) * nzeta[j];
      double t3 = G(3, 1) * nxi[j] + G(3, 2) * neta[j] + G(3, 3) * nzeta[j];
      b(i, j + totdof * 0) = t1;
      b(i, j + totdof * 3) = t2;
      b(i, j + totdof * 5) = t3;
      b(i, bpos1 + j + totdof * 1) = t2;
      b(i, bpos1 + j + totdof * 3) = t1;
      b(i, bpos1 + j + totdof * 4) = t3;
      b(i, bpos2 + j + totdof * 2) = t3;
      b(i, bpos2 + j + totdof * 4) = t2;
      b(i, bpos2 + j + totdof * 5) = t1;
    }
  }
}

// ---------------------------------------------------------------------
// b-bar (mean dilatation) of the 8-node brick. vol: (span, 8, 3) held as
// A2 with index j + 8k (node j, derivative k = x, y, z).
// ---------------------------------------------------------------------
// vol_terms, src/vol_terms.f:14-108: adds one Gauss point's
// det[J] dN_j/dx_k to vol and det[J] to volume
void vol_terms(int span, A2& gama, const double* dj, A2& vol, const double* nxi, const double* neta,
               const double* nzeta, double* volume) {
  for (int i = 0; i < span; ++i) {
    const double d = dj[i];
    for (int k = 1; k <= 3; ++k) {
      const double a = G(k, 1), bb = G(k, 2), c = G(k, 3);
      for (int j = 0; j < 8; ++j)
        vol(i, j + 8 * (k - 1)) = vol(i, j + 8 * (k - 1)) + (a * nxi[j] + bb * neta[j] + c * nzeta[j]) * d;
    }
    volume[i] = volume[i] + d;
  }
}

// vol_avg, src/vol_avg.f:13-68: volume-averaged derivatives
void vol_avg(int span, A2& vol, const double* volume) {
  for (int i = 0; i < span; ++i) {
    const double voli = one / volume[i];
    for (int k = 0; k < 24; ++k) vol(i, k) = vol(i, k) * voli;
  }
}

// bmod, src/bmod.f:16-205: replaces the dilatational part of [B] (rows
// xx, yy, zz) by the element's mean dilatation, in the reference's order
// of updates (the second loop reads entries the first has rewritten)
void bmod(int span, A2& b, int totdof, A2& vol, double eps_stab) {
  const double alpha = (two + eps_stab) * third;
  const double beta = (one - eps_stab) * third;
#define BB(i, j, k) b(i, (j) + totdof * (k))
#define VB(i, j, k) vol(i, (j) + 8 * (k))
  for (int i = 0; i < span; ++i) {
    double dummy[8];
    for (int j = 0; j < 8; ++j) dummy[j] = BB(i, j, 0);
    for (int j = 0; j < 8; ++j) BB(i, j, 0) = alpha * dummy[j] + beta * VB(i, j, 0);
    for (int j = 0; j < 8; ++j) BB(i, j, 1) = beta * (VB(i, j, 0) - dummy[j]);
  }
  for (int i = 0; i < span; ++i) {
    for (int j = 0; j < 8; ++j) BB(i, 8 + j, 0) = beta * (VB(i, j, 1) - BB(i, 8 + j, 1));
    for (int j = 0; j < 8; ++j) BB(i, 16 + j, 0) = beta * (VB(i, j, 2) - BB(i, 16 + j, 2));
    for (int j = 0; j < 8; ++j) BB(i, 8 + j, 1) = alpha * BB(i, 8 + j, 1) + beta * VB(i, j, 1);
    for (int j = 0; j < 8; ++j) BB(i, 16 + j, 1) = BB(i, 16 + j, 0);
    for (int j = 0; j < 8; ++j) BB(i, j, 2) = BB(i, j, 1);
    for (int j = 0; j < 8; ++j) BB(i, 8 + j, 2) = BB(i, 8 + j, 0);
    for (int j = 0; j < 8; ++j) BB(i, 16 + j, 2) = alpha * BB(i, 16 + j, 2) + beta * VB(i, j, 2);
  }
#undef BB
#undef VB
}

// getrm1, src/gtmat1.f:740-960. r: (span, 9) column-major 3x3 at one GP
// (rot(r,c) -> r + 3c). q: (span, 36), q(i, r, c) -> (r-1) + 6(c-1).
void getrm1(int span, A2& q, const double* const* rcol /* 9 columns */, int opt) {
  for (int i = 0; i < span; ++i) {
#define R(a, b) rcol[(a - 1) + 3 * (b - 1)][i]
#define Q(a, b) q(i, (a - 1) + 6 * (b - 1))
    if (opt == 1) {
      Q(1, 1) = R(1, 1) * R(1, 1); Q(1, 2) = R(2, 1) * R(2, 1); Q(1, 3) = R(3, 1) * R(3, 1);
      Q(1, 4) = R(1, 1) * R(2, 1); Q(1, 5) = R(3, 1) * R(2, 1); Q(1, 6) = R(1, 1) * R(3, 1);
      Q(2, 1) = R(1, 2) * R(1, 2); Q(2, 2) = R(2, 2) * R(2, 2); Q(2, 3) = R(3, 2) * R(3, 2);
      Q(2, 4) = R(1, 2) * R(2, 2); Q(2, 5) = R(3, 2) * R(2, 2); Q(2, 6) = R(1, 2) * R(3, 2);
      Q(3, 1) = R(1, 3) * R(1, 3); Q(3, 2) = R(2, 3) * R(2, 3); Q(3, 3) = R(3, 3) * R(3, 3);
      Q(3, 4) = R(1, 3) * R(2, 3); Q(3, 5) = R(3, 3) * R(2, 3); Q(3, 6) = R(1, 3) * R(3, 3);
      Q(4, 1) = two * R(1, 1) * R(1, 2); Q(4, 2) = two * R(2, 1) * R(2, 2);
      Q(4, 3) = two * R(3, 1) * R(3, 2);
      Q(4, 4) = R(1, 1) * R(2, 2) + R(1, 2) * R(2, 1);
      Q(4, 5) = R(2, 1) * R(3, 2) + R(3, 1) * R(2, 2);
      Q(4, 6) = R(1, 1) * R(3, 2) + R(3, 1) * R(1, 2);
      Q(5, 1) = two * R(1, 2) * R(1, 3); Q(5, 2) = two * R(2, 3) * R(2, 2);
      Q(5, 3) = two * R(3, 2) * R(3, 3);
      Q(5, 4) = R(1, 2) * R(2, 3) + R(2, 2) * R(1, 3);
      Q(5, 5) = R(2, 2) * R(3, 3) + R(2, 3) * R(3, 2);
      Q(5, 6) = R(1, 2) * R(3, 3) + R(3, 2) * R(1, 3);
      Q(6, 1) = two * R(1, 1) * R(1, 3); Q(6, 2) = two * R(2, 1) * R(2, 3);
      Q(6, 3) = two * R(3, 1) * R(3, 3);
      Q(6, 4) = R(1, 1) * R(2, 3) + R(2, 1) * R(1, 3);
      Q(6, 5) = R(2, 1) * R(3, 3) + R(3, 1) * R(2, 3);
      Q(6, 6) = R(1, 1) * R(3, 3) + R(1, 3) * R(3, 1);
    } else {  // opt 2
      Q(1, 1) = R(1, 1) * R(1, 1); Q(1, 2) = R(1, 2) * R(1, 2); Q(1, 3) = R(1, 3) * R(1, 3);
      Q(1, 4) = two * R(1, 1) * R(1, 2); Q(1, 5) = two * R(1, 3) * R(1, 2);
      Q(1, 6) = two * R(1, 1) * R(1, 3);
      Q(2, 1) = R(2, 1) * R(2, 1); Q(2, 2) = R(2, 2) * R(2, 2); Q(2, 3) = R(2, 3) * R(2, 3);
      Q(2, 4) = two * R(2, 1) * R(2, 2); Q(2, 5) = two * R(2, 3) * R(2, 2);
      Q(2, 6) = two * R(2, 1) * R(2, 3);
      Q(3, 1) = R(3, 1) * R(3, 1); Q(3, 2) = R(3, 2) * R(3, 2); Q(3, 3) = R(3, 3) * R(3, 3);
      Q(3, 4) = two * R(3, 1) * R(3, 2); Q(3, 5) = two * R(3, 3) * R(3, 2);
      Q(3, 6) = two * R(3, 1) * R(3, 3);
      Q(4, 1) = R(1, 1) * R(2, 1); Q(4, 2) = R(1, 2) * R(2, 2); Q(4, 3) = R(1, 3) * R(2, 3);
      Q(4, 4) = R(1, 1) * R(2, 2) + R(2, 1) * R(1, 2);
      Q(4, 5) = R(1, 2) * R(2, 3) + R(1, 3) * R(2, 2);
      Q(4, 6) = R(1, 1) * R(2, 3) + R(1, 3) * R(2, 1);
      Q(5, 1) = R(2, 1) * R(3, 1); Q(5, 2) = R(3, 2) * R(2, 2); Q(5, 3) = R(2, 3) * R(3, 3);
      Q(5, 4) = R(2, 1) * R(3, 2) + R(2, 2) * R(3, 1);
      Q(5, 5) = R(2, 2) * R(3, 3) + R(3, 2) * R(2, 3);
      Q(5, 6) = R(2, 1) * R(3, 3) + R(2, 3) * R(3, 1);
      Q(6, 1) = R(1, 1) * R(3, 1); Q(6, 2) = R(1, 2) * R(3, 2); Q(6, 3) = R(1, 3) * R(3, 3);
      Q(6, 4) = R(1, 1) * R(3, 2) + R(1, 2) * R(3, 1);
      Q(6, 5) = R(1, 2) * R(3, 3) + R(1, 3) * R(3, 2);
      Q(6, 6) = R(1, 1) * R(3, 3) + R(3, 1) * R(1, 3);
    }
#undef R
#undef Q
  }
}

// qmply1, src/qmply1.f:15-36: m2 = q * m1 (6x6 * 6)
void qmply1(int span, A2& q, const double* const* m1, double* const* m2) {
  for (int j = 1; j <= 6; ++j)
    for (int i = 0; i < span; ++i) {
#define Q(a, b) q(i, (a - 1) + 6 * (b - 1))
      m2[j - 1][i] = Q(j, 1) * m1[0][i] + Q(j, 2) * m1[1][i] + Q(j, 3) * m1[2][i] +
                     Q(j, 4) * m1[3][i] + Q(j, 5) * m1[4][i] + Q(j, 6) * m1[5][i];
#undef Q
    }
}

// tcomp1, src/gtmat1.f:522-590: displacement gradient theta (span, 9)
void tcomp1(int span, A2& theta, const double* nxi, const double* neta, const double* nzeta,
            A2& gama, A2& ue, int nnode) {
  theta.zero();
  std::vector<double> th((size_t)3 * MXVL * nnode);
  auto T = [&](int i, int j, int k) -> double& { return th[((size_t)k * nnode + j) * MXVL + i]; };
  for (int j = 0; j < nnode; ++j)
    for (int i = 0; i < span; ++i) {
      T(i, j, 0) = G(1, 1) * nxi[j] + G(1, 2) * neta[j] + G(1, 3) * nzeta[j];
      T(i, j, 1) = G(2, 1) * nxi[j] + G(2, 2) * neta[j] + G(2, 3) * nzeta[j];
      T(i, j, 2) = G(3, 1) * nxi[j] + G(3, 2) * neta[j] + G(3, 3) * nzeta[j];
    }
  // the accumulation theta = theta + thtemp*ue as one fused multiply-add
  // per term (what an FMA-contracting Fortran build executes; the CUDA
  // engine uses the same fused operations in the same order)
  int tpos1 = nnode, tpos2 = 2 * nnode;
  for (int j = 0; j < nnode; ++j)
    for (int i = 0; i < span; ++i) {
      theta(i, 0) = std::fma(T(i, j, 0), ue(i, j), theta(i, 0));
      theta(i, 1) = std::fma(T(i, j, 0), ue(i, tpos1 + j), theta(i, 1));
      theta(i, 2) = std::fma(T(i, j, 0), ue(i, tpos2 + j), theta(i, 2));
      theta(i, 3) = std::fma(T(i, j, 1), ue(i, j), theta(i, 3));
      theta(i, 4) = std::fma(T(i, j, 1), ue(i, tpos1 + j), theta(i, 4));
      theta(i, 5) = std::fma(T(i, j, 1), ue(i, tpos2 + j), theta(i, 5));
      theta(i, 6) = std::fma(T(i, j, 2), ue(i, j), theta(i, 6));
      theta(i, 7) = std::fma(T(i, j, 2), ue(i, tpos1 + j), theta(i, 7));
      theta(i, 8) = std::fma(T(i, j, 2), ue(i, tpos2 + j), theta(i, 8));
    }
}

// fcomp1, src/gtmat1.f:601-690: [F] (span, 9 column-major) and det[F].
// Returns the 0-based relative element of the first det <= 1e-20, or -1.
int fcomp1(int span, A2& f, double* df, A2& theta) {
#define F(r, c) f(i, (r - 1) + 3 * (c - 1))
  for (int i = 0; i < span; ++i) {
    F(1, 1) = theta(i, 0) + one; F(1, 2) = theta(i, 3); F(1, 3) = theta(i, 6);
    F(2, 1) = theta(i, 1); F(2, 2) = theta(i, 4) + one; F(2, 3) = theta(i, 7);
    F(3, 1) = theta(i, 2); F(3, 2) = theta(i, 5); F(3, 3) = theta(i, 8) + one;
  }
  int bad = -1;
  for (int i = 0; i < span; ++i) {
    // a*b - c*d as fma(a, b, -(c*d)); the cofactor sum left to right, fused
    double f1 = std::fma(F(2, 2), F(3, 3), -(F(2, 3) * F(3, 2)));
    double f2 = std::fma(F(2, 1), F(3, 3), -(F(2, 3) * F(3, 1)));
    double f3 = std::fma(F(2, 1), F(3, 2), -(F(2, 2) * F(3, 1)));
    df[i] = std::fma(F(1, 3), f3, std::fma(F(1, 1), f1, -(F(1, 2) * f2)));
    if (df[i] <= 1.0e-20 && bad < 0) bad = i;
  }
  return bad;
}

// evcmp1_new, src/gtmat1.f:1134-1210: Cardano eigenvalues of the metric
// tensor, increasing order. c: (span, 6) upper-triangular form.
void evcmp1_new(int span, A2& c, A2& lamda) {
  for (int bel = 0; bel < span; ++bel) {
    double m11 = c(bel, 0), m12 = c(bel, 1), m13 = c(bel, 3);
    double m22 = c(bel, 2), m23 = c(bel, 4), m33 = c(bel, 5);
    // the reference's expressions with each product-sum fused, left to
    // right: a*b + c*d + e*f -> fma(e, f, fma(c, d, a*b)); x - a*b -> fma(-a, b, x)
    double de = m12 * m23;
    double dd = m12 * m12;
    double ee = m23 * m23;
    double ff = m13 * m13;
    double m = m11 + m22 + m33;
    double c1 = std::fma(m22, m33, std::fma(m11, m33, m11 * m22)) - (dd + ee + ff);
    double c0 = std::fma(-(two * m13), de,
                         std::fma(-(m11 * m22), m33, std::fma(m22, ff, std::fma(m11, ee, m33 * dd))));
    double p = std::fma(m, m, -(three * c1));
    double q = std::fma(m, p - onept5 * c1, -(thirteenpt5 * c0));
    double sqrtp = std::sqrt(std::fabs(p));
    double phi = twentyseven * std::fma(quarter * c1 * c1, p - c1, c0 * std::fma(sixpt75, c0, q));
    phi = third * std::atan2(std::sqrt(std::fabs(phi)), q);
    double cphi = sqrtp * std::cos(phi);
    double sphi = iroot3 * sqrtp * std::sin(phi);
    double e2 = third * (m - cphi);
    double e3 = e2 + sphi;
    double e1 = e2 + cphi;
    e2 = e2 - sphi;
    if (e2 < e1) std::swap(e1, e2);
    if (e3 < e1) std::swap(e1, e3);
    if (e3 < e2) std::swap(e2, e3);
    lamda(bel, 0) = e1; lamda(bel, 1) = e2; lamda(bel, 2) = e3;
  }
}

// ivcmp1 + irscp1 + rtcmp1, src/gtmat1.f:691-735, 961-1130: [R] = [F][U]^-1
void rtcmp1(int span, A2& f, double* const* rcol) {
  A2 c(6), cc(6), ev(3);
  // three-term products sums fused left to right: fma(e, f, fma(c, d, a*b))
  auto dot3 = [](double a, double b, double c2_, double d, double e, double f) {
    return std::fma(e, f, std::fma(c2_, d, a * b));
  };
  for (int i = 0; i < span; ++i) {
    c(i, 0) = dot3(F(1, 1), F(1, 1), F(2, 1), F(2, 1), F(3, 1), F(3, 1));
    c(i, 1) = dot3(F(1, 1), F(1, 2), F(2, 1), F(2, 2), F(3, 1), F(3, 2));
    c(i, 2) = dot3(F(1, 2), F(1, 2), F(2, 2), F(2, 2), F(3, 2), F(3, 2));
    c(i, 3) = dot3(F(1, 1), F(1, 3), F(2, 1), F(2, 3), F(3, 1), F(3, 3));
    c(i, 4) = dot3(F(1, 2), F(1, 3), F(2, 2), F(2, 3), F(3, 2), F(3, 3));
    c(i, 5) = dot3(F(1, 3), F(1, 3), F(2, 3), F(2, 3), F(3, 3), F(3, 3));
  }
  for (int i = 0; i < span; ++i) {
    cc(i, 0) = dot3(c(i, 0), c(i, 0), c(i, 1), c(i, 1), c(i, 3), c(i, 3));
    cc(i, 1) = dot3(c(i, 0), c(i, 1), c(i, 1), c(i, 2), c(i, 3), c(i, 4));
    cc(i, 2) = dot3(c(i, 1), c(i, 1), c(i, 2), c(i, 2), c(i, 4), c(i, 4));
    cc(i, 3) = dot3(c(i, 0), c(i, 3), c(i, 1), c(i, 4), c(i, 3), c(i, 5));
    cc(i, 4) = dot3(c(i, 1), c(i, 3), c(i, 2), c(i, 4), c(i, 4), c(i, 5));
    cc(i, 5) = dot3(c(i, 3), c(i, 3), c(i, 4), c(i, 4), c(i, 5), c(i, 5));
  }
  evcmp1_new(span, c, ev);
  for (int i = 0; i < span; ++i) {
    ev(i, 0) = std::sqrt(ev(i, 0)); ev(i, 1) = std::sqrt(ev(i, 1)); ev(i, 2) = std::sqrt(ev(i, 2));
  }
  for (int i = 0; i < span; ++i) {
    double iu = ev(i, 0) + ev(i, 1) + ev(i, 2);
    double iiu = std::fma(ev(i, 0), ev(i, 2), std::fma(ev(i, 1), ev(i, 2), ev(i, 0) * ev(i, 1)));
    double iiiu = ev(i, 0) * ev(i, 1) * ev(i, 2);
    double a2 = one / (iiiu * std::fma(iu, iiu, -iiiu));
    double b2 = std::fma(iu * iiu, iiu, -(iiiu * std::fma(iu, iu, iiu)));
    double c2 = std::fma(-iu, std::fma(iu, iu, -(two * iiu)), -iiiu);
    double d2 = iu;
    double ui[6];
    ui[0] = a2 * std::fma(d2, cc(i, 0), std::fma(c2, c(i, 0), b2));
    ui[1] = a2 * std::fma(d2, cc(i, 1), c2 * c(i, 1));
    ui[2] = a2 * std::fma(d2, cc(i, 2), std::fma(c2, c(i, 2), b2));
    ui[3] = a2 * std::fma(d2, cc(i, 3), c2 * c(i, 3));
    ui[4] = a2 * std::fma(d2, cc(i, 4), c2 * c(i, 4));
    ui[5] = a2 * std::fma(d2, cc(i, 5), std::fma(c2, c(i, 5), b2));
#define RR(a, b) rcol[(a - 1) + 3 * (b - 1)][i]
    RR(1, 1) = dot3(F(1, 1), ui[0], F(1, 2), ui[1], F(1, 3), ui[3]);
    RR(1, 2) = dot3(F(1, 1), ui[1], F(1, 2), ui[2], F(1, 3), ui[4]);
    RR(1, 3) = dot3(F(1, 1), ui[3], F(1, 2), ui[4], F(1, 3), ui[5]);
    RR(2, 1) = dot3(F(2, 1), ui[0], F(2, 2), ui[1], F(2, 3), ui[3]);
    RR(2, 2) = dot3(F(2, 1), ui[1], F(2, 2), ui[2], F(2, 3), ui[4]);
    RR(2, 3) = dot3(F(2, 1), ui[3], F(2, 2), ui[4], F(2, 3), ui[5]);
    RR(3, 1) = dot3(F(3, 1), ui[0], F(3, 2), ui[1], F(3, 3), ui[3]);
    RR(3, 2) = dot3(F(3, 1), ui[1], F(3, 2), ui[2], F(3, 3), ui[4]);
    RR(3, 3) = dot3(F(3, 1), ui[3], F(3, 2), ui[4], F(3, 3), ui[5]);
#undef RR
  }
}
#undef F

// ---------------------------------------------------------------------
// mm01, src/mm01.f
// ---------------------------------------------------------------------
struct MatVecs {  // setup_mm01_rknstr, src/rknstr.f:1018-1054
  double e[MXVL], nu[MXVL], beta[MXVL], h[MXVL], yld[MXVL];
  bool lnelas[MXVL];
};

void mm01_set_history(A2& history, A2& history1, const double* const* cgn, double* cgn8, double* cgn9,
                      const double* sigma_o, const double* hprime, int span) {
  const double root3 = std::sqrt(3.0);
  double dword = state_word(3);
  for (int i = 0; i < span; ++i) {
    double kn = sigma_o[i] / root3;
    history(i, 0) = zero; history(i, 1) = kn; history(i, 2) = zero; history(i, 3) = dword;
    history(i, 4) = hprime[i];
    for (int k = 5; k < 11; ++k) history(i, k) = zero;
    history1(i, 0) = zero; history1(i, 1) = kn; history1(i, 2) = zero; history1(i, 3) = dword;
    history1(i, 4) = hprime[i];
    for (int k = 5; k < 11; ++k) history1(i, k) = zero;
    cgn8[i] = zero; cgn9[i] = zero;
  }
  (void)cgn;
}

// mm01 (src/mm01.f:24-233) with mm01_init (:308-522), mm01_general
// (:776-953), mm01_sig_final (:600-655), mm01_wrapup (:524-598).
// cgn/cgn1: 9 column pointers; deps: 6; rtse: (span, 6).
void mm01(int span, int step, const MatVecs& mv, double* const* cgn, double* const* cgn1,
          double* const* deps, A2& history, A2& history1, A2& rtse) {
  if (step == 1)
    mm01_set_history(history, history1, cgn, cgn[7], cgn[8], mv.yld, mv.h, span);

  // ---- mm01_init
  const double temper_tol = 0.00001, htol = 0.000001;
  const double root3 = std::sqrt(3.0), root2 = std::sqrt(2.0), yld_tol = 0.0000001;
  double shear_mod[MXVL], alpha_n[6][MXVL], lk[MXVL], kbar[MXVL], mrts[MXVL], yf[MXVL];
  double eps_vol_n1[MXVL];
  int instat[MXVL];
  bool yield[MXVL];
  for (int i = 0; i < span; ++i) {
    double deps_vol = deps[0][i] + deps[1][i] + deps[2][i];
    double eps_mean = deps_vol / three;
    double de1 = deps[0][i] - eps_mean;
    double de2 = deps[1][i] - eps_mean;
    double de3 = deps[2][i] - eps_mean;
    double de4 = deps[3][i], de5 = deps[4][i], de6 = deps[5][i];
    double e_n = mv.e[i], nu_n = mv.nu[i];
    double g_n = e_n / two / (one + nu_n);
    double een1 = (cgn[0][i] - nu_n * (cgn[1][i] + cgn[2][i])) / e_n;
    double een2 = (cgn[1][i] - nu_n * (cgn[0][i] + cgn[2][i])) / e_n;
    double een3 = (cgn[2][i] - nu_n * (cgn[0][i] + cgn[1][i])) / e_n;
    double een4 = cgn[3][i] / g_n;
    double een5 = cgn[4][i] / g_n;
    double een6 = cgn[5][i] / g_n;
    eps_vol_n1[i] = een1 + een2 + een3 + deps_vol;
    double eps_mean_n = (een1 + een2 + een3) / three;
    double e1 = (een1 - eps_mean_n) + de1;
    double e2 = (een2 - eps_mean_n) + de2;
    double e3 = (een3 - eps_mean_n) + de3;
    double e4 = een4 + de4, e5 = een5 + de5, e6 = een6 + de6;
    shear_mod[i] = mv.e[i] / (two * (one + mv.nu[i]));
    double d1 = two * shear_mod[i] * e1, d2 = two * shear_mod[i] * e2, d3 = two * shear_mod[i] * e3;
    double d4 = shear_mod[i] * e4, d5 = shear_mod[i] * e5, d6 = shear_mod[i] * e6;
    for (int k = 0; k < 6; ++k) alpha_n[k][i] = history(i, 5 + k);
    double hbari_np1 = mv.beta[i] * mv.h[i];
    double hbark_np1 = (one - mv.beta[i]) * mv.h[i];
    double hbark_n = (one - mv.beta[i]) * history(i, 4);
    kbar[i] = (mv.yld[i] + hbari_np1 * history(i, 2)) / root3;
    lk[i] = one;
    if (std::fabs(hbark_n) > htol) lk[i] = hbark_np1 / hbark_n;
    rtse(i, 0) = d1 - alpha_n[0][i] * lk[i];
    rtse(i, 1) = d2 - alpha_n[1][i] * lk[i];
    rtse(i, 2) = d3 - alpha_n[2][i] * lk[i];
    rtse(i, 3) = d4 - alpha_n[3][i] * lk[i];
    rtse(i, 4) = d5 - alpha_n[4][i] * lk[i];
    rtse(i, 5) = d6 - alpha_n[5][i] * lk[i];
    mrts[i] = std::sqrt(rtse(i, 0) * rtse(i, 0) + rtse(i, 1) * rtse(i, 1) + rtse(i, 2) * rtse(i, 2) +
                        two * (rtse(i, 3) * rtse(i, 3) + rtse(i, 4) * rtse(i, 4) + rtse(i, 5) * rtse(i, 5)));
    yf[i] = mrts[i] - root2 * kbar[i];
    rtse(i, 0) = d1 - alpha_n[0][i];
    rtse(i, 1) = d2 - alpha_n[1][i];
    rtse(i, 2) = d3 - alpha_n[2][i];
    rtse(i, 3) = d4 - alpha_n[3][i];
    rtse(i, 4) = d5 - alpha_n[4][i];
    rtse(i, 5) = d6 - alpha_n[5][i];
    mrts[i] = std::sqrt(rtse(i, 0) * rtse(i, 0) + rtse(i, 1) * rtse(i, 1) + rtse(i, 2) * rtse(i, 2) +
                        two * (rtse(i, 3) * rtse(i, 3) + rtse(i, 4) * rtse(i, 4) + rtse(i, 5) * rtse(i, 5)));
    (void)temper_tol;
    instat[i] = 3;
    yield[i] = false;
    if (mv.lnelas[i]) continue;
    if (yf[i] >= yld_tol * root2 * kbar[i]) { yield[i] = true; instat[i] = 1; }
  }

  // ---- mm01_general
  double devstr_n1[6][MXVL];
  {
    const double root2c = 1.414213562373095, twthrd = 0.666666666666667, root23 = 0.816496580927,
                 four = 4.0, root2o3 = 0.4714045207910;
    // qroot1/qroot2 keep their values from the previous yielding element
    // of the loop (src/mm01.f:863-881 reads them again after a negative
    // discriminant); zero before the first.
    double qroot1 = zero, qroot2 = zero;
    for (int i = 0; i < span; ++i) {
      if (!yield[i]) continue;
      double hbari_np1 = mv.beta[i] * mv.h[i];
      double hbark_np1 = (one - mv.beta[i]) * mv.h[i];
      double a = (two * shear_mod[i] + twthrd * hbark_np1) / mrts[i];
      double b = one - lk[i];
      double d = root2o3 * hbari_np1;
      double vbar = mrts[i] * mrts[i];
      // the shear term uses history(1,11): element 1 of the block
      // (src/mm01.f:843-845)
      double wbar = history(i, 5) * history(i, 5) + history(i, 6) * history(i, 6) +
                    history(i, 7) * history(i, 7) +
                    two * (history(i, 8) * history(i, 8) + history(i, 9) * history(i, 9) +
                           history(0, 10) * history(0, 10));
      double vwbar = rtse(i, 0) * history(i, 5) + rtse(i, 1) * history(i, 6) + rtse(i, 2) * history(i, 7) +
                     two * (rtse(i, 3) * history(i, 8) + rtse(i, 4) * history(i, 9) +
                            rtse(i, 5) * history(i, 10));
      double t1 = a * a * vbar - two * d * d;
      double t2 = -four * d * kbar[i] - two * a * vbar - two * a * b * vwbar;
      double t3 = b * b * wbar + two * b * vwbar + vbar - two * kbar[i] * kbar[i];
      double discr = t2 * t2 - four * t1 * t3;
      if (!(discr < zero)) {
        qroot1 = (-t2 + std::sqrt(discr)) / (two * t1);
        qroot2 = (-t2 - std::sqrt(discr)) / (two * t1);
      }
      double lambda_deltat = std::min(qroot1, qroot2);
      history1(i, 0) = lambda_deltat;
      history1(i, 1) = kbar[i] + (root2c / three) * hbari_np1 * lambda_deltat;
      history1(i, 2) = history(i, 2) + lambda_deltat * root23;
      history1(i, 4) = mv.h[i];
      double const1 = twthrd * hbark_np1 * lambda_deltat / mrts[i];
      double const2 = one - lambda_deltat * (twthrd * hbark_np1 + two * shear_mod[i]) / mrts[i];
      b = one - lk[i];
      for (int k = 0; k < 6; ++k) history1(i, 5 + k) = lk[i] * history(i, 5 + k) + const1 * rtse(i, k);
      for (int k = 0; k < 6; ++k)
        devstr_n1[k][i] = history1(i, 5 + k) + b * history(i, 5 + k) + const2 * rtse(i, k);
    }
  }
  // ---- linear elastic points (src/mm01.f:194-203)
  for (int i = 0; i < span; ++i) {
    if (yield[i]) continue;
    history1(i, 0) = zero;
    history1(i, 1) = kbar[i];
    if (mv.lnelas[i]) history1(i, 1) = zero;
    history1(i, 2) = history(i, 2);
    history1(i, 4) = mv.h[i];
    for (int k = 0; k < 6; ++k) history1(i, 5 + k) = alpha_n[k][i] * lk[i];
    for (int k = 0; k < 6; ++k) devstr_n1[k][i] = rtse(i, k) + alpha_n[k][i];
  }
  // ---- mm01_sig_final
  for (int i = 0; i < span; ++i) {
    double ym = mv.e[i], nu = mv.nu[i];
    double sig_mean_np1 =
        eps_vol_n1[i] * (three * ym * nu / ((one + nu) * (one - two * nu)) + two * shear_mod[i]) / three;
    cgn1[0][i] = devstr_n1[0][i] + sig_mean_np1;
    cgn1[1][i] = devstr_n1[1][i] + sig_mean_np1;
    cgn1[2][i] = devstr_n1[2][i] + sig_mean_np1;
    cgn1[3][i] = devstr_n1[3][i];
    cgn1[4][i] = devstr_n1[4][i];
    cgn1[5][i] = devstr_n1[5][i];
    cgn1[6][i] = cgn[6][i] + half * (deps[0][i] * (cgn1[0][i] + cgn[0][i]) +
                                     deps[1][i] * (cgn1[1][i] + cgn[1][i]) +
                                     deps[2][i] * (cgn1[2][i] + cgn[2][i]) +
                                     deps[3][i] * (cgn1[3][i] + cgn[3][i]) +
                                     deps[4][i] * (cgn1[4][i] + cgn[4][i]) +
                                     deps[5][i] * (cgn1[5][i] + cgn[5][i]));
    history1(i, 3) = state_word(instat[i]);
  }
  // ---- mm01_wrapup (eps_elas is not used by the hot path)
  {
    const double six = 6.0, root2w = std::sqrt(2.0);
    for (int i = 0; i < span; ++i) {
      cgn1[7][i] = cgn[7][i];
      cgn1[8][i] = cgn[8][i];
      if (!yield[i]) continue;
      double s[6];
      for (int k = 0; k < 6; ++k) s[k] = cgn[k][i];
      double sbar_n = std::sqrt((s[0] - s[1]) * (s[0] - s[1]) + (s[1] - s[2]) * (s[1] - s[2]) +
                                (s[0] - s[2]) * (s[0] - s[2]) +
                                six * (s[3] * s[3] + s[4] * s[4] + s[5] * s[5])) / root2w;
      for (int k = 0; k < 6; ++k) s[k] = cgn1[k][i];
      double sbar_n1 = std::sqrt((s[0] - s[1]) * (s[0] - s[1]) + (s[1] - s[2]) * (s[1] - s[2]) +
                                 (s[0] - s[2]) * (s[0] - s[2]) +
                                 six * (s[3] * s[3] + s[4] * s[4] + s[5] * s[5])) / root2w;
      double depbar = history1(i, 2) - history(i, 2);
      cgn1[7][i] = cgn[7][i] + half * (sbar_n1 + sbar_n) * depbar;
      cgn1[8][i] = cgn[8][i] + depbar;
    }
  }
}

// cnst1, src/mm01.f:1196-1348. cep (span, 36): (r, c) -> (r-1) + 6(c-1)
void cnst1(int span, A2& cep, A2& rtsg, const MatVecs& mv, const double* kn1, const double* hprime,
           const double* ldt, const double* dstates) {
  const double root2 = 1.414213562;
  for (int i = 0; i < span; ++i) {
#define C(a, b) cep(i, (a - 1) + 6 * (b - 1))
    bool yield = state_of(dstates[i]) == 1;
    double nu = mv.nu[i], e = mv.e[i];
    if (!yield) {
      for (int k = 0; k < 36; ++k) cep(i, k) = zero;
      double c1 = (e / ((one + nu) * (one - two * nu)));
      double c2 = (one - nu) * c1;
      double c3 = ((one - two * nu) / two) * c1;
      double c4 = nu * c1;
      C(1, 1) = c2; C(2, 2) = c2; C(3, 3) = c2;
      C(4, 4) = c3; C(5, 5) = c3; C(6, 6) = c3;
      C(1, 2) = c4; C(1, 3) = c4; C(2, 1) = c4; C(3, 1) = c4; C(2, 3) = c4; C(3, 2) = c4;
      continue;
    }
    double g = e / (two * (one + nu));
    double l = (e * nu) / ((one + nu) * (one - two * nu));
    double k = (three * l + two * g) / three;
    double r1 = rtsg(i, 0), r2 = rtsg(i, 1), r3 = rtsg(i, 2), r4 = rtsg(i, 3), r5 = rtsg(i, 4), r6 = rtsg(i, 5);
    double mrtsq = r1 * r1 + r2 * r2 + r3 * r3 + two * (r4 * r4 + r5 * r5 + r6 * r6);
    double bb = (root2 * kn1[i] + (two / three) * (one - mv.beta[i]) * hprime[i] * ldt[i]) / std::sqrt(mrtsq);
    double gamma = one / (one + hprime[i] / (three * g));
    double gambar = gamma - one + bb;
    double gbar = g * bb;
    double albar = k - two * gbar / three;
    double thbar = two * g * gambar;
    C(1, 1) = (albar + two * gbar - thbar * (r1 * r1) / mrtsq);
    C(2, 2) = (albar + two * gbar - thbar * (r2 * r2) / mrtsq);
    C(3, 3) = (albar + two * gbar - thbar * (r3 * r3) / mrtsq);
    C(4, 4) = (gbar - thbar * (r4 * r4) / mrtsq);
    C(5, 5) = (gbar - thbar * (r5 * r5) / mrtsq);
    C(6, 6) = (gbar - thbar * (r6 * r6) / mrtsq);
    C(2, 1) = (albar - thbar * r1 * r2 / mrtsq);
    C(3, 1) = (albar - thbar * r1 * r3 / mrtsq);
    C(4, 1) = -(thbar * r1 * r4 / mrtsq);
    C(5, 1) = -(thbar * r1 * r5 / mrtsq);
    C(6, 1) = -(thbar * r1 * r6 / mrtsq);
    C(3, 2) = (albar - thbar * r3 * r2 / mrtsq);
    C(4, 2) = -(thbar * r2 * r4 / mrtsq);
    C(5, 2) = -(thbar * r2 * r5 / mrtsq);
    C(6, 2) = -(thbar * r2 * r6 / mrtsq);
    C(4, 3) = -(thbar * r3 * r4 / mrtsq);
    C(5, 3) = -(thbar * r3 * r5 / mrtsq);
    C(6, 3) = -(thbar * r3 * r6 / mrtsq);
    C(5, 4) = -(thbar * r4 * r5 / mrtsq);
    C(6, 4) = -(thbar * r4 * r6 / mrtsq);
    C(6, 5) = -(thbar * r5 * r6 / mrtsq);
    C(1, 2) = C(2, 1); C(1, 3) = C(3, 1); C(1, 4) = C(4, 1); C(1, 5) = C(5, 1); C(1, 6) = C(6, 1);
    C(2, 3) = C(3, 2); C(2, 4) = C(4, 2); C(2, 5) = C(5, 2); C(2, 6) = C(6, 2);
    C(3, 4) = C(4, 3); C(3, 5) = C(5, 3); C(3, 6) = C(6, 3);
    C(4, 5) = C(5, 4); C(4, 6) = C(6, 4); C(5, 6) = C(6, 5);
#undef C
  }
}

// lower-triangle packing of [D], src/rstgp1.f:5370-5397
const int kLowerR[21] = {1, 2, 2, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 5, 6, 6, 6, 6, 6, 6};
const int kLowerC[21] = {1, 1, 2, 1, 2, 3, 1, 2, 3, 4, 1, 2, 3, 4, 5, 1, 2, 3, 4, 5, 6};

// ---------------------------------------------------------------------
// recovery for one block: do_nleps_block, src/drive_eps_sig_internal_forces.f:399-703
// ---------------------------------------------------------------------
struct RecOut {
  int status = 0; int bad_elem = 0;
  double energy = 0.0, plastic = 0.0;
};

RecOut recover_block(const w3g_model_desc* m, const w3g_block_state* s, const Blk& B, int step, int iter,
                     bool extrapolated_du, const double* c, const double* u, const double* du) {
  RecOut out;
  const int span = B.span, nnode = B.nnode, ngp = B.ngp, totdof = B.totdof;
  const int* edest = m->edest[B.blk];
  const int* cdest = m->cdest[B.blk];
  const int hist = hist_size(B.mat_type);
  const bool crystal = B.mat_type == W3G_MAT_CRYSTAL;
  const bool umat = B.mat_type == W3G_MAT_UMAT;

  // dupstr: element displacements (src/drive_eps_sig_internal_forces.f:560)
  A2 ue(totdof), due(totdof);
  for (int j = 0; j < totdof; ++j)
    for (int i = 0; i < span; ++i) {
      ue(i, j) = u[edest[(size_t)i * totdof + j] - 1];
      due(i, j) = du[edest[(size_t)i * totdof + j] - 1];
    }
  // dupstr_blocked: coordinates (:1699-1754)
  A2 ce0(totdof), cen(totdof), cemid(totdof), cen1(totdof);
  for (int k = 0; k < totdof; ++k)
    for (int i = 0; i < span; ++i) ce0(i, k) = c[cdest[(size_t)i * totdof + k] - 1];
  bool update = !(step == 1 && iter == 0);
  bool update_coords = B.geonl && update;
  for (int j = 0; j < totdof; ++j)
    for (int i = 0; i < span; ++i) {
      if (update_coords) {
        cen(i, j) = ce0(i, j) + ue(i, j);
        cemid(i, j) = ce0(i, j) + ue(i, j) + half * due(i, j);
        cen1(i, j) = ce0(i, j) + ue(i, j) + due(i, j);
      } else {
        cen(i, j) = ce0(i, j); cemid(i, j) = ce0(i, j); cen1(i, j) = ce0(i, j);
      }
    }
  // gather state at n: history (hist, ngp, span) -> (span, hist, ngp)
  std::vector<A2> ehist(ngp, A2(hist)), ehist1(ngp, A2(hist));
  std::vector<A2> ddtse(ngp, A2(NSTR)), urcs_n(ngp, A2(NSTRS)), urcs_n1(ngp, A2(NSTRS));
  std::vector<A2> rot(ngp, A2(9)), rtse(ngp, A2(NSTR));
  for (int g = 0; g < ngp; ++g)
    for (int i = 0; i < span; ++i) {
      const double* h = s->history[B.blk] + ((size_t)i * ngp + g) * hist;
      for (int k = 0; k < hist; ++k) ehist[g](i, k) = h[k];
      const double* ep = s->eps_n[B.blk] + ((size_t)i * ngp + g) * NSTR;
      for (int k = 0; k < NSTR; ++k) ddtse[g](i, k) = ep[k];
      const double* up = s->urcs_n[B.blk] + ((size_t)i * ngp + g) * NSTRS;
      for (int k = 0; k < NSTRS; ++k) urcs_n[g](i, k) = up[k];
    }
  // setup_mm01_rknstr (src/rknstr.f:1018-1054): float props -> double
  MatVecs mv;
  for (int i = 0; i < span; ++i) {
    const float* p = m->props + (size_t)(B.felem - 1 + i) * MXELPR;
    const int* lp = m->lprops + (size_t)(B.felem - 1 + i) * MXELPR;
    mv.e[i] = p[6]; mv.nu[i] = p[7]; mv.beta[i] = p[13]; mv.h[i] = p[14];
    mv.lnelas[i] = flog(lp[16]); mv.yld[i] = p[22];
  }

  // rknstr_geonl (src/rknstr.f:455-540): [J] at the mid-step
  // configuration; rknstr_sm_displ (:555-610): [J] at t = 0. For 8-node
  // bricks with b-bar, the mean-dilatation terms of that configuration
  // (vol_terms per Gauss point, then vol_avg).
  const bool bbar = B.bbar && B.etype == W3G_ETYPE_L3DISOP;
  std::vector<double> nxi((size_t)ngp * nnode), neta((size_t)ngp * nnode), nzeta((size_t)ngp * nnode),
      weights(ngp);
  std::vector<std::vector<double>> det_j_mid(ngp, std::vector<double>(MXVL));
  std::vector<A2> gama_mid(ngp, A2(9));
  A2 vol(24);
  std::vector<double> volume(MXVL, zero);
  for (int g = 0; g < ngp; ++g) {
    double xi, eta, zeta;
    getgpts(B.etype, B.order, g + 1, xi, eta, zeta, weights[g]);
    derivs(B.etype, xi, eta, zeta, &nxi[g * nnode], &neta[g * nnode], &nzeta[g * nnode]);
    if (B.geonl)
      jacob1(span, nnode, &nxi[g * nnode], &neta[g * nnode], &nzeta[g * nnode], cemid,
             det_j_mid[g].data(), gama_mid[g]);
    else
      jacob1(span, nnode, &nxi[g * nnode], &neta[g * nnode], &nzeta[g * nnode], ce0,
             det_j_mid[g].data(), gama_mid[g]);
    if (bbar)
      vol_terms(span, gama_mid[g], det_j_mid[g].data(), vol, &nxi[g * nnode], &neta[g * nnode],
                &nzeta[g * nnode], volume.data());
  }
  if (bbar) vol_avg(span, vol, volume.data());

  std::vector<std::vector<double>> det_j(ngp, std::vector<double>(MXVL));
  std::vector<A2> gama(ngp, A2(9));
  A2 uenh(totdof), uen1(totdof);
  A2 b(totdof * 6);
  double internal_energy = 0.0, plastic_work = 0.0;
  std::vector<double> dfn1_all((size_t)ngp * MXVL);

  for (int g = 0; g < ngp; ++g) {
    // ---- rstgp1 (src/rstgp1.f:19-332) for geonl blocks, rstgp2
    // (:351-598) for small-displacement blocks
    A2 ddt(NSTR), uddt(NSTR);
    A2 theta(9), fn1(9), fnh(9), qnhalf(36);
    double dfn1[MXVL], dfh[MXVL];
    A2 rnh(9);
    if (B.geonl) {
      // rstgp1_a
      for (int j = 0; j < totdof; ++j)
        for (int i = 0; i < span; ++i) {
          uenh(i, j) = ue(i, j) + half * due(i, j);
          uen1(i, j) = ue(i, j) + due(i, j);
        }
      // gtmat1 (src/gtmat1.f:17-190)
      jacob1(span, nnode, &nxi[g * nnode], &neta[g * nnode], &nzeta[g * nnode], ce0, det_j[g].data(), gama[g]);
      tcomp1(span, theta, &nxi[g * nnode], &neta[g * nnode], &nzeta[g * nnode], gama[g], uen1, nnode);
      int bad = fcomp1(span, fn1, dfn1, theta);
      if (bad >= 0) { out.status = W3G_STEP_CUT; out.bad_elem = B.felem + bad; return out; }
      {
        double* rc[9];
        for (int k = 0; k < 9; ++k) rc[k] = rot[g].col(k);
        rtcmp1(span, fn1, rc);
      }
      tcomp1(span, theta, &nxi[g * nnode], &neta[g * nnode], &nzeta[g * nnode], gama[g], uenh, nnode);
      bad = fcomp1(span, fnh, dfh, theta);
      if (bad >= 0) { out.status = W3G_STEP_CUT; out.bad_elem = B.felem + bad; return out; }
      {
        double* rc[9];
        for (int k = 0; k < 9; ++k) rc[k] = rnh.col(k);
        rtcmp1(span, fnh, rc);
        const double* rcc[9];
        for (int k = 0; k < 9; ++k) rcc[k] = rnh.col(k);
        getrm1(span, qnhalf, rcc, 1);
      }
      for (int i = 0; i < span; ++i) dfn1_all[(size_t)g * MXVL + i] = dfn1[i];
    } else {
      // rstgp2: det[J] of rknstr_sm_displ; drive_10_update sets the
      // rotations of small-displacement blocks to identity (rstgp1.f:4415-4432)
      for (int i = 0; i < span; ++i) {
        det_j[g][i] = det_j_mid[g][i];
        for (int k = 0; k < 9; ++k) rot[g](i, k) = (k % 4 == 0) ? one : zero;
      }
    }
    // gtlsn1 (src/gtlsn1.f:25-85), with bmod for b-bar
    b.zero();
    blcmp1(span, b, totdof, gama_mid[g], &nxi[g * nnode], &neta[g * nnode], &nzeta[g * nnode], nnode);
    if (bbar) bmod(span, b, totdof, vol, m->eps_bbar);
    ddt.zero();
    {
      int bpos1 = nnode, bpos2 = 2 * nnode;
#define BB(i, j, k) b(i, (j) + totdof * (k))
      for (int j = 0; j < nnode; ++j)
        for (int i = 0; i < span; ++i) {
          ddt(i, 0) = ddt(i, 0) + BB(i, j, 0) * due(i, j) + BB(i, bpos1 + j, 0) * due(i, bpos1 + j) +
                      BB(i, bpos2 + j, 0) * due(i, bpos2 + j);
          ddt(i, 1) = ddt(i, 1) + BB(i, j, 1) * due(i, j) + BB(i, bpos1 + j, 1) * due(i, bpos1 + j) +
                      BB(i, bpos2 + j, 1) * due(i, bpos2 + j);
          ddt(i, 2) = ddt(i, 2) + BB(i, j, 2) * due(i, j) + BB(i, bpos1 + j, 2) * due(i, bpos1 + j) +
                      BB(i, bpos2 + j, 2) * due(i, bpos2 + j);
          ddt(i, 3) = ddt(i, 3) + BB(i, j, 3) * due(i, j) + BB(i, bpos1 + j, 3) * due(i, bpos1 + j);
          ddt(i, 4) = ddt(i, 4) + BB(i, bpos1 + j, 4) * due(i, bpos1 + j) + BB(i, bpos2 + j, 4) * due(i, bpos2 + j);
          ddt(i, 5) = ddt(i, 5) + BB(i, j, 5) * due(i, j) + BB(i, bpos2 + j, 5) * due(i, bpos2 + j);
        }
#undef BB
    }
    // qmply1 (geonl: unrotated increment; rstgp2 takes ddt as it is) +
    // rstgp1_update_strains
    {
      if (B.geonl) {
        const double* m1[6]; double* m2[6];
        for (int k = 0; k < 6; ++k) { m1[k] = ddt.col(k); m2[k] = uddt.col(k); }
        qmply1(span, qnhalf, m1, m2);
      } else {
        for (int k = 0; k < 6; ++k)
          for (int i = 0; i < span; ++i) uddt(i, k) = ddt(i, k);
      }
      for (int i = 0; i < span; ++i)
        for (int k = 0; k < 6; ++k) ddtse[g](i, k) = ddtse[g](i, k) + uddt(i, k);
    }
    // drive_01_update (src/rstgp1.f:614-1034)
    A2 cep(36);
    cep.zero();
    bool nonlinear_update = iter >= 1 || extrapolated_du;
    double* cgn[9]; double* cgn1[9]; double* dep[6];
    for (int k = 0; k < 9; ++k) { cgn[k] = urcs_n[g].col(k); cgn1[k] = urcs_n1[g].col(k); }
    for (int k = 0; k < 6; ++k) dep[k] = uddt.col(k);
    if (crystal) {
      // drive_10_update (src/rstgp1.f:4327-4510): mm10 per element; the
      // consistent [D] goes to history(1:36), cep_blocks is not written
      for (int i = 0; i < span; ++i) {
        w3o::CrystalProps cp;
        const int e = B.felem - 1 + i;
        w3o::mm10_element_props(m->crystals[m->elem_crystal[e]], m->elem_angles + 3 * (size_t)e, cp);
        cp.asymmetric = m->asymmetric_assembly;
        double hn[MM10_HIST], hn1[MM10_HIST], un[9], un1[9], dd[6], rr[9];
        for (int k = 0; k < MM10_HIST; ++k) { hn[k] = ehist[g](i, k); hn1[k] = ehist1[g](i, k); }
        for (int k = 0; k < 9; ++k) { un[k] = urcs_n[g](i, k); un1[k] = zero; rr[k] = rot[g](i, k); }
        for (int k = 0; k < 6; ++k) dd[k] = uddt(i, k);
        int st = w3o::mm10_point(cp, step, iter, extrapolated_du, m->dt, e + 1, g + 1, hn, hn1, un, un1, dd, rr);
        if (st != 0) { out.status = W3G_LOCAL_FAIL; out.bad_elem = e + 1; return out; }
        for (int k = 0; k < MM10_HIST; ++k) ehist1[g](i, k) = hn1[k];
        for (int k = 0; k < 9; ++k) urcs_n1[g](i, k) = un1[k];
      }
    } else if (umat) {
      // drive_umat_update (src/rstgp1.f:3476-4010); the [D] goes to cep
      // already symmetrised (rstgp1_make_symmetric_store)
      for (int i = 0; i < span; ++i) {
        const int e = B.felem - 1 + i;
        double hn[w3o::UMAT_NSTATV], hn1[w3o::UMAT_NSTATV], un[9], un1[9], en[6], dd[6], c21[21];
        for (int k = 0; k < w3o::UMAT_NSTATV; ++k) { hn[k] = ehist[g](i, k); hn1[k] = ehist1[g](i, k); }
        for (int k = 0; k < 9; ++k) un[k] = urcs_n[g](i, k);
        const double* epn = s->eps_n[B.blk] + ((size_t)i * ngp + g) * NSTR;
        for (int k = 0; k < 6; ++k) { en[k] = epn[k]; dd[k] = uddt(i, k); }
        const bool cut = w3o::umat_drive(m->umat_props + (size_t)e * w3o::UMAT_NPROPS, step, iter, extrapolated_du,
                                         un, en, dd, hn, w3o::UMAT_NSTATV, un1, hn1, c21);
        if (cut) { out.status = W3G_LOCAL_FAIL; out.bad_elem = e + 1; return out; }
        for (int k = 0; k < w3o::UMAT_NSTATV; ++k) ehist1[g](i, k) = hn1[k];
        for (int k = 0; k < 9; ++k) urcs_n1[g](i, k) = un1[k];
        for (int k = 0; k < 21; ++k) {
          const int r = kLowerR[k] - 1, c = kLowerC[k] - 1;
          cep(i, r + 6 * c) = c21[k];
          cep(i, c + 6 * r) = c21[k];
        }
      }
    } else if (nonlinear_update) {
      mm01(span, step, mv, cgn, cgn1, dep, ehist[g], ehist1[g], rtse[g]);
      cnst1(span, cep, rtse[g], mv, ehist1[g].col(1), ehist1[g].col(4), ehist1[g].col(0), ehist1[g].col(3));
    } else {
      // drive_01_update_a / _b (src/rstgp1.f:942-1034)
      for (int i = 0; i < span; ++i) {
        double e = mv.e[i], nu = mv.nu[i];
        double c1 = (e / ((one + nu) * (one - two * nu)));
        double c2 = (one - nu) * c1;
        double c3 = ((one - two * nu) / two) * c1;
        double c4 = nu * c1;
#define C(a, bq) cep(i, (a - 1) + 6 * (bq - 1))
        C(1, 1) = c2; C(2, 2) = c2; C(3, 3) = c2; C(4, 4) = c3; C(5, 5) = c3; C(6, 6) = c3;
        C(1, 2) = c4; C(1, 3) = c4; C(2, 1) = c4; C(3, 1) = c4; C(2, 3) = c4; C(3, 2) = c4;
#undef C
      }
      for (int i = 0; i < span; ++i)
        for (int k = 0; k < 6; ++k) cgn1[k][i] = cgn[k][i];
      for (int k = 0; k < 6; ++k)
        for (int mm = 0; mm < 6; ++mm)
          for (int i = 0; i < span; ++i)
            cgn1[k][i] = cgn1[k][i] + cep(i, mm + 6 * k) * dep[mm][i];
    }
    // rstgp1_store_cep (src/rstgp1.f:5360-5397): (21, span, ngp)
    if (!crystal) {
      double* gc = s->cep[B.blk];
      for (int i = 0; i < span; ++i)
        for (int k = 0; k < 21; ++k)
          gc[((size_t)g * span + i) * 21 + k] = cep(i, (kLowerR[k] - 1) + 6 * (kLowerC[k] - 1));
    }
    // rstgp1_b (src/rstgp1.f:5189-5241): large-strain (itype 1) or
    // small-strain (itype 2) branch
    if (iter != 0) {
      for (int i = 0; i < span; ++i) {
        double factor = B.geonl ? dfn1[i] * det_j[g][i] * m->beta_fact * weights[g]
                                : det_j[g][i] * m->beta_fact * weights[g];
        internal_energy = internal_energy + urcs_n1[g](i, 6) * factor;
        plastic_work = plastic_work + urcs_n1[g](i, 7) * factor;
      }
    }
  }
  out.energy = internal_energy;
  out.plastic = plastic_work;

  // rplstr (src/rplstr.f:15-90)
  for (int g = 0; g < ngp; ++g)
    for (int i = 0; i < span; ++i) {
      double* up = s->urcs_n1[B.blk] + ((size_t)i * ngp + g) * NSTRS;
      for (int k = 0; k < NSTRS; ++k) up[k] = urcs_n1[g](i, k);
      double* ep = s->eps_n1[B.blk] + ((size_t)i * ngp + g) * NSTR;
      for (int k = 0; k < NSTR; ++k) ep[k] = ddtse[g](i, k);
      if (iter > 0 && B.geonl) {
        double* rp = s->rot_n1[B.blk] + ((size_t)i * ngp + g) * 9;
        for (int k = 0; k < 9; ++k) rp[k] = rot[g](i, k);
      }
      if (iter > 0 || crystal) {   // rplstr: mm10 history at every iteration
        double* hp = s->history1[B.blk] + ((size_t)i * ngp + g) * hist;
        for (int k = 0; k < hist; ++k) hp[k] = ehist1[g](i, k);
      }
    }

  // rknifv / rknifv_std / gpifv1 (src/rknifv.f:15-217, src/gpifv1.f:16-154)
  A2 eleifv(totdof);
  eleifv.zero();
  double elem_vol[MXVL];
  for (int i = 0; i < span; ++i) elem_vol[i] = zero;
  if (bbar) {
    vol.zero();
    for (int i = 0; i < span; ++i) volume[i] = zero;
  }
  for (int g = 0; g < ngp; ++g) {
    jacob1(span, nnode, &nxi[g * nnode], &neta[g * nnode], &nzeta[g * nnode], cen1, det_j[g].data(), gama[g]);
    if (bbar)
      vol_terms(span, gama[g], det_j[g].data(), vol, &nxi[g * nnode], &neta[g * nnode], &nzeta[g * nnode],
                volume.data());
  }
  if (bbar) vol_avg(span, vol, volume.data());
  for (int g = 0; g < ngp; ++g) {
    double w = weights[g] * adjust_scalar(B.etype);   // gpifv1.f:43-47
    b.zero();
    blcmp1(span, b, totdof, gama[g], &nxi[g * nnode], &neta[g * nnode], &nzeta[g * nnode], nnode);
    if (bbar) bmod(span, b, totdof, vol, m->eps_bbar);
    const double* dj = det_j[g].data();
    if (B.geonl) {
      A2 qtn1(36), cs(6);
      const double* rc[9];
      for (int k = 0; k < 9; ++k) rc[k] = rot[g].col(k);
      getrm1(span, qtn1, rc, 2);
      const double* m1[6]; double* m2[6];
      for (int k = 0; k < 6; ++k) { m1[k] = urcs_n1[g].col(k); m2[k] = cs.col(k); }
      qmply1(span, qtn1, m1, m2);
      for (int j = 0; j < totdof; ++j)
        for (int i = 0; i < span; ++i)
          eleifv(i, j) = eleifv(i, j) + b(i, j + totdof * 0) * cs(i, 0) * w * dj[i] +
                         b(i, j + totdof * 1) * cs(i, 1) * w * dj[i] + b(i, j + totdof * 2) * cs(i, 2) * w * dj[i] +
                         b(i, j + totdof * 3) * cs(i, 3) * w * dj[i] + b(i, j + totdof * 4) * cs(i, 4) * w * dj[i] +
                         b(i, j + totdof * 5) * cs(i, 5) * w * dj[i];
    } else {
      for (int j = 0; j < totdof; ++j)
        for (int i = 0; i < span; ++i)
          eleifv(i, j) = eleifv(i, j) + b(i, j + totdof * 0) * urcs_n1[g](i, 0) * w * dj[i] +
                         b(i, j + totdof * 1) * urcs_n1[g](i, 1) * w * dj[i] +
                         b(i, j + totdof * 2) * urcs_n1[g](i, 2) * w * dj[i] +
                         b(i, j + totdof * 3) * urcs_n1[g](i, 3) * w * dj[i] +
                         b(i, j + totdof * 4) * urcs_n1[g](i, 4) * w * dj[i] +
                         b(i, j + totdof * 5) * urcs_n1[g](i, 5) * w * dj[i];
    }
    for (int i = 0; i < span; ++i) elem_vol[i] = elem_vol[i] + w * dj[i];
  }
  double* ev = s->einfvec[B.blk];
  for (int j = 0; j < totdof; ++j)
    for (int i = 0; i < span; ++i) ev[(size_t)j * span + i] = eleifv(i, j);
  if (s->element_vol && s->element_vol[B.blk])
    for (int i = 0; i < span; ++i) s->element_vol[B.blk][i] = elem_vol[i];
  return out;
}

// ---------------------------------------------------------------------
// tangent for one block: do_nlek_block + rktstf + gptns1
// (src/tanstf.f:119-328, src/rktstf.f:15-221, src/gptns1.f:16-341)
// ---------------------------------------------------------------------
int tangent_block(const w3g_model_desc* m, const w3g_block_state* s, const Blk& B, const double* c,
                  const double* u, const double* du, double* estiff) {
  const int span = B.span, nnode = B.nnode, ngp = B.ngp, totdof = B.totdof, utsz = B.utsz;
  // asymmetric assembly: full element matrices, ek_full(span, totdof**2)
  // column-major (tanstf.f:223-225, gptns1.f:241-246 bdbt_asym)
  const bool asym = m->asymmetric_assembly != 0;
  const int nrow = asym ? totdof * totdof : utsz;
  const int* edest = m->edest[B.blk];
  const int* cdest = m->cdest[B.blk];
  for (size_t k = 0; k < (size_t)nrow * span; ++k) estiff[k] = zero;

  // dptstf (src/dptstf.f:86-156)
  A2 ce(totdof), ue(totdof), due(totdof);
  for (int k = 0; k < totdof; ++k)
    for (int i = 0; i < span; ++i) ce(i, k) = c[cdest[(size_t)i * totdof + k] - 1];
  if (B.geonl) {
    for (int j = 0; j < totdof; ++j)
      for (int i = 0; i < span; ++i) {
        ue(i, j) = u[edest[(size_t)i * totdof + j] - 1];
        due(i, j) = du[edest[(size_t)i * totdof + j] - 1];
      }
    for (int j = 0; j < totdof; ++j)
      for (int i = 0; i < span; ++i) ce(i, j) = ce(i, j) + ue(i, j) + due(i, j);
  }
  // dptstf_blocks / tanstf_gastr (src/tanstf.f:642-707, :1138-1180)
  std::vector<A2> rot(ngp, A2(9)), urcs(ngp, A2(NSTRS));
  for (int g = 0; g < ngp; ++g)
    for (int i = 0; i < span; ++i) {
      if (B.geonl) {
        const double* rp = s->rot_n1[B.blk] + ((size_t)i * ngp + g) * 9;
        for (int k = 0; k < 9; ++k) rot[g](i, k) = rp[k];
      }
      const double* up = s->urcs_n1[B.blk] + ((size_t)i * ngp + g) * NSTRS;
      for (int k = 0; k < NSTRS; ++k) urcs[g](i, k) = up[k];
    }
  // rktstf GP loop 1 (src/rktstf.f:98-145), with the b-bar volume terms
  // of the configuration at n+1 (geonl) or t = 0
  const bool bbar = B.bbar && B.etype == W3G_ETYPE_L3DISOP;
  std::vector<double> nxi((size_t)ngp * nnode), neta((size_t)ngp * nnode), nzeta((size_t)ngp * nnode),
      weights(ngp);
  std::vector<std::vector<double>> dj(ngp, std::vector<double>(MXVL));
  std::vector<A2> gama(ngp, A2(9));
  A2 vol(24);
  std::vector<double> volume(MXVL, zero);
  for (int g = 0; g < ngp; ++g) {
    double xi, eta, zeta;
    getgpts(B.etype, B.order, g + 1, xi, eta, zeta, weights[g]);
    derivs(B.etype, xi, eta, zeta, &nxi[g * nnode], &neta[g * nnode], &nzeta[g * nnode]);
    jacob1(span, nnode, &nxi[g * nnode], &neta[g * nnode], &nzeta[g * nnode], ce, dj[g].data(), gama[g]);
    if (bbar)
      vol_terms(span, gama[g], dj[g].data(), vol, &nxi[g * nnode], &neta[g * nnode], &nzeta[g * nnode],
                volume.data());
  }
  if (bbar) vol_avg(span, vol, volume.data());
  A2 ek(nrow);
  ek.zero();
  A2 b(totdof * 6), bd(totdof * 6);
  b.zero(); bd.zero();
  // icp: column-packed upper triangle, src/setup.f:265-275
  std::vector<int> icp_r(utsz), icp_c(utsz);
  for (int j = 1; j <= totdof; ++j)
    for (int i = 1; i <= j; ++i) {
      int pos = j * (j - 1) / 2 + i;
      icp_r[pos - 1] = i; icp_c[pos - 1] = j;
    }
  const bool include_qbar = m->qbar_flag != 0;
  for (int g = 0; g < ngp; ++g) {
    double weight = weights[g];
    // gptns1_a
    A2 qn1(36), cs(6);
    if (B.geonl) {
      const double* rc[9];
      for (int k = 0; k < 9; ++k) rc[k] = rot[g].col(k);
      getrm1(span, qn1, rc, 2);
      const double* m1[6]; double* m2[6];
      for (int k = 0; k < 6; ++k) { m1[k] = urcs[g].col(k); m2[k] = cs.col(k); }
      qmply1(span, qn1, m1, m2);
    }
    blcmp1(span, b, totdof, gama[g], &nxi[g * nnode], &neta[g * nnode], &nzeta[g * nnode], nnode);
    if (bbar) bmod(span, b, totdof, vol, m->eps_bbar);
    // drive_01_cnst -> extract_D_symmetric (src/gptns1.f:1174-1266), or
    // drive_10_cnst (:1371-1455): [D] = w det[J] history1(1:36)
    A2 cep(36);
    if (B.mat_type == W3G_MAT_CRYSTAL) {
      for (int i = 0; i < span; ++i) {
        double f = weight * dj[g][i];
        const double* h1 = s->history1[B.blk] + ((size_t)i * ngp + g) * MM10_HIST;
        for (int k = 0; k < 36; ++k) cep(i, k) = h1[k] * f;
      }
    } else {
      const double* gc = s->cep[B.blk];
      for (int i = 0; i < span; ++i) {
        double f = weight * dj[g][i];
        double sp[21];
        for (int k = 0; k < 21; ++k) sp[k] = f * gc[((size_t)g * span + i) * 21 + k];
        for (int k = 0; k < 21; ++k) {
          int r = kLowerR[k], cc = kLowerC[k];
          cep(i, (r - 1) + 6 * (cc - 1)) = sp[k];
          cep(i, (cc - 1) + 6 * (r - 1)) = sp[k];
        }
      }
    }
    // ctran1 (src/gptns1.f:1735-1969)
    if (B.geonl) {
      A2 tc(36);
      for (int j = 1; j <= 6; ++j)
        for (int i = 0; i < span; ++i)
          for (int kk = 1; kk <= 6; ++kk) {
#define Q(a, bq) qn1(i, (a - 1) + 6 * (bq - 1))
#define CE(a, bq) cep(i, (a - 1) + 6 * (bq - 1))
            tc(i, (j - 1) + 6 * (kk - 1)) = (Q(j, 1) * CE(1, kk) + Q(j, 2) * CE(2, kk) + Q(j, 3) * CE(3, kk) +
                                             Q(j, 4) * CE(4, kk) + Q(j, 5) * CE(5, kk) + Q(j, 6) * CE(6, kk));
          }
      for (int j = 1; j <= 6; ++j)
        for (int i = 0; i < span; ++i)
          for (int kk = 1; kk <= 6; ++kk) {
#define TC(a, bq) tc(i, (a - 1) + 6 * (bq - 1))
            CE(j, kk) = TC(j, 1) * Q(kk, 1) + TC(j, 2) * Q(kk, 2) + TC(j, 3) * Q(kk, 3) + TC(j, 4) * Q(kk, 4) +
                        TC(j, 5) * Q(kk, 5) + TC(j, 6) * Q(kk, 6);
#undef TC
          }
      if (include_qbar) {
        for (int i = 0; i < span; ++i) {
          double wf = dj[g][i] * weight;
          double halfw = half * wf;
          double xx = cs(i, 0), yy = cs(i, 1), zz = cs(i, 2), xy = cs(i, 3), yz = cs(i, 4), xz = cs(i, 5);
          CE(1, 1) = CE(1, 1) - two * xx * wf;
          CE(2, 2) = CE(2, 2) - two * yy * wf;
          CE(3, 3) = CE(3, 3) - two * zz * wf;
          CE(4, 1) = CE(4, 1) - xy * wf;
          CE(6, 1) = CE(6, 1) - xz * wf;
          CE(4, 2) = CE(4, 2) - xy * wf;
          CE(5, 2) = CE(5, 2) - yz * wf;
          CE(5, 3) = CE(5, 3) - yz * wf;
          CE(6, 3) = CE(6, 3) - xz * wf;
          CE(4, 4) = CE(4, 4) - halfw * (xx + yy);
          CE(5, 5) = CE(5, 5) - halfw * (yy + zz);
          CE(6, 6) = CE(6, 6) - halfw * (xx + zz);
          CE(5, 4) = CE(5, 4) - wf * xz;
          CE(6, 4) = CE(6, 4) - wf * yz;
          CE(6, 5) = CE(6, 5) - wf * xy;
          CE(1, 4) = CE(4, 1); CE(1, 6) = CE(6, 1); CE(2, 4) = CE(4, 2); CE(2, 5) = CE(5, 2);
          CE(3, 5) = CE(5, 3); CE(3, 6) = CE(6, 3); CE(4, 5) = CE(5, 4); CE(4, 6) = CE(6, 4);
          CE(5, 6) = CE(6, 5);
        }
      }
#undef Q
    }
    // adjust_cnst (src/gpmas1.f:399-430): tetrahedra scale [D] by 1/6
    // after ctran1; the geometric stiffness below is not scaled
    // (gptns1.f:222-225 then :278-288)
    if (B.etype == W3G_ETYPE_TET10) {
      const double scalar = adjust_scalar(B.etype);
      for (int k = 0; k < 36; ++k)
        for (int i = 0; i < span; ++i) cep(i, k) = scalar * cep(i, k);
    }
    // bdbtgen (src/gptns1.f:1628-1718)
#define BB(i, j, k) b(i, (j) + totdof * (k))
#define BD(i, j, k) bd(i, (j) + totdof * (k))
    for (int j = 0; j < totdof; ++j)
      for (int i = 0; i < span; ++i)
        for (int kk = 1; kk <= 6; ++kk)
          BD(i, j, kk - 1) = CE(1, kk) * BB(i, j, 0) + CE(2, kk) * BB(i, j, 1) + CE(3, kk) * BB(i, j, 2) +
                             CE(4, kk) * BB(i, j, 3) + CE(5, kk) * BB(i, j, 4) + CE(6, kk) * BB(i, j, 5);
    if (asym) {   // bdbt_asym (src/gptns1.f:1513-1612): every (row, col)
      int j = 0;
      for (int col = 0; col < totdof; ++col)
        for (int row = 0; row < totdof; ++row, ++j)
          for (int i = 0; i < span; ++i)
            ek(i, j) = ek(i, j) + BB(i, col, 0) * BD(i, row, 0) + BB(i, col, 1) * BD(i, row, 1) +
                       BB(i, col, 2) * BD(i, row, 2) + BB(i, col, 3) * BD(i, row, 3) +
                       BB(i, col, 4) * BD(i, row, 4) + BB(i, col, 5) * BD(i, row, 5);
    } else {
      for (int j = 0; j < utsz; ++j) {
        int row = icp_r[j] - 1, col = icp_c[j] - 1;
        for (int i = 0; i < span; ++i)
          ek(i, j) = ek(i, j) + BB(i, col, 0) * BD(i, row, 0) + BB(i, col, 1) * BD(i, row, 1) +
                     BB(i, col, 2) * BD(i, row, 2) + BB(i, col, 3) * BD(i, row, 3) +
                     BB(i, col, 4) * BD(i, row, 4) + BB(i, col, 5) * BD(i, row, 5);
      }
    }
#undef BB
#undef BD
#undef CE
    // kgstiff (src/kg1.f:16-110), symmetric assembly; with b-bar the
    // volume-averaged derivatives replace the Gauss point's (kg1.f:46-54)
    if (B.geonl) {
      std::vector<double> gxi((size_t)MXVL * nnode), geta((size_t)MXVL * nnode), gzeta((size_t)MXVL * nnode);
      A2& gm = gama[g];
      for (int j = 0; j < nnode; ++j)
        for (int i = 0; i < span; ++i) {
          if (bbar) {
            gxi[(size_t)j * MXVL + i] = vol(i, j);
            geta[(size_t)j * MXVL + i] = vol(i, j + 8);
            gzeta[(size_t)j * MXVL + i] = vol(i, j + 16);
            continue;
          }
          const double* nx = &nxi[g * nnode]; const double* ne = &neta[g * nnode]; const double* nz = &nzeta[g * nnode];
          gxi[(size_t)j * MXVL + i] = gm(i, 0) * nx[j] + gm(i, 3) * ne[j] + gm(i, 6) * nz[j];
          geta[(size_t)j * MXVL + i] = gm(i, 1) * nx[j] + gm(i, 4) * ne[j] + gm(i, 7) * nz[j];
          gzeta[(size_t)j * MXVL + i] = gm(i, 2) * nx[j] + gm(i, 5) * ne[j] + gm(i, 8) * nz[j];
        }
      int nus = nnode * (nnode - 1) / 2 + nnode;
      A2 gtg(nus);
      for (int j = 0; j < nus; ++j) {
        int a = icp_r[j] - 1, bq = icp_c[j] - 1;
        for (int i = 0; i < span; ++i) {
#define GX(n) gxi[(size_t)(n) * MXVL + i]
#define GE(n) geta[(size_t)(n) * MXVL + i]
#define GZ(n) gzeta[(size_t)(n) * MXVL + i]
          gtg(i, j) = (GX(a) * GX(bq) * cs(i, 0) + GE(a) * GE(bq) * cs(i, 1) + GZ(a) * GZ(bq) * cs(i, 2) +
                       (GX(a) * GE(bq) + GX(bq) * GE(a)) * cs(i, 3) + (GE(a) * GZ(bq) + GE(bq) * GZ(a)) * cs(i, 4) +
                       (GX(a) * GZ(bq) + GX(bq) * GZ(a)) * cs(i, 5)) *
                      dj[g][i] * weight;
#undef GX
#undef GE
#undef GZ
        }
      }
      for (int enode = 1; enode <= nnode; ++enode) {
        int cp1 = enode * (enode - 1) / 2;
        int cp2 = (nnode + enode) * (nnode + enode - 1) / 2 + nnode;
        int cp3 = (2 * nnode + enode) * (2 * nnode + enode - 1) / 2 + 2 * nnode;
        for (int j = 1; j <= enode; ++j) {
          if (asym) {   // kg1.f:112-178: (row j, col enode) and its mirror
            for (int d = 0; d < 3; ++d) {
              const int r = d * nnode + j, c = d * nnode + enode;   // 1-based
              const int k = (c - 1) * totdof + r - 1, kt = (r - 1) * totdof + c - 1;
              for (int i = 0; i < span; ++i) {
                ek(i, k) = ek(i, k) + gtg(i, cp1 + j - 1);
                if (r != c) ek(i, kt) = ek(i, kt) + gtg(i, cp1 + j - 1);
              }
            }
            continue;
          }
          for (int i = 0; i < span; ++i) {
            ek(i, cp1 + j - 1) = ek(i, cp1 + j - 1) + gtg(i, cp1 + j - 1);
            ek(i, cp2 + j - 1) = ek(i, cp2 + j - 1) + gtg(i, cp1 + j - 1);
            ek(i, cp3 + j - 1) = ek(i, cp3 + j - 1) + gtg(i, cp1 + j - 1);
          }
        }
      }
    }
  }
  // rktstf_do_transpose + beta_fact (src/rktstf.f:160-172, :221-290)
  for (int i = 0; i < span; ++i)
    for (int k = 0; k < nrow; ++k) estiff[(size_t)i * nrow + k] = ek(i, k);
  if (m->beta_fact != one)
    for (size_t k = 0; k < (size_t)nrow * span; ++k) estiff[k] = m->beta_fact * estiff[k];
  return 0;
}

}  // namespace

// =====================================================================
// C entry points
// =====================================================================
extern "C" {

void w3o_set_threads(int n) { g_threads = n; }
void w3o_set_deterministic(int on) { g_deterministic = on; }

int w3o_gauss_point(int etype, int order, int gpn, double* xyzw) {
  return getgpts(etype, order, gpn, xyzw[0], xyzw[1], xyzw[2], xyzw[3]) ? 0 : W3G_EUNSUPPORTED;
}

int w3o_shape_derivs(int etype, double xi, double eta, double zeta, double* nxi, double* neta, double* nzeta) {
  return derivs(etype, xi, eta, zeta, nxi, neta, nzeta) ? 0 : W3G_EUNSUPPORTED;
}

int w3o_tanstf(const w3g_model_desc* m, const w3g_block_state* s, int step, int iter, const double* c,
               const double* u, const double* du, double* const* estiff) {
  (void)step; (void)iter;
  for (int blk = 0; blk < m->nelblk; ++blk) {
    Blk B;
    if (!block_info(m, blk, B)) return W3G_EUNSUPPORTED;
  }
#ifdef _OPENMP
  if (g_threads > 0) omp_set_num_threads(g_threads);
  omp_set_dynamic(0);
#endif
  int status = 0;
#pragma omp parallel for schedule(static)
  for (int blk = 0; blk < m->nelblk; ++blk) {
    Blk B;
    block_info(m, blk, B);
    int st = tangent_block(m, s, B, c, u, du, estiff[blk]);
    if (st != 0) {
#pragma omp critical
      status = st;
    }
  }
  return status;
}

int w3o_recover(const w3g_model_desc* m, const w3g_block_state* s, int step, int iter, int extrapolated_du,
                const double* c, const double* u, const double* du, double* ifv, w3g_recover_info* info) {
  for (int blk = 0; blk < m->nelblk; ++blk) {
    Blk B;
    if (!block_info(m, blk, B)) return W3G_EUNSUPPORTED;
    if (B.mat_type != W3G_MAT_BILINEAR && B.mat_type != W3G_MAT_CRYSTAL && B.mat_type != W3G_MAT_UMAT)
      return W3G_EUNSUPPORTED;
    if (B.mat_type == W3G_MAT_UMAT && !m->umat_props) return W3G_EARG;
    // With b-bar WARP3D also scales F_n and F_n+1 of mm10 blocks to F-bar
    // (gtmat1_make_fbar, gtmat1.f:145-151), but only UMATs read those
    // (rstgp1.f:3786-3787): mm10 blocks take the b-bar strain increment,
    // internal forces and tangent restated here.
    if (B.mat_type == W3G_MAT_CRYSTAL && (!m->crystals || !m->elem_crystal || !m->elem_angles))
      return W3G_EARG;
  }
#ifdef _OPENMP
  if (g_threads > 0) omp_set_num_threads(g_threads);
  omp_set_dynamic(0);
#endif
  std::vector<RecOut> outs(m->nelblk);
#pragma omp parallel for schedule(static)
  for (int blk = 0; blk < m->nelblk; ++blk) {
    Blk B;
    block_info(m, blk, B);
    outs[blk] = recover_block(m, s, B, step, iter, extrapolated_du != 0, c, u, du);
  }
  // serial reductions (src/drive_eps_sig_internal_forces.f:210-226)
  w3g_recover_info r{};
  int cut_status = 0;
  for (int blk = 0; blk < m->nelblk; ++blk) {
    if (outs[blk].status == W3G_STEP_CUT || outs[blk].status == W3G_LOCAL_FAIL) {
      r.material_cut_step = 1;
      if (r.first_bad_element == 0 || outs[blk].bad_elem < r.first_bad_element) {
        r.first_bad_element = outs[blk].bad_elem;
        cut_status = outs[blk].status;
      }
    }
    r.internal_energy = r.internal_energy + outs[blk].energy;
    r.plastic_work = r.plastic_work + outs[blk].plastic;
  }
  if (info) *info = r;
  for (int k = 0; k < m->nodof; ++k) ifv[k] = zero;
  if (r.material_cut_step) return cut_status;
  // addifv_standard (src/addifv.f:86-124)
  double sum_ifv = 0.0;
  long long nterm = 0;
  if (g_deterministic) {
    for (int blk = 0; blk < m->nelblk; ++blk) {
      Blk B;
      block_info(m, blk, B);
      const int* edest = m->edest[blk];
      const double* ev = s->einfvec[blk];
      for (int j = 0; j < B.totdof; ++j)
        for (int i = 0; i < B.span; ++i) ifv[edest[(size_t)i * B.totdof + j] - 1] += ev[(size_t)j * B.span + i];
      for (int j = 0; j < B.totdof; ++j)
        for (int i = 0; i < B.span; ++i) sum_ifv = sum_ifv + std::fabs(ev[(size_t)j * B.span + i]);
      nterm += (long long)B.totdof * B.span;
    }
  } else {
#pragma omp parallel for schedule(static) reduction(+ : sum_ifv, nterm)
    for (int blk = 0; blk < m->nelblk; ++blk) {
      Blk B;
      block_info(m, blk, B);
      const int* edest = m->edest[blk];
      const double* ev = s->einfvec[blk];
      for (int j = 0; j < B.totdof; ++j)
        for (int i = 0; i < B.span; ++i) {
#pragma omp atomic update
          ifv[edest[(size_t)i * B.totdof + j] - 1] += ev[(size_t)j * B.span + i];
        }
      for (int j = 0; j < B.totdof; ++j)
        for (int i = 0; i < B.span; ++i) sum_ifv = sum_ifv + std::fabs(ev[(size_t)j * B.span + i]);
      nterm += (long long)B.totdof * B.span;
    }
  }
  if (info) { info->sum_ifv = sum_ifv; info->num_term_ifv = nterm; }
  return 0;
}

int w3o_update(const w3g_model_desc* m, const w3g_block_state* s) {
  for (int blk = 0; blk < m->nelblk; ++blk) {
    Blk B;
    if (!block_info(m, blk, B)) return W3G_EUNSUPPORTED;
    size_t n = (size_t)B.span * B.ngp;
    std::memcpy(s->history[blk], s->history1[blk], n * hist_size(B.mat_type) * sizeof(double));
    std::memcpy(s->eps_n[blk], s->eps_n1[blk], n * NSTR * sizeof(double));
    std::memcpy(s->urcs_n[blk], s->urcs_n1[blk], n * NSTRS * sizeof(double));
  }
  return 0;
}

int w3o_mm01_point(int span, int step, const double* e, const double* nu, const double* beta, const double* hprime,
                   const double* yld, const double* cgn_in, double* cgn1_out, const double* deps_in,
                   double* history_io, double* history1_out, double* cep_out) {
  if (span < 1 || span > MXVL) return W3G_EARG;
  MatVecs mv;
  for (int i = 0; i < span; ++i) {
    mv.e[i] = e[i]; mv.nu[i] = nu[i]; mv.beta[i] = beta[i]; mv.h[i] = hprime[i]; mv.yld[i] = yld[i];
    mv.lnelas[i] = false;
  }
  A2 cgn(9), cgn1(9), dep(6), h(MM01_HIST), h1(MM01_HIST), rtse(6), cep(36);
  for (int k = 0; k < 9; ++k) for (int i = 0; i < span; ++i) cgn(i, k) = cgn_in[(size_t)k * span + i];
  for (int k = 0; k < 6; ++k) for (int i = 0; i < span; ++i) dep(i, k) = deps_in[(size_t)k * span + i];
  for (int k = 0; k < MM01_HIST; ++k) for (int i = 0; i < span; ++i) h(i, k) = history_io[(size_t)k * span + i];
  double* pc[9]; double* pc1[9]; double* pd[6];
  for (int k = 0; k < 9; ++k) { pc[k] = cgn.col(k); pc1[k] = cgn1.col(k); }
  for (int k = 0; k < 6; ++k) pd[k] = dep.col(k);
  mm01(span, step, mv, pc, pc1, pd, h, h1, rtse);
  cnst1(span, cep, rtse, mv, h1.col(1), h1.col(4), h1.col(0), h1.col(3));
  for (int k = 0; k < 9; ++k) for (int i = 0; i < span; ++i) cgn1_out[(size_t)k * span + i] = cgn1(i, k);
  for (int k = 0; k < MM01_HIST; ++k)
    for (int i = 0; i < span; ++i) {
      history_io[(size_t)k * span + i] = h(i, k);
      history1_out[(size_t)k * span + i] = h1(i, k);
    }
  for (int k = 0; k < 36; ++k) for (int i = 0; i < span; ++i) cep_out[(size_t)k * span + i] = cep(i, k);
  return 0;
}

}  // extern "C"

extern "C" int w3o_mm10_point(const w3g_crystal* crystal, const double* angles, int step, int iter,
                              int extrapolated_du, double dt, double* hist_n, double* hist_n1,
                              const double* urcs_n, double* urcs_n1, const double* uddt, const double* rot_n1) {
  w3o::CrystalProps cp;
  w3o::mm10_element_props(*crystal, angles, cp);
  return w3o::mm10_point(cp, step, iter, extrapolated_du != 0, dt, 1, 1, hist_n, hist_n1, urcs_n, urcs_n1, uddt,
                         rot_n1);
}
