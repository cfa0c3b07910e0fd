// w3g_elem.cuh -- element library for the kernels: Gauss points and
// shape-function derivatives, evaluated once on the host with the same
// formulas as WARP3D (src/getgpts.f, src/derivs.f) and uploaded with the
// model; each CTA stages its element type's table into shared memory.
#pragma once
#include <cuda_runtime.h>

namespace w3g {

// 8-node hexahedron, 2x2x2 rule: quad2 (src/getgpts.f:642-700) and
// deriv2 (src/derivs.f:283-328). Node order (xi, eta, zeta):
// 1(-,-,+) 2(-,-,-) 3(-,+,-) 4(-,+,+) 5(+,-,+) 6(+,-,-) 7(+,+,-) 8(+,+,+);
// GP order: eta fastest, then xi, then zeta.
struct Hex8 {
  static constexpr int SLOT = 0;   // type_slot
  static constexpr int NN = 8;
  static constexpr int NG = 8;
  static constexpr int TOTDOF = 24;
  static constexpr int UTSZ = 300;
  static constexpr bool TET = false;

  static void gauss_point(int g, double& xi, double& eta, double& zeta, double& w) {
    const double l1 = 0.5773502691896257645;
    static const int sx[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
    static const int se[8] = {-1, 1, -1, 1, -1, 1, -1, 1};
    static const int sz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
    xi = sx[g] * l1; eta = se[g] * l1; zeta = sz[g] * l1; w = 1.0;
  }
  static void derivs(double xi, double eta, double zeta, double* nxi, double* neta, double* nzeta) {
    const double one = 1.0, one25 = 0.125;
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
};

// 20-node hexahedron (q3disop), 3x3x3 rule: quad1 order 1
// (src/getgpts.f:177-420) and deriv1 (src/derivs.f:182-281). Corner nodes
// as the 8-node brick; mid-edge nodes 9-20.
struct Hex20 {
  static constexpr int SLOT = 1;   // type_slot
  static constexpr int NN = 20;
  static constexpr int NG = 27;
  static constexpr int TOTDOF = 60;
  static constexpr int UTSZ = 1830;
  static constexpr bool TET = false;

  static void gauss_point(int g, double& xi, double& eta, double& zeta, double& w) {
    const double l1 = 0.774596669241483, l2 = 0.0;
    const double ws[4] = {0.1714677640603571, 0.2743484224965712, 0.4389574759945135, 0.7023319615912210};
    const double v[3] = {-l1, l2, l1};
    int ie = g % 3, ix = (g / 3) % 3, iz = g / 9;
    xi = v[ix]; eta = v[ie]; zeta = v[iz];
    w = ws[(ix == 1) + (ie == 1) + (iz == 1)];
  }
  static void derivs(double r, double s, double t, double* nr, double* ns, double* nt) {
    const double one = 1.0, half = 0.5, fourth = 0.25, eighth = 0.125;
    double rp1 = one + r, rm1 = one - r, sp1 = one + s, sm1 = one - s, tp1 = one + t, tm1 = one - t;
    double rps = r + s, rms = r - s, spt = s + t, smt = s - t;
    nr[0] = sm1 * (rp1 + rps - t) * tp1 * eighth;   nr[1] = sm1 * (rp1 + rps + t) * tm1 * eighth;
    nr[2] = sp1 * (rp1 + rms + t) * tm1 * eighth;   nr[3] = sp1 * (rp1 + rms - t) * tp1 * eighth;
    nr[4] = -sm1 * (rm1 - rms - t) * tp1 * eighth;  nr[5] = -sm1 * (rm1 - rms + t) * tm1 * eighth;
    nr[6] = -sp1 * (rm1 - rps + t) * tm1 * eighth;  nr[7] = -sp1 * (rm1 - rps - t) * tp1 * eighth;
    nr[8] = -sm1 * tm1 * tp1 * fourth;  nr[9] = -sm1 * sp1 * tm1 * fourth;
    nr[10] = -sp1 * tm1 * tp1 * fourth; nr[11] = -sm1 * sp1 * tp1 * fourth;
    nr[12] = sm1 * tm1 * tp1 * fourth;  nr[13] = sm1 * sp1 * tm1 * fourth;
    nr[14] = sp1 * tm1 * tp1 * fourth;  nr[15] = sm1 * sp1 * tp1 * fourth;
    nr[16] = -r * sm1 * tp1 * half;     nr[17] = -r * sm1 * tm1 * half;
    nr[18] = -r * sp1 * tm1 * half;     nr[19] = -r * sp1 * tp1 * half;
    ns[0] = rm1 * (rp1 + s + smt) * tp1 * eighth;   ns[1] = rm1 * (rp1 + s + spt) * tm1 * eighth;
    ns[2] = -rm1 * (rp1 - s - smt) * tm1 * eighth;  ns[3] = -rm1 * (rp1 - s - spt) * tp1 * eighth;
    ns[4] = rp1 * (rm1 + s + smt) * tp1 * eighth;   ns[5] = rp1 * (rm1 + s + spt) * tm1 * eighth;
    ns[6] = -rp1 * (rm1 - s - smt) * tm1 * eighth;  ns[7] = -rp1 * (rm1 - s - spt) * tp1 * eighth;
    ns[8] = -rm1 * tm1 * tp1 * fourth;  ns[9] = -rm1 * s * tm1 * half;
    ns[10] = rm1 * tm1 * tp1 * fourth;  ns[11] = -rm1 * s * tp1 * half;
    ns[12] = -rp1 * tm1 * tp1 * fourth; ns[13] = -rp1 * s * tm1 * half;
    ns[14] = rp1 * tm1 * tp1 * fourth;  ns[15] = -rp1 * s * tp1 * half;
    ns[16] = -rm1 * rp1 * tp1 * fourth; ns[17] = -rm1 * rp1 * tm1 * fourth;
    ns[18] = rm1 * rp1 * tm1 * fourth;  ns[19] = rm1 * rp1 * tp1 * fourth;
    nt[0] = -rm1 * sm1 * (rp1 + smt - t) * eighth;  nt[1] = rm1 * sm1 * (rp1 + spt + t) * eighth;
    nt[2] = rm1 * sp1 * (rp1 - smt + t) * eighth;   nt[3] = -rm1 * sp1 * (rp1 - spt - t) * eighth;
    nt[4] = -rp1 * sm1 * (rm1 + smt - t) * eighth;  nt[5] = rp1 * sm1 * (rm1 + spt + t) * eighth;
    nt[6] = rp1 * sp1 * (rm1 - smt + t) * eighth;   nt[7] = -rp1 * sp1 * (rm1 - spt - t) * eighth;
    nt[8] = -rm1 * sm1 * t * half;      nt[9] = -rm1 * sm1 * sp1 * fourth;
    nt[10] = -rm1 * sp1 * t * half;     nt[11] = rm1 * sm1 * sp1 * fourth;
    nt[12] = -rp1 * sm1 * t * half;     nt[13] = -rp1 * sm1 * sp1 * fourth;
    nt[14] = -rp1 * sp1 * t * half;     nt[15] = rp1 * sm1 * sp1 * fourth;
    nt[16] = rm1 * rp1 * sm1 * fourth;  nt[17] = -rm1 * rp1 * sm1 * fourth;
    nt[18] = -rm1 * rp1 * sp1 * fourth; nt[19] = rm1 * rp1 * sp1 * fourth;
  }
};

// 10-node tetrahedron, 4-point rule: quad6 order 4 (src/getgpts.f:771-850)
// and deriv6 (src/derivs.f:606-662); weights sum to 1, so [D] and the
// internal-force weights carry 1/6 (adjust_scalar_weights,
// src/initst.f:888-930).
struct Tet10 {
  static constexpr int SLOT = 2;   // type_slot
  static constexpr int NN = 10;
  static constexpr int NG = 4;
  static constexpr int TOTDOF = 30;
  static constexpr int UTSZ = 465;
  static constexpr bool TET = true;

  static void gauss_point(int g, double& xi, double& eta, double& zeta, double& w) {
    const double a = 0.58541020, b = 0.13819660;
    w = 0.25;
    xi = g == 1 ? a : b;
    eta = g == 2 ? a : b;
    zeta = g == 3 ? a : b;
  }
  static void derivs(double s2, double s3, double s4, double* q2, double* q3, double* q4) {
    const double zero = 0.0, one = 1.0, four = 4.0;
    double s1 = one - s2 - s3 - s4;
    q2[0] = one - four * s1; q2[1] = four * s2 - one; q2[2] = zero; q2[3] = zero; q2[4] = four * (s1 - s2);
    q2[5] = four * s3; q2[6] = -four * s3; q2[7] = -four * s4; q2[8] = four * s4; q2[9] = zero;
    q3[0] = one - four * s1; q3[1] = zero; q3[2] = four * s3 - one; q3[3] = zero; q3[4] = -four * s2;
    q3[5] = four * s2; q3[6] = four * (s1 - s3); q3[7] = -four * s4; q3[8] = zero; q3[9] = four * s4;
    q4[0] = one - four * s1; q4[1] = zero; q4[2] = zero; q4[3] = four * s4 - one; q4[4] = -four * s2;
    q4[5] = zero; q4[6] = -four * s3; q4[7] = four * (s1 - s4); q4[8] = four * s2; q4[9] = four * s3;
  }
};

// dN table layout: [g][d][a] with d = 0 (xi), 1 (eta), 2 (zeta),
// followed by the NG weights.
template <class E>
void fill_dn_table(double* t) {
  for (int g = 0; g < E::NG; ++g) {
    double xi, eta, zeta, w;
    E::gauss_point(g, xi, eta, zeta, w);
    E::derivs(xi, eta, zeta, t + (g * 3 + 0) * E::NN, t + (g * 3 + 1) * E::NN, t + (g * 3 + 2) * E::NN);
    t[E::NG * 3 * E::NN + g] = w;
  }
}
template <class E>
constexpr int dn_table_size() { return E::NG * 3 * E::NN + E::NG; }

}  // namespace w3g
