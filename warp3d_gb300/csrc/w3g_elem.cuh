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
  static constexpr int NN = 8;
  static constexpr int NG = 8;
  static constexpr int TOTDOF = 24;
  static constexpr int UTSZ = 300;

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
