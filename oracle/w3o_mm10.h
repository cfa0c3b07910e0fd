// w3o_mm10.h -- the oracle's restatement of WARP3D's mm10 crystal
// plasticity update for one Gauss point (one crystal). TEST
// INFRASTRUCTURE ONLY (parity checker and CPU baseline).
//
// Scope: fcc slip systems (slip_type 1), isotropic elasticity
// (elastic_type 1), Voce hardening (h_type 1, one hardening variable),
// the Newton solver with line search (solver = .true., tang_calc = 0),
// adaptive sub-stepping, the consistent tangent and the history layout of
// mm10_set_history_locs (src/mm10_d.f:25-390) for one crystal.
#pragma once
#include "../include/w3g.h"

namespace w3o {

constexpr int MM10_NSLIP = 12;
// history per Gauss point for one fcc crystal with one hardening
// variable: common 36 + 27 + 9 + 3 + 12, crystal 6+3+9+6+6+12+1+15+1+6+6
constexpr int MM10_HIST = 87 + 71;

// per-element crystal properties after setup_mm10_rknstr
// (src/rknstr.f:1568-2027) and mm10_init_cc_props (src/mm10_a.f:1840)
struct CrystalProps {
  double stiffness[36];          // (6,6) column-major, rotated to the reference frame
  double ms[MM10_NSLIP][6];      // sym(b x n) Voigt (engineering shear)
  double qs[MM10_NSLIP][3];      // skew(b x n) as (w23, w13, w12)
  double ns[MM10_NSLIP][3];
  double g[9];                   // rotation_g, column-major
  double angles[3];              // initial Euler angles (degrees, Kocks)
  double rate_n, tau_y, tau_v, theta_0, voche_m, iD_v, k_0, burgers;
  double atol, atol1, rtol, rtol1;
  int miter;
  int asymmetric = 0;            // asymmetric assembly: tangent left unsymmetrized
};

// builds the element's crystal properties from a crystal definition and
// the element's Euler angles (degrees, Kocks convention)
void mm10_element_props(const w3g_crystal& c, const double* angles, CrystalProps& p);

// the mm10 update of one Gauss point (mm10, src/mm10_a.f:29-362) as
// drive_10_update calls it (src/rstgp1.f:4327-4510). hist_n / hist_n1:
// MM10_HIST values; urcs_n / urcs_n1: 9 values; uddt: 6; rot_n1: 9
// (column-major R at n+1). Returns 0, or W3G_LOCAL_FAIL when the local
// solve failed after all step cuts.
int mm10_point(const CrystalProps& p, int step, int iter, bool extrapolated_du, double dt, int elem, int gpn,
               double* hist_n /* modified at step 1 as the reference does */, double* hist_n1,
               const double* urcs_n, double* urcs_n1, const double* uddt, const double* rot_n1);

}  // namespace w3o
