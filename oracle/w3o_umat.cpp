// w3o_umat.cpp -- TEST INFRASTRUCTURE ONLY (the oracle): restatement of
// WARP3D's UMAT path for one material point, the checker of the CUDA
// engine's W3G_MAT_UMAT blocks.
//
//   umat_example   the reference's example UMAT, Mises plasticity with
//                  linear kinematic hardening (src/user_routines_umat.f:
//                  77-330), Abaqus ordering xx yy zz xy xz yz
//   rotsig         the Abaqus utility it calls (R t R^T; drot = identity
//                  from WARP3D)
//   umat_drive     drive_umat_update for one point (src/rstgp1.f:
//                  3476-4010): shear order swaps, statev from history,
//                  the kiter = 0 path, the work terms, and the symmetrised
//                  [D] (rstgp1_make_symmetric_store, :5095-5146)
// Temperatures are not part of this path (dtemp = 0); coords and celent
// are zero. Parity unpinned against executions of WARP3D, as the rest of
// the oracle; pinned by the closed-form tests in tests/.
#include "w3o_umat.h"

#include <algorithm>
#include <cmath>

namespace w3o {

namespace {

void rotsig(const double* s, const double* drot, double* out, int lstr) {
  const double f = lstr == 2 ? 0.5 : 1.0;
  const double t[9] = {s[0], f * s[3], f * s[4], f * s[3], s[1], f * s[5], f * s[4], f * s[5], s[2]};
  double a[9], o[9];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r)
      a[r + 3 * c] = drot[r] * t[3 * c] + drot[r + 3] * t[1 + 3 * c] + drot[r + 6] * t[2 + 3 * c];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) o[r + 3 * c] = a[r] * drot[c] + a[r + 3] * drot[c + 3] + a[r + 6] * drot[c + 6];
  const double g = lstr == 2 ? 2.0 : 1.0;
  out[0] = o[0]; out[1] = o[4]; out[2] = o[8];
  out[3] = g * o[3]; out[4] = g * o[6]; out[5] = g * o[7];
}

}  // namespace

// user_routines_umat.f:77-330 (statev: 1-6 elastic strains, 7-12 plastic
// strains, 13-18 back stress, 19 equivalent plastic strain, 20 state;
// props: E, nu, yield stress, H', thermal expansion coefficient)
void umat_example(double* stress, double* statev, double* ddsdde, double& sse, double& spd, double* dstran,
                  const double* props, const double* drot, double dtemp) {
  const double zero = 0.0, one = 1.0, two = 2.0, three = 3.0, six = 6.0, half = 0.5;
  const double enumax = 0.4999, toler = 1.0e-6;
#define DD(r, c) ddsdde[(r) + 6 * (c)]
  const double cte = props[4];
  dstran[0] = dstran[0] - cte * dtemp;
  dstran[1] = dstran[1] - cte * dtemp;
  dstran[2] = dstran[2] - cte * dtemp;
  const double emod = props[0];
  const double enu = std::min(props[1], enumax);
  const double ebulk3 = emod / (one - two * enu);
  const double eg2 = emod / (one + enu);
  const double eg = eg2 / two;
  const double eg3 = three * eg;
  const double elam = (ebulk3 - eg2) / three;
  for (int k1 = 0; k1 < 3; ++k1) {
    for (int k2 = 0; k2 < 3; ++k2) DD(k2, k1) = elam;
    DD(k1, k1) = eg2 + elam;
  }
  DD(3, 3) = eg; DD(4, 4) = eg; DD(5, 5) = eg;
  bool yielding = false;
  double eelas[6], eplas[6], alpha[6], flow[6], olds[6];
  rotsig(statev + 0, drot, eelas, 2);
  rotsig(statev + 6, drot, eplas, 2);
  rotsig(statev + 12, drot, alpha, 1);
  const double old_eqpl = statev[18];
  double deqpl = zero, dspd = zero, dsst = zero, state_np1 = zero;
  if (old_eqpl > zero) state_np1 = two;
  for (int k1 = 0; k1 < 6; ++k1) olds[k1] = stress[k1];
  for (int k1 = 0; k1 < 6; ++k1) {
    eelas[k1] = eelas[k1] + dstran[k1];
    for (int k2 = 0; k2 < 6; ++k2) stress[k2] = stress[k2] + DD(k2, k1) * dstran[k1];
  }
  const double t0 = stress[0] - alpha[0] - stress[1] + alpha[1];
  const double t1 = stress[1] - alpha[1] - stress[2] + alpha[2];
  const double t2 = stress[2] - alpha[2] - stress[0] + alpha[0];
  double smises = t0 * t0 + t1 * t1 + t2 * t2;
  for (int k = 3; k < 6; ++k) {
    const double d = stress[k] - alpha[k];
    smises = smises + six * (d * d);
  }
  smises = std::sqrt(smises / two);
  const double syield = props[2];
  const double hard = props[3];
  const double constant_hard = hard;
  if (smises > (one + toler) * syield) {
    const double shydro = (stress[0] + stress[1] + stress[2]) / three;
    for (int k = 0; k < 3; ++k) flow[k] = (stress[k] - alpha[k] - shydro) / smises;
    for (int k = 3; k < 6; ++k) flow[k] = (stress[k] - alpha[k]) / smises;
    deqpl = (smises - syield) / (eg3 + hard);
    state_np1 = one;
    yielding = true;
    for (int k = 0; k < 3; ++k) {
      alpha[k] = alpha[k] + hard * flow[k] * deqpl;
      eplas[k] = eplas[k] + three / two * flow[k] * deqpl;
      eelas[k] = eelas[k] - three / two * flow[k] * deqpl;
      stress[k] = alpha[k] + flow[k] * syield + shydro;
    }
    for (int k = 3; k < 6; ++k) {
      alpha[k] = alpha[k] + hard * flow[k] * deqpl;
      eplas[k] = eplas[k] + three * flow[k] * deqpl;
      eelas[k] = eelas[k] - three * flow[k] * deqpl;
      stress[k] = alpha[k] + flow[k] * syield;
    }
    const double effg = eg * (syield + hard * deqpl) / smises;
    const double effg2 = two * effg;
    const double effg3 = three * effg;
    const double efflam = (ebulk3 - effg2) / three;
    const double effhrd = eg3 * hard / (eg3 + hard) - effg3;
    for (int k1 = 0; k1 < 3; ++k1) {
      for (int k2 = 0; k2 < 3; ++k2) DD(k2, k1) = efflam;
      DD(k1, k1) = effg2 + efflam;
    }
    DD(3, 3) = effg; DD(4, 4) = effg; DD(5, 5) = effg;
    for (int k1 = 0; k1 < 6; ++k1)
      for (int k2 = 0; k2 < 6; ++k2) DD(k2, k1) = DD(k2, k1) + effhrd * flow[k2] * flow[k1];
  }
  for (int k1 = 0; k1 < 6; ++k1) {
    statev[k1] = eelas[k1];
    statev[k1 + 6] = eplas[k1];
    statev[k1 + 12] = alpha[k1];
    const double avg = (stress[k1] + olds[k1]) / two;
    dsst = dsst + avg * dstran[k1];
  }
  if (yielding) {
    const double new_eqpl = deqpl + old_eqpl;
    const double osy = syield + constant_hard * old_eqpl;
    const double nsy = syield + constant_hard * new_eqpl;
    dspd = deqpl * (osy + nsy) * half;
  }
  statev[18] = old_eqpl + deqpl;
  statev[19] = state_np1;
  sse = sse + (dsst - dspd);
  spd = spd + dspd;
#undef DD
}

// drive_umat_update, one point (rstgp1.f:3700-3930). urcs_n/urcs_n1:
// 9 values in WARP3D order; eps_n, uddt: 6; hist/hist1: nstatv; cep21: the
// symmetrised [D] in cep order. hist1 is written only when iter > 0.
// Returns true when the UMAT asked for a smaller step (pnewdt < 1).
bool umat_drive(const double* props, int step, int iter, bool extrapolated_du, const double* urcs_n,
                const double* eps_n, const double* uddt, const double* hist, int nstatv, double* urcs_n1,
                double* hist1, double* cep21) {
  static const int map[6] = {0, 1, 2, 3, 5, 4};
  double stress[6], stran[6], dstran[6], dstran_displ[6], statev[64], ddsdde[36];
  const bool first = step == 1;     // init_sig_eps / init_history / statev = 0 at step 1
  for (int j = 0; j < 6; ++j) {
    stress[map[j]] = first ? 0.0 : urcs_n[j];
    stran[map[j]] = first ? 0.0 : eps_n[j];
    dstran_displ[map[j]] = uddt[j];
    dstran[map[j]] = uddt[j];
  }
  (void)stran;
  const bool process_flag = iter == 0 && !extrapolated_du;
  if (process_flag)
    for (int j = 0; j < 6; ++j) dstran[j] = 0.0;
  for (int k = 0; k < nstatv; ++k) statev[k] = first ? 0.0 : hist[k];
  for (int k = 0; k < 36; ++k) ddsdde[k] = 0.0;
  double sse = 0.0, spd = first ? 0.0 : urcs_n[7];
  const double pnewdt = 1.0e6;   // the example UMAT never lowers it
  const double drot[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  umat_example(stress, statev, ddsdde, sse, spd, dstran, props, drot, 0.0);
  // rstgp1_make_symmetric_store
  double sv[36];
  for (int j = 0; j < 6; ++j)
    for (int i = 0; i < 6; ++i) sv[map[i] + 6 * map[j]] = 0.5 * (ddsdde[i + 6 * j] + ddsdde[j + 6 * i]);
  int k = 0;
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c <= r; ++c) cep21[k++] = sv[r + 6 * c];
  if (iter == 0) {
    if (process_flag)
      for (int r = 0; r < 6; ++r) {
        double s = 0.0;
        for (int j = 0; j < 6; ++j) s = s + ddsdde[r + 6 * j] * dstran_displ[j];
        stress[r] = stress[r] + s;
      }
    for (int j = 0; j < 6; ++j) urcs_n1[j] = stress[map[j]];
    urcs_n1[6] = 0.0; urcs_n1[7] = 0.0; urcs_n1[8] = 0.0;
    return false;
  }
  for (int j = 0; j < 6; ++j) urcs_n1[j] = stress[map[j]];
  for (int q = 0; q < nstatv; ++q) hist1[q] = statev[q];
  double w = first ? 0.0 : urcs_n[6];
  for (int j = 0; j < 6; ++j) {
    const double avg = 0.5 * ((first ? 0.0 : urcs_n[j]) + urcs_n1[j]);
    w = w + avg * dstran[map[j]];
  }
  urcs_n1[6] = w;
  urcs_n1[7] = spd;
  urcs_n1[8] = 0.0;
  return pnewdt < 1.0;
}

}  // namespace w3o

// one point of the UMAT path, for tests: the arrays of umat_drive, the
// 50 umat properties, the 20 state variables of the example
extern "C" int w3o_umat_point(const double* props, int step, int iter, int extrapolated_du, const double* urcs_n,
                              const double* eps_n, const double* uddt, const double* hist, double* urcs_n1,
                              double* hist1, double* cep21) {
  return w3o::umat_drive(props, step, iter, extrapolated_du != 0, urcs_n, eps_n, uddt, hist, w3o::UMAT_NSTATV,
                         urcs_n1, hist1, cep21) ? 2 : 0;
}
