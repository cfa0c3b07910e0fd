// w3g_umat.cuh -- the UMAT interface of the recovery kernels: material
// model 8 (Abaqus UMAT) of WARP3D, driven per material point as WARP3D's
// drive_umat_update does (src/rstgp1.f:3476-4010).
//
// umat() below has the Abaqus argument list (less the character name and
// WARP3D's nonlocal sharing vector) and is the routine a user replaces,
// exactly as a WARP3D user edits src/user_routines_umat.f and relinks; the
// library is then rebuilt. kUmatInfo describes it as umat_set_features
// does (src/user_routines_umat.f:35-66). The routine compiled here is the
// reference's example: isotropic elasticity and Mises plasticity with
// linear kinematic hardening (src/user_routines_umat.f:77-330), 20 state
// variables per point (elastic strains, plastic strains, back stress,
// equivalent plastic strain, state), props = (E, nu, yield stress, H',
// thermal expansion coefficient).
//
// umat_point() is WARP3D's side of the interface for one point of one
// element: WARP3D's shear order (xx yy zz xy yz xz) swapped to Abaqus's
// (xx yy zz xy xz yz) and back, statev from history at n (zero at step 1),
// identity drot (WARP3D rotates the stresses itself: the UMAT sees
// unrotated quantities), F at n and n+1, the kiter = 0 path (only [D] and
// the stress of the imposed increment, no history update), the work terms
// of the stress vector (7: total work by the trapezoid rule over the
// increment, 8: the UMAT's plastic dissipation spd) and the symmetrised
// [D] in cep order (rstgp1_make_symmetric_store, :5095-5146).
// Temperatures are not part of this path (dtemp = 0, temp = 0); coords
// and celent are passed as zero; dfgrd0/dfgrd1 are the plain deformation
// gradients (WARP3D passes F-bar ones for b-bar bricks).
#pragma once
#include <cuda_runtime.h>

namespace w3g {

constexpr int kUmatNstatv = 20;                          // info_vector(1)
constexpr int kUmatInfo[4] = {kUmatNstatv, 21, 0, 14};   // umat_set_features
constexpr int kUmatNprops = W3G_UMAT_NPROPS;

// rotsig (Abaqus utility): R t R^T of a symmetric tensor in Abaqus Voigt
// order; lstr = 1 tensor shears (stress), 2 engineering shears (strain)
__device__ __forceinline__ void umat_rotsig(const double* s, const double* drot, double* out, int lstr) {
  const double f = lstr == 2 ? 0.5 : 1.0;
  const double t[9] = {s[0], f * s[3], f * s[4], f * s[3], s[1], f * s[5], f * s[4], f * s[5], s[2]};
  double a[9];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r)
      a[r + 3 * c] = drot[r] * t[3 * c] + drot[r + 3] * t[1 + 3 * c] + drot[r + 6] * t[2 + 3 * c];
  double o[9];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) o[r + 3 * c] = a[r] * drot[c] + a[r + 3] * drot[c + 3] + a[r + 6] * drot[c + 6];
  const double g = lstr == 2 ? 2.0 : 1.0;
  out[0] = o[0]; out[1] = o[4]; out[2] = o[8];
  out[3] = g * o[3]; out[4] = g * o[6]; out[5] = g * o[7];
}

// The UMAT (Abaqus argument meanings; ddsdde column-major ntens x ntens).
__device__ inline void umat(double* stress, double* statev, double* ddsdde, double& sse, double& spd, double& scd,
                            double& rpl, double* ddsddt, double* drplde, double& drpldt, const double* stran,
                            double* dstran, const double* time, double dtime, double temp, double dtemp,
                            const double* predef, const double* dpred, int ndi, int nshr, int ntens, int nstatv,
                            const double* props, int nprops, const double* coords, const double* drot,
                            double& pnewdt, double celent, const double* dfgrd0, const double* dfgrd1, int noel,
                            int npt, int layer, int kspt, int kstep, int kinc, int kiter) {
  (void)scd; (void)rpl; (void)ddsddt; (void)drplde; (void)drpldt; (void)stran; (void)time; (void)dtime;
  (void)temp; (void)predef; (void)dpred; (void)ndi; (void)nshr; (void)ntens; (void)nstatv; (void)nprops;
  (void)coords; (void)pnewdt; (void)celent; (void)dfgrd0; (void)dfgrd1; (void)noel; (void)npt; (void)layer;
  (void)kspt; (void)kstep; (void)kinc; (void)kiter;
  const double zero = 0.0, one = 1.0, two = 2.0, three = 3.0, six = 6.0, half = 0.5;
  const double enumax = 0.4999, toler = 1.0e-6;
#define DD(r, c) ddsdde[(r) + 6 * (c)]
  const double cte = props[4];
  dstran[0] = dstran[0] - cte * dtemp;
  dstran[1] = dstran[1] - cte * dtemp;
  dstran[2] = dstran[2] - cte * dtemp;
  // elastic constants and stiffness
  const double emod = props[0];
  const double enu = fmin(props[1], enumax);
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
  // elastic strain, plastic strain, back stress at n, rotated by drot
  double eelas[6], eplas[6], alpha[6], flow[6], olds[6], avg;
  umat_rotsig(statev + 0, drot, eelas, 2);
  umat_rotsig(statev + 6, drot, eplas, 2);
  umat_rotsig(statev + 12, drot, alpha, 1);
  const double old_eqpl = statev[18];
  double deqpl = zero, dspd = zero, dsst = zero, state_np1 = zero;
  if (old_eqpl > zero) state_np1 = two;
  for (int k1 = 0; k1 < 6; ++k1) olds[k1] = stress[k1];
  // elastic predictor
  for (int k1 = 0; k1 < 6; ++k1) {
    eelas[k1] = eelas[k1] + dstran[k1];
    for (int k2 = 0; k2 < 6; ++k2) stress[k2] = stress[k2] + DD(k2, k1) * dstran[k1];
  }
  // equivalent Mises stress of stress - alpha
  double t0 = stress[0] - alpha[0] - stress[1] + alpha[1];
  double t1 = stress[1] - alpha[1] - stress[2] + alpha[2];
  double t2 = stress[2] - alpha[2] - stress[0] + alpha[0];
  double smises = t0 * t0 + t1 * t1 + t2 * t2;
  for (int k = 3; k < 6; ++k) {
    const double d = stress[k] - alpha[k];
    smises = smises + six * (d * d);
  }
  smises = sqrt(smises / two);
  const double syield = props[2];
  const double hard = props[3];
  const double constant_hard = hard;
  if (smises > (one + toler) * syield) {   // actively yielding: radial return
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
    // consistent tangent from the effective moduli
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
    avg = (stress[k1] + olds[k1]) / two;
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

// rstgp1_make_symmetric_store: 0.5 (D + D^T) with shears 5 and 6 swapped
// back to WARP3D order, lower triangle by rows (cep order)
__device__ __forceinline__ void umat_symmetric_store(const double* ddsdde, double* cep21) {
  const int map[6] = {0, 1, 2, 3, 5, 4};
  double sv[36];
  for (int j = 0; j < 6; ++j)
    for (int i = 0; i < 6; ++i) sv[map[i] + 6 * map[j]] = 0.5 * (ddsdde[i + 6 * j] + ddsdde[j + 6 * i]);
  int k = 0;
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c <= r; ++c) cep21[k++] = sv[r + 6 * c];
}

// One material point of drive_umat_update. urcs_n/urcs_n1 (9, WARP3D
// order), eps_n (6), uddt (6, unrotated increment), hist/hist1
// (kUmatNstatv), F at n and n+1 (column-major; identity for small
// displacement). hist1 is written only when iter > 0 (kiter = 0 returns
// after [D] and the stress). Returns true when the UMAT asked for a
// smaller load step (pnewdt < 1).
__device__ inline bool umat_point(const double* props, int step, int iter, bool extrapolated_du, double dt,
                                  int noel, int npt, const double* urcs_n, const double* eps_n, const double* uddt,
                                  const double* hist, const double* fn, const double* fn1, double* urcs_n1,
                                  double* hist1, double* cep21) {
  const int map[6] = {0, 1, 2, 3, 5, 4};   // WARP3D -> Abaqus position
  double stress[6], stran[6], dstran[6], dstran_displ[6], statev[kUmatNstatv], ddsdde[36];
  const bool first = step == 1;            // stresses, strains and history start at zero
  for (int j = 0; j < 6; ++j) {
    stress[map[j]] = first ? 0.0 : urcs_n[j];
    stran[map[j]] = first ? 0.0 : eps_n[j];
    dstran_displ[map[j]] = uddt[j];
    dstran[map[j]] = uddt[j];
  }
  const bool process_flag = iter == 0 && !extrapolated_du;
  if (process_flag)
    for (int j = 0; j < 6; ++j) dstran[j] = 0.0;   // thermal part only: none here
  for (int k = 0; k < kUmatNstatv; ++k) statev[k] = first ? 0.0 : hist[k];
  for (int k = 0; k < 36; ++k) ddsdde[k] = 0.0;
  double sse = 0.0, spd = first ? 0.0 : urcs_n[7], scd = 0.0, rpl = 0.0, drpldt = 0.0, pnewdt = 1.0e6;
  double ddsddt[6] = {0, 0, 0, 0, 0, 0}, drplde[6] = {0, 0, 0, 0, 0, 0};
  const double time[2] = {(step - 1) * dt, step * dt};
  const double predef[1] = {0.0}, dpred[1] = {0.0}, coords[3] = {0.0, 0.0, 0.0};
  const double drot[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  umat(stress, statev, ddsdde, sse, spd, scd, rpl, ddsddt, drplde, drpldt, stran, dstran, time, dt, 0.0, 0.0,
       predef, dpred, 3, 3, 6, kUmatNstatv, props, kUmatNprops, coords, drot, pnewdt, 0.0, fn, fn1, noel, npt, 1, 1,
       1, step, iter);
  umat_symmetric_store(ddsdde, cep21);
  if (iter == 0) {
    if (process_flag)   // add the stress of the imposed increment (not seen by the UMAT)
      for (int k = 0; k < 6; ++k) {
        double s = 0.0;
        for (int j = 0; j < 6; ++j) s = s + ddsdde[k + 6 * j] * dstran_displ[j];
        stress[k] = stress[k] + s;
      }
    for (int j = 0; j < 6; ++j) urcs_n1[j] = stress[map[j]];
    urcs_n1[6] = 0.0; urcs_n1[7] = 0.0; urcs_n1[8] = 0.0;
    return false;
  }
  for (int j = 0; j < 6; ++j) urcs_n1[j] = stress[map[j]];
  for (int k = 0; k < kUmatNstatv; ++k) hist1[k] = statev[k];
  // work densities: total by the trapezoid rule, plastic from the UMAT
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

}  // namespace w3g
