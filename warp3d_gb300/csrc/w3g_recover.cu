// w3g_recover.cu -- strain/stress recovery with the mm01 update, element
// internal forces and their deterministic assembly into the nodal vector
// (drive_eps_sig_internal_forces / do_nleps_block / rknstr / rstgp1 /
// drive_01_update / rplstr / rknifv / gpifv1 / addifv).
//
// k_recover_hex8: one CTA = 2 warps = one chunk of <= 8 elements of one
// block, one thread per (element, Gauss point). Element nodal data is
// staged once in shared memory; the 8 Gauss-point threads of an element
// are 8 consecutive lanes, so the element's internal-force vector and
// volume are summed over its Gauss points with warp shuffles in a fixed
// order. Everything here is FP64.
//
// k_assemble_ifv: one thread per global dof sums the element
// contributions that map to it (a CSR built from edest at model creation,
// contributions in ascending einfvec order). This replaces the OpenMP
// ATOMIC scatter of addifv.f:93-98 with a deterministic gather.
#include <climits>
#include "w3g_internal.cuh"
#include "w3g_elem.cuh"
#include "w3g_math.cuh"

namespace w3g {

namespace {

constexpr int NN = Hex8::NN;
constexpr int NG = Hex8::NG;
constexpr int TOT = Hex8::TOTDOF;
constexpr int kDnSize = NG * 3 * NN + NG;
constexpr int kThreads = kChunk * NG;   // 64

__global__ void __launch_bounds__(kThreads) k_recover_hex8(RecoverArgs a) {
  __shared__ double sdn[kDnSize];
  __shared__ double sce[kChunk][3 * NN];
  __shared__ double sue[kChunk][TOT];
  __shared__ double sdu[kChunk][TOT];
  __shared__ double sred[2][2];

  const int tid = threadIdx.x;
  const int ge = tid >> 3;
  const int g = tid & 7;
  const Chunk ch = a.chunks[blockIdx.x];
  const BlockDesc bd = a.blocks[ch.blk];
  const bool active = ge < ch.n;
  const int i = ch.i0 + ge;

  for (int k = tid; k < kDnSize; k += kThreads) sdn[k] = a.dn[k];
  if (active) {   // dupstr + dupstr_blocked gathers: lane g loads node g
    const long long dbase = bd.einf_off + (long long)i * TOT;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int j = d * NN + g;
      sce[ge][j] = a.c[a.cdest[dbase + j] - 1];
      const int eidx = a.edest[dbase + j] - 1;
      sue[ge][j] = a.u[eidx];
      sdu[ge][j] = a.du[eidx];
    }
  }
  __syncthreads();

  double fe[TOT];
#pragma unroll
  for (int k = 0; k < TOT; ++k) fe[k] = 0.0;
  double vol = 0.0, en = 0.0, pw = 0.0;

  if (active) {
    const int eg = bd.felem + i;   // global element (0-based)
    const MatProps mpd = a.mat[eg];
    MM01In mp;
    mp.e = mpd.e; mp.nu = mpd.nu; mp.beta = mpd.beta; mp.h = mpd.h; mp.yld = mpd.yld;
    mp.lnelas = mpd.lnelas != 0.0;
    const double* dnx = sdn + (g * 3 + 0) * NN;
    const double* dne = sdn + (g * 3 + 1) * NN;
    const double* dnz = sdn + (g * 3 + 2) * NN;
    const double w = sdn[NG * 3 * NN + g];
    const double* x0 = &sce[ge][0];
    const double* y0 = &sce[ge][NN];
    const double* z0 = &sce[ge][2 * NN];
    const double* ue = &sue[ge][0];
    const double* du = &sdu[ge][0];
    const bool update_coords = bd.geonl && !(a.step == 1 && a.iter == 0);

    // ---- gtmat1 (src/gtmat1.f:17-190), reference-order arithmetic ----
    double gama0[9], dj0;
    jacob1_ref<NN>(dnx, dne, dnz, x0, y0, z0, gama0, dj0);
    double th1[9], thh[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) { th1[k] = 0.0; thh[k] = 0.0; }
#pragma unroll
    for (int n = 0; n < NN; ++n) {   // tcomp1 for u_{n+1} and u_{n+1/2} (rstgp1_a)
      double tx, ty, tz;
      grad_ref(gama0, dnx[n], dne[n], dnz[n], tx, ty, tz);
      const double u1x = ra(ue[n], du[n]), u1y = ra(ue[NN + n], du[NN + n]),
                   u1z = ra(ue[2 * NN + n], du[2 * NN + n]);
      const double uhx = ra(ue[n], rm(0.5, du[n])), uhy = ra(ue[NN + n], rm(0.5, du[NN + n])),
                   uhz = ra(ue[2 * NN + n], rm(0.5, du[2 * NN + n]));
      th1[0] = ra(th1[0], rm(tx, u1x)); th1[1] = ra(th1[1], rm(tx, u1y)); th1[2] = ra(th1[2], rm(tx, u1z));
      th1[3] = ra(th1[3], rm(ty, u1x)); th1[4] = ra(th1[4], rm(ty, u1y)); th1[5] = ra(th1[5], rm(ty, u1z));
      th1[6] = ra(th1[6], rm(tz, u1x)); th1[7] = ra(th1[7], rm(tz, u1y)); th1[8] = ra(th1[8], rm(tz, u1z));
      thh[0] = ra(thh[0], rm(tx, uhx)); thh[1] = ra(thh[1], rm(tx, uhy)); thh[2] = ra(thh[2], rm(tx, uhz));
      thh[3] = ra(thh[3], rm(ty, uhx)); thh[4] = ra(thh[4], rm(ty, uhy)); thh[5] = ra(thh[5], rm(ty, uhz));
      thh[6] = ra(thh[6], rm(tz, uhx)); thh[7] = ra(thh[7], rm(tz, uhy)); thh[8] = ra(thh[8], rm(tz, uhz));
    }
    // fcomp1: F column-major
    double F1[9] = {th1[0] + 1.0, th1[1], th1[2], th1[3], th1[4] + 1.0, th1[5], th1[6], th1[7], th1[8] + 1.0};
    double Fh[9] = {thh[0] + 1.0, thh[1], thh[2], thh[3], thh[4] + 1.0, thh[5], thh[6], thh[7], thh[8] + 1.0};
    const double dfn1 = det_ref(F1);
    const double dfh = det_ref(Fh);
    if (dfn1 <= 1.0e-20) atomicMin(a.status, bad_point_key(ch.blk, g, 0, i));
    else if (dfh <= 1.0e-20) atomicMin(a.status, bad_point_key(ch.blk, g, 1, i));
    double R1[9], Rh[9], qnh[36];
    polar_rotation_ref(F1, R1);
    polar_rotation_ref(Fh, Rh);
    rotation_q1(Rh, qnh);

    // ---- rknstr_geonl: jacobian at mid-step; gtlsn1 + qmply1 ----
    double xm[NN], ym[NN], zm[NN];
#pragma unroll
    for (int n = 0; n < NN; ++n) {
      if (update_coords) {
        xm[n] = x0[n] + ue[n] + 0.5 * du[n];
        ym[n] = y0[n] + ue[NN + n] + 0.5 * du[NN + n];
        zm[n] = z0[n] + ue[2 * NN + n] + 0.5 * du[2 * NN + n];
      } else {
        xm[n] = x0[n]; ym[n] = y0[n]; zm[n] = z0[n];
      }
    }
    double gm[9], djm;
    jacobian_inverse<NN, double>(dnx, dne, dnz, xm, ym, zm, gm, djm);
    double ddt[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int n = 0; n < NN; ++n) {
      double gx, gy, gz;
      shape_gradient<double>(gm, dnx[n], dne[n], dnz[n], gx, gy, gz);
      const double dx = du[n], dy = du[NN + n], dz = du[2 * NN + n];
      ddt[0] += gx * dx;
      ddt[1] += gy * dy;
      ddt[2] += gz * dz;
      ddt[3] += gy * dx + gx * dy;
      ddt[4] += gz * dy + gy * dz;
      ddt[5] += gz * dx + gx * dz;
    }
    double uddt[6];
    qmply<double>(qnh, ddt, uddt);

    // ---- state at n ----
    const long long gpi = bd.gp_off + (long long)i * NG + g;
    double cgn[9], hist[11], cgn1[9], hist1[11], cep21[21], eps1[6];
#pragma unroll
    for (int k = 0; k < 9; ++k) cgn[k] = a.urcs_n[gpi * 9 + k];
#pragma unroll
    for (int k = 0; k < 6; ++k) eps1[k] = a.eps_n[gpi * 6 + k] + uddt[k];
#pragma unroll
    for (int k = 0; k < 11; ++k) hist[k] = a.hist[gpi * kHistMM01 + k];

    // ---- drive_01_update (src/rstgp1.f:614-1034) ----
    if (a.nonlinear) {
      const long long gpf = bd.gp_off + g;   // block's first element, this GP
      const double alpha11_first = a.hist[gpf * kHistMM01 + 10];
      mm01_point(mp, a.step, cgn, uddt, hist, alpha11_first, cgn1, hist1, cep21);
    } else {   // drive_01_update_a/_b: linear-elastic [D], sigma = sigma_n + D uddt
      const double e = mp.e, nu = mp.nu;
      const double c1 = (e / ((1.0 + nu) * (1.0 - 2.0 * nu)));
      const double c2 = (1.0 - nu) * c1, c3 = ((1.0 - 2.0 * nu) / 2.0) * c1, c4 = nu * c1;
#pragma unroll
      for (int k = 0; k < 21; ++k) cep21[k] = 0.0;
      cep21[0] = c2; cep21[1] = c4; cep21[2] = c2; cep21[3] = c4; cep21[4] = c4; cep21[5] = c2;
      cep21[9] = c3; cep21[14] = c3; cep21[20] = c3;
      cgn1[0] = cgn[0] + c2 * uddt[0] + c4 * uddt[1] + c4 * uddt[2];
      cgn1[1] = cgn[1] + c4 * uddt[0] + c2 * uddt[1] + c4 * uddt[2];
      cgn1[2] = cgn[2] + c4 * uddt[0] + c4 * uddt[1] + c2 * uddt[2];
      cgn1[3] = cgn[3] + c3 * uddt[3];
      cgn1[4] = cgn[4] + c3 * uddt[4];
      cgn1[5] = cgn[5] + c3 * uddt[5];
      cgn1[6] = 0.0; cgn1[7] = 0.0; cgn1[8] = 0.0;
    }
    // rstgp1_store_cep: (21, span, ngp)
    double* cp = a.cep + bd.cep_off + ((long long)g * bd.span + i) * 21;
#pragma unroll
    for (int k = 0; k < 21; ++k) cp[k] = cep21[k];
    // rstgp1_b: energy and plastic work (large-strain branch)
    if (a.iter != 0) {
      const double factor = dfn1 * dj0 * a.beta_fact * w;
      en = cgn1[6] * factor;
      pw = cgn1[7] * factor;
    }
    // rplstr (src/rplstr.f:15-90)
#pragma unroll
    for (int k = 0; k < 9; ++k) a.urcs_n1[gpi * 9 + k] = cgn1[k];
#pragma unroll
    for (int k = 0; k < 6; ++k) a.eps_n1[gpi * 6 + k] = eps1[k];
    if (a.iter > 0) {
      if (bd.geonl) {
#pragma unroll
        for (int k = 0; k < 9; ++k) a.rot_n1[gpi * 9 + k] = R1[k];
      }
#pragma unroll
      for (int k = 0; k < 11; ++k) a.hist1[gpi * kHistMM01 + k] = hist1[k];
    }

    // ---- rknifv_std + gpifv1 (src/rknifv.f:141-217, src/gpifv1.f:16-154) ----
    double x1[NN], y1[NN], z1[NN];
#pragma unroll
    for (int n = 0; n < NN; ++n) {
      if (update_coords) {
        x1[n] = x0[n] + ue[n] + du[n];
        y1[n] = y0[n] + ue[NN + n] + du[NN + n];
        z1[n] = z0[n] + ue[2 * NN + n] + du[2 * NN + n];
      } else {
        x1[n] = x0[n]; y1[n] = y0[n]; z1[n] = z0[n];
      }
    }
    double g1[9], dj1;
    jacobian_inverse<NN, double>(dnx, dne, dnz, x1, y1, z1, g1, dj1);
    double cs[6];
    if (bd.geonl) {
      double q2[36];
      rotation_q2<double>(R1, q2);
      qmply<double>(q2, cgn1, cs);
    } else {
#pragma unroll
      for (int k = 0; k < 6; ++k) cs[k] = cgn1[k];
    }
    const double wdj = w * dj1;
#pragma unroll
    for (int k = 0; k < 6; ++k) cs[k] = cs[k] * wdj;
#pragma unroll
    for (int n = 0; n < NN; ++n) {
      double gx, gy, gz;
      shape_gradient<double>(g1, dnx[n], dne[n], dnz[n], gx, gy, gz);
      fe[n] = gx * cs[0] + gy * cs[3] + gz * cs[5];
      fe[NN + n] = gy * cs[1] + gx * cs[3] + gz * cs[4];
      fe[2 * NN + n] = gz * cs[2] + gy * cs[4] + gx * cs[5];
    }
    vol = wdj;
  }

  // ---- sum over the element's 8 Gauss points (lanes g = 0..7) ----
#pragma unroll
  for (int off = 1; off < NG; off <<= 1) {
#pragma unroll
    for (int k = 0; k < TOT; ++k) fe[k] += __shfl_xor_sync(0xffffffffu, fe[k], off);
    vol += __shfl_xor_sync(0xffffffffu, vol, off);
    en += __shfl_xor_sync(0xffffffffu, en, off);
    pw += __shfl_xor_sync(0xffffffffu, pw, off);
  }
  if (active) {
    // einfvec (span, totdof): lane g writes the dofs of node g
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int j = d * NN + g;
      double v = fe[0];
#pragma unroll
      for (int k = 0; k < TOT; ++k)
        if (k == j) v = fe[k];
      a.einf[bd.einf_off + (long long)j * bd.span + i] = v;
    }
    if (g == 0) a.evol[bd.felem + i] = vol;
  }
  // ---- chunk energy: sum over the 4 elements of the warp, then warps ----
  en += __shfl_xor_sync(0xffffffffu, en, 8);
  pw += __shfl_xor_sync(0xffffffffu, pw, 8);
  en += __shfl_xor_sync(0xffffffffu, en, 16);
  pw += __shfl_xor_sync(0xffffffffu, pw, 16);
  if ((tid & 31) == 0) { sred[tid >> 5][0] = en; sred[tid >> 5][1] = pw; }
  __syncthreads();
  if (tid == 0) {
    a.partials[2 * blockIdx.x + 0] = sred[0][0] + sred[1][0];
    a.partials[2 * blockIdx.x + 1] = sred[0][1] + sred[1][1];
  }
}

constexpr int kAsmThreads = 256;

__global__ void __launch_bounds__(kAsmThreads) k_assemble_ifv(int nodof, const int* __restrict__ rowptr,
                                                              const long long* __restrict__ src,
                                                              const double* __restrict__ einf, double* ifv,
                                                              double* partials) {
  __shared__ double sw[kAsmThreads / 32];
  const int d = blockIdx.x * kAsmThreads + threadIdx.x;
  double s = 0.0, sa = 0.0;
  if (d < nodof) {
    for (int k = rowptr[d]; k < rowptr[d + 1]; ++k) {
      const double v = einf[src[k]];
      s += v;
      sa += fabs(v);
    }
    ifv[d] = s;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) sa += __shfl_xor_sync(0xffffffffu, sa, off);
  if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = sa;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < kAsmThreads / 32; ++k) t += sw[k];
    partials[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(256) k_finalize(int nchunks, const double* partials, int nparts,
                                                  const double* ifv_partials, const unsigned long long* status,
                                                  const BlockDesc* blocks, long long num_term,
                                                  w3g_recover_info* info) {
  __shared__ double s0[256], s1[256], s2[256];
  double e = 0.0, p = 0.0, f = 0.0;
  for (int k = threadIdx.x; k < nchunks; k += 256) { e += partials[2 * k]; p += partials[2 * k + 1]; }
  for (int k = threadIdx.x; k < nparts; k += 256) f += ifv_partials[k];
  s0[threadIdx.x] = e; s1[threadIdx.x] = p; s2[threadIdx.x] = f;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      s0[threadIdx.x] += s0[threadIdx.x + w];
      s1[threadIdx.x] += s1[threadIdx.x + w];
      s2[threadIdx.x] += s2[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const unsigned long long st = status[0];
    const bool cut = st != ~0ull;
    info->internal_energy = s0[0];
    info->plastic_work = s1[0];
    info->sum_ifv = s2[0];
    info->num_term_ifv = num_term;
    info->material_cut_step = cut ? 1 : 0;
    info->first_bad_element = cut ? blocks[st >> 40].felem + (int)(st & 0xFFFFFull) + 1 : 0;
  }
}

}  // namespace

int assemble_ifv_parts(int nodof) { return (nodof + kAsmThreads - 1) / kAsmThreads; }

cudaError_t launch_recover(const DeviceModel& m, const RecoverArgs& a, cudaStream_t s) {
  if (m.nchunks == 0) return cudaSuccess;
  k_recover_hex8<<<m.nchunks, kThreads, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_assemble_ifv(const DeviceModel& m, const double* einf, double* ifv, double* ifv_partials,
                                int nparts, cudaStream_t s) {
  if (m.nodof == 0) return cudaSuccess;
  k_assemble_ifv<<<nparts, kAsmThreads, 0, s>>>(m.nodof, m.ifv_rowptr, m.ifv_src, einf, ifv, ifv_partials);
  return cudaGetLastError();
}

cudaError_t launch_finalize(const DeviceModel& m, const double* partials, const double* ifv_partials, int nparts,
                            const unsigned long long* status, w3g_recover_info* d_info, cudaStream_t s) {
  k_finalize<<<1, 256, 0, s>>>(m.nchunks, partials, nparts, ifv_partials, status, m.blocks, m.einf_total, d_info);
  return cudaGetLastError();
}

}  // namespace w3g
