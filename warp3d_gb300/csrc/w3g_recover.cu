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
constexpr int kGeo = 3 * NN + 1;        // cached dN/dX (24) + det[J0] per GP

// 3x3 inverse of F (column-major) from its cofactors and det[F]
__device__ __forceinline__ void inverse3(const double* F, double det, double* Fi) {
  const double r = 1.0 / det;
  Fi[0] = (F[4] * F[8] - F[7] * F[5]) * r;
  Fi[3] = (F[6] * F[5] - F[3] * F[8]) * r;
  Fi[6] = (F[3] * F[7] - F[6] * F[4]) * r;
  Fi[1] = (F[7] * F[2] - F[1] * F[8]) * r;
  Fi[4] = (F[0] * F[8] - F[6] * F[2]) * r;
  Fi[7] = (F[6] * F[1] - F[0] * F[7]) * r;
  Fi[2] = (F[1] * F[5] - F[4] * F[2]) * r;
  Fi[5] = (F[3] * F[2] - F[0] * F[5]) * r;
  Fi[8] = (F[0] * F[4] - F[3] * F[1]) * r;
}

__global__ void __launch_bounds__(kThreads) k_recover_hex8(RecoverArgs a) {
  __shared__ double sdn[kDnSize];
  __shared__ double sce[kChunk][3 * NN];
  __shared__ double sue[kChunk][TOT];
  __shared__ double sdu[kChunk][TOT];
  __shared__ double sfe[kChunk][NG][TOT + 1];
  __shared__ double sred[2][2];

  const int tid = threadIdx.x;
  const int ge = tid >> 3;
  const int g = tid & 7;
  const int cidx = a.chunk0 + blockIdx.x;
  const Chunk ch = a.chunks[cidx];
  const BlockDesc bd = a.blocks[ch.blk];
  const bool active = ge < ch.n;
  const int i = ch.i0 + ge;
  const bool dirty = *a.geo_dirty != 0;

  for (int k = tid; k < kDnSize; k += kThreads) sdn[k] = a.dn[k];
  if (active) {   // dupstr + dupstr_blocked gathers: lane g loads node g
    const long long dbase = bd.einf_off + (long long)i * TOT;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int j = d * NN + g;
      if (dirty) sce[ge][j] = a.c[a.cdest[dbase + j] - 1];
      const int eidx = a.edest[dbase + j] - 1;
      sue[ge][j] = a.u[eidx];
      sdu[ge][j] = a.du[eidx];
    }
  }
  __syncthreads();

  double vol = 0.0, en = 0.0, pw = 0.0;

  if (active) {
    const int eg = bd.felem + i;   // global element (0-based)
    const MatProps mp = a.mat[eg];
    const double w = sdn[NG * 3 * NN + g];
    const double* ue = &sue[ge][0];
    const double* du = &sdu[ge][0];
    const bool update_coords = bd.geonl && !(a.step == 1 && a.iter == 0);
    const long long gpi = bd.gp_off + (long long)i * NG + g;

    // ---- undeformed geometry: dN/dX and det[J] at t = 0 (jacob1 on the
    // initial coordinates inside gtmat1, src/gtmat1.f:59-63). Constant over
    // the analysis: computed in reference order on the first call after
    // the coordinates change, then read back.
    double tg0[3 * NN], dj0;
    double* geo = a.geo + bd.geo_off + ((long long)i * NG + g) * kGeo;
    if (dirty) {
      const double* dnx = sdn + (g * 3 + 0) * NN;
      const double* dne = sdn + (g * 3 + 1) * NN;
      const double* dnz = sdn + (g * 3 + 2) * NN;
      double gama0[9];
      jacob1_ref<NN>(dnx, dne, dnz, &sce[ge][0], &sce[ge][NN], &sce[ge][2 * NN], gama0, dj0);
#pragma unroll
      for (int n = 0; n < NN; ++n) grad_ref(gama0, dnx[n], dne[n], dnz[n], tg0[3 * n], tg0[3 * n + 1], tg0[3 * n + 2]);
#pragma unroll
      for (int k = 0; k < 3 * NN; ++k) geo[k] = tg0[k];
      geo[3 * NN] = dj0;
    } else {
#pragma unroll
      for (int k = 0; k < 3 * NN; ++k) tg0[k] = geo[k];
      dj0 = geo[3 * NN];
    }

    // ---- gtmat1: tcomp1/fcomp1 for u_{n+1} and u_{n+1/2} (rstgp1_a),
    // reference-order arithmetic up to the polar decompositions
    double th1[9], thh[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) { th1[k] = 0.0; thh[k] = 0.0; }
#pragma unroll
    for (int n = 0; n < NN; ++n) {
      const double tx = tg0[3 * n], ty = tg0[3 * n + 1], tz = tg0[3 * n + 2];
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
    const double F1[9] = {th1[0] + 1.0, th1[1], th1[2], th1[3], th1[4] + 1.0, th1[5], th1[6], th1[7], th1[8] + 1.0};
    const double Fh[9] = {thh[0] + 1.0, thh[1], thh[2], thh[3], thh[4] + 1.0, thh[5], thh[6], thh[7], thh[8] + 1.0};
    const double dfn1 = det_ref(F1);
    const double dfh = det_ref(Fh);
    if (dfn1 <= 1.0e-20) atomicMin(a.status, bad_point_key(ch.blk, g, 0, i));
    else if (dfh <= 1.0e-20) atomicMin(a.status, bad_point_key(ch.blk, g, 1, i));
    double R1[9], Rh[9];
    polar_rotation_ref(F1, R1);
    polar_rotation_ref(Fh, Rh);

    // ---- rate of deformation over the step: d = sym(dDu/dx_mid) with
    // x_mid = X + u + du/2 (gtlsn1 with [B] at the mid-step shape,
    // rknstr_geonl): dDu/dx_mid = (dDu/dX) Fh^-1.
    double L[9];
    {
      double dth[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) dth[k] = 0.0;   // dth[r + 3c] = dDu_r/dX_c
#pragma unroll
      for (int n = 0; n < NN; ++n) {
        const double dx = du[n], dy = du[NN + n], dz = du[2 * NN + n];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const double t = tg0[3 * n + c];
          dth[3 * c + 0] += dx * t; dth[3 * c + 1] += dy * t; dth[3 * c + 2] += dz * t;
        }
      }
      if (update_coords) {
        double Fi[9];
        inverse3(Fh, dfh, Fi);
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int r = 0; r < 3; ++r)
            L[r + 3 * c] = dth[r] * Fi[3 * c] + dth[r + 3] * Fi[1 + 3 * c] + dth[r + 6] * Fi[2 + 3 * c];
      } else {
#pragma unroll
        for (int k = 0; k < 9; ++k) L[k] = dth[k];
      }
    }
    const double ddt[6] = {L[0], L[4], L[8], L[3] + L[1], L[7] + L[5], L[6] + L[2]};
    double uddt[6];
    rotate_to_unrotated(Rh, ddt, uddt);   // qmply1 with getrm1 opt 1 at n+1/2

    // ---- state at n ----
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
#pragma unroll
      for (int k = 0; k < 21; ++k) cep21[k] = 0.0;
      cep21[0] = mp.c2; cep21[1] = mp.c4; cep21[2] = mp.c2; cep21[3] = mp.c4; cep21[4] = mp.c4; cep21[5] = mp.c2;
      cep21[9] = mp.c3; cep21[14] = mp.c3; cep21[20] = mp.c3;
      cgn1[0] = cgn[0] + mp.c2 * uddt[0] + mp.c4 * uddt[1] + mp.c4 * uddt[2];
      cgn1[1] = cgn[1] + mp.c4 * uddt[0] + mp.c2 * uddt[1] + mp.c4 * uddt[2];
      cgn1[2] = cgn[2] + mp.c4 * uddt[0] + mp.c4 * uddt[1] + mp.c2 * uddt[2];
      cgn1[3] = cgn[3] + mp.c3 * uddt[3];
      cgn1[4] = cgn[4] + mp.c3 * uddt[4];
      cgn1[5] = cgn[5] + mp.c3 * uddt[5];
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

    // ---- rknifv_std + gpifv1 (src/rknifv.f:141-217, src/gpifv1.f:16-154):
    // f_a = w det[J_{n+1}] [T] dN_a/dx_{n+1}, with dN/dx_{n+1} = F1^-T dN/dX
    // and det[J_{n+1}] = det[F1] det[J_0], i.e. f_a = P dN_a/dX with
    // P = w det[J_{n+1}] [T] F1^-T.
    double S[6];
    if (bd.geonl) rotate_to_spatial(R1, cgn1, S);
    else {
#pragma unroll
      for (int k = 0; k < 6; ++k) S[k] = cgn1[k];
    }
    double P[9];
    if (update_coords) {
      double Fi[9];
      inverse3(F1, dfn1, Fi);
      const double wdj = w * (dfn1 * dj0);
      const double T[9] = {S[0] * wdj, S[3] * wdj, S[5] * wdj, S[3] * wdj, S[1] * wdj,
                           S[4] * wdj, S[5] * wdj, S[4] * wdj, S[2] * wdj};
      // P_rc = sum_k T_rk Fi_ck
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) P[r + 3 * c] = T[r] * Fi[c] + T[r + 3] * Fi[c + 3] + T[r + 6] * Fi[c + 6];
      vol = wdj;
    } else {
      const double wdj = w * dj0;
      P[0] = S[0] * wdj; P[1] = S[3] * wdj; P[2] = S[5] * wdj;
      P[3] = S[3] * wdj; P[4] = S[1] * wdj; P[5] = S[4] * wdj;
      P[6] = S[5] * wdj; P[7] = S[4] * wdj; P[8] = S[2] * wdj;
      vol = wdj;
    }
    double* fe = &sfe[ge][g][0];
#pragma unroll
    for (int n = 0; n < NN; ++n) {
      const double tx = tg0[3 * n], ty = tg0[3 * n + 1], tz = tg0[3 * n + 2];
      fe[n] = P[0] * tx + P[3] * ty + P[6] * tz;
      fe[NN + n] = P[1] * tx + P[4] * ty + P[7] * tz;
      fe[2 * NN + n] = P[2] * tx + P[5] * ty + P[8] * tz;
    }
  }
  __syncthreads();

  // ---- element forces: lane g sums the dofs of node g over the 8 GPs ----
  if (active) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int j = d * NN + g;
      double v = sfe[ge][0][j];
#pragma unroll
      for (int q = 1; q < NG; ++q) v += sfe[ge][q][j];
      a.einf[bd.einf_off + (long long)j * bd.span + i] = v;
    }
  }
#pragma unroll
  for (int off = 1; off < NG; off <<= 1) {
    vol += __shfl_xor_sync(0xffffffffu, vol, off);
    en += __shfl_xor_sync(0xffffffffu, en, off);
    pw += __shfl_xor_sync(0xffffffffu, pw, off);
  }
  if (active && g == 0) a.evol[bd.felem + i] = vol;
  // ---- chunk energy: sum over the 4 elements of the warp, then warps ----
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

// the undeformed-geometry cache is valid while the coordinates equal the
// ones it was built from; a changed coordinate marks it dirty
__global__ void k_check_coords(const double* __restrict__ c, const double* __restrict__ c_geo, int n, int* dirty) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n && c[k] != c_geo[k]) *dirty = 1;
}

__global__ void k_commit_coords(const double* __restrict__ c, double* c_geo, int n, int* dirty) {
  if (*dirty == 0) return;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) c_geo[k] = c[k];
}

__global__ void k_clear_dirty(int* dirty) { *dirty = 0; }

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

cudaError_t launch_recover(const DeviceModel& m, const RecoverArgs& a, double* c_geo, cudaStream_t s) {
  if (m.nchunks == 0) return cudaSuccess;
  const int nb = (m.ncoord + 255) / 256;
  k_check_coords<<<nb, 256, 0, s>>>(a.c, c_geo, m.ncoord, a.geo_dirty);
  if (m.type_chunks[0] > 0) {
    RecoverArgs h = a;
    h.dn = m.dn_hex8;
    h.chunk0 = m.type_chunk0[0];
    k_recover_hex8<<<m.type_chunks[0], kThreads, 0, s>>>(h);
  }
  cudaError_t e = launch_recover_other(m, a, s);
  if (e != cudaSuccess) return e;
  k_commit_coords<<<nb, 256, 0, s>>>(a.c, c_geo, m.ncoord, a.geo_dirty);
  k_clear_dirty<<<1, 1, 0, s>>>(a.geo_dirty);
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
