// w3g_recover_items.cuh -- one recovery work item: strains, stresses and
// the mm01 update, [D] storage, element internal forces
// (drive_eps_sig_internal_forces / do_nleps_block / rknstr / rstgp1 /
// drive_01_update / rplstr / rknifv / gpifv1) for a chunk of consecutive
// elements of one block, on kRecoverThreads (64) threads with one thread
// per (element, Gauss point):
//
//   8-node brick      8 elements x 8 Gauss points  (recover_item_hex8)
//   20-node brick     2 elements x 32 lanes, 27 Gauss points
//   10-node tet      16 elements x 4 Gauss points  (recover_item_gen)
//
// Element nodal data is staged in shared memory; the element's Gauss-point
// lanes are consecutive, so its internal-force vector, volume and energy
// are summed in a fixed order (shared memory, warp shuffles). All FP64.
// The kinematics (jacob1 at t = 0, tcomp1/fcomp1, the polar
// decompositions) run in the reference's operation order without fused
// multiply-add: that polar decomposition amplifies rounding differences
// to ~1e-9 near F = I. The items are called by the per-type kernels and
// by the persistent work-queue kernel (w3g_recover.cu).
//
// Tetrahedra: the internal-force weights carry 1/6 while the energy
// weights do not (gpifv1.f:43-47, rstgp1.f:5228-5236), as in the
// reference.
#pragma once
#include "w3g_internal.cuh"
#include "w3g_elem.cuh"
#include "w3g_math.cuh"
#include "w3g_umat.cuh"

namespace w3g {

// drive_umat_update at one Gauss point (w3g_umat.cuh): state at n and
// history from the blocked arrays, history at n+1 written when iter > 0,
// F at n from the undeformed gradients (identity for small displacement).
// A UMAT asking for a smaller load step (pnewdt < 1) sets the step-cut key
// of a failed material update (WARP3D's material_cut_step).
template <int NN>
__device__ __forceinline__ void umat_gauss_point(const RecoverArgs& a, const IterParams& p, int blk,
                                                 const BlockDesc& bd, int i, int g, long long gpi, const double* tg0,
                                                 const double* ue, const double* F1, const double* uddt,
                                                 double* cgn1, double* cep21) {
  double fn[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, f1[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  if (bd.geonl) {
    double th[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int n = 0; n < NN; ++n)
      tcomp1_node(th, tg0[3 * n], tg0[3 * n + 1], tg0[3 * n + 2], ue[n], ue[NN + n], ue[2 * NN + n]);
    for (int k = 0; k < 9; ++k) { fn[k] = th[k] + ((k % 4 == 0) ? 1.0 : 0.0); f1[k] = F1[k]; }
  }
  const long long hoff = bd.hist_off + ((long long)i * bd.ngp + g) * kUmatNstatv;
  double hist1[kUmatNstatv];
  // at iteration 0 the recovery is nonlinear exactly when du is extrapolated
  const bool cut = umat_point(a.umat_props + (long long)(bd.felem + i) * kUmatNprops, p.step, p.iter,
                              p.iter == 0 && p.nonlinear, a.dt, bd.felem + i + 1, g + 1, a.urcs_n + gpi * 9,
                              a.eps_n + gpi * 6, uddt, a.hist + hoff, fn, f1, cgn1, hist1, cep21);
  if (p.iter > 0)
    for (int k = 0; k < kUmatNstatv; ++k) a.hist1[hoff + k] = hist1[k];
  if (cut) atomicMin(a.status, bad_point_key(blk, g, 2, i));
}

// the chunk belongs to a block of material model 8 (UMAT): its elements
// take the kUmat instantiation of recover_item_gen, so that the mm01 items
// carry no UMAT code
__device__ __forceinline__ bool umat_chunk(const RecoverArgs& a, int cidx) {
  return a.blocks[a.chunks[cidx].blk].mat == W3G_MAT_UMAT;
}

// shared memory of one recovery item of element type E, EPC elements
template <class E, int EPC>
struct RecoverSmem {
  double dn[E::NG * 3 * E::NN + E::NG];     // fill_dn_table
  double ce[EPC][3 * E::NN];                // initial coordinates (cache rebuild)
  double ue[EPC][E::TOTDOF];                // u
  double du[EPC][E::TOTDOF];                // du
  double fe[EPC][E::NG][E::TOTDOF + 1];     // element forces per Gauss point
  double red[2][2];                         // energy, plastic work per warp
};

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

namespace hex8r {
constexpr int NN = Hex8::NN;
constexpr int NG = Hex8::NG;
constexpr int TOT = Hex8::TOTDOF;
constexpr int kDnSize = NG * 3 * NN + NG;
constexpr int kGeo = 3 * NN + 1;        // cached dN/dX (24) + det[J0] per GP

__device__ __noinline__ void recover_item_hex8(const RecoverArgs& a, const IterParams& p, int cidx,
                                                  unsigned char* smem) {
  RecoverSmem<Hex8, 8>& S = *reinterpret_cast<RecoverSmem<Hex8, 8>*>(smem);
  double* sdn = S.dn;
  auto& sce = S.ce;
  auto& sue = S.ue;
  auto& sdu = S.du;
  auto& sfe = S.fe;
  auto& sred = S.red;

  const int tid = threadIdx.x;
  const int ge = tid >> 3;
  const int g = tid & 7;
  const Chunk ch = a.chunks[cidx];
  const BlockDesc bd = a.blocks[ch.blk];
  const bool active = ge < ch.n;
  const int i = ch.i0 + ge;
  const bool dirty = *a.geo_dirty != 0;

  for (int k = tid; k < kDnSize; k += kRecoverThreads) sdn[k] = a.dn[0][k];
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
    const bool update_coords = bd.geonl && !(p.step == 1 && p.iter == 0);
    const long long gpi = bd.gp_off + (long long)i * NG + g;
    const long long hoff = bd.hist_off + ((long long)i * NG + g) * kHistMM01;

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
    // reference-order arithmetic up to the polar decompositions; small-
    // displacement blocks (rstgp2) have no deformation gradient
    double F1[9], Fh[9], R1[9], Rh[9];
    double dfn1 = 1.0, dfh = 1.0;
    if (bd.geonl) {
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
#pragma unroll
      for (int k = 0; k < 9; ++k) F1[k] = Fh[k] = R1[k] = Rh[k] = (k % 4 == 0) ? 1.0 : 0.0;
    }
    // the element's 8 Gauss-point lanes (b-bar sums over them)
    const unsigned gmask = 0xFFu << (tid & 24);

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
    double ddt[6] = {L[0], L[4], L[8], L[3] + L[1], L[7] + L[5], L[6] + L[2]};
    if (bd.bbar) {
      // b-bar (rknstr vol_terms/vol_avg at the mid-step shape, gtlsn1 with
      // bmod): column (n, k) of B-bar adds beta (v_nk - g_nk) to the three
      // normal rows, so each normal component of d gains beta (tr_bar -
      // tr L), tr_bar = sum_gp det[J_mid] tr L / sum_gp det[J_mid] being the
      // element's mean dilatation rate
      const double jm = update_coords ? dfh * dj0 : dj0;
      const double trl = L[0] + L[4] + L[8];
      double s1 = jm * trl, s0 = jm;
#pragma unroll
      for (int off = 1; off < NG; off <<= 1) {
        s1 += __shfl_xor_sync(gmask, s1, off);
        s0 += __shfl_xor_sync(gmask, s0, off);
      }
      const double cb = a.bbar_beta * (s1 * (1.0 / s0) - trl);
      ddt[0] += cb; ddt[1] += cb; ddt[2] += cb;
    }
    double uddt[6];
    if (bd.geonl) rotate_to_unrotated(Rh, ddt, uddt);   // qmply1 with getrm1 opt 1 at n+1/2
    else {
#pragma unroll
      for (int k = 0; k < 6; ++k) uddt[k] = ddt[k];    // rstgp2: the increment as it is
    }

    // ---- state at n ----
    double cgn[9], hist[11], cgn1[9], hist1[11], cep21[21], eps1[6];
#pragma unroll
    for (int k = 0; k < 9; ++k) cgn[k] = a.urcs_n[gpi * 9 + k];
#pragma unroll
    for (int k = 0; k < 6; ++k) eps1[k] = a.eps_n[gpi * 6 + k] + uddt[k];
#pragma unroll
    for (int k = 0; k < 11; ++k) hist[k] = a.hist[hoff + k];

    // ---- drive_01_update (src/rstgp1.f:614-1034) ----
    if (p.nonlinear) {
      // block's first element, this GP
      const double alpha11_first = a.hist[bd.hist_off + (long long)g * kHistMM01 + 10];
      mm01_point(mp, p.step, cgn, uddt, hist, alpha11_first, cgn1, hist1, cep21);
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
    // rstgp1_b: energy and plastic work (large- or small-strain branch)
    if (p.iter != 0) {
      const double factor = bd.geonl ? dfn1 * dj0 * a.beta_fact * w : dj0 * a.beta_fact * w;
      en = cgn1[6] * factor;
      pw = cgn1[7] * factor;
    }
    // rplstr (src/rplstr.f:15-90)
#pragma unroll
    for (int k = 0; k < 9; ++k) a.urcs_n1[gpi * 9 + k] = cgn1[k];
#pragma unroll
    for (int k = 0; k < 6; ++k) a.eps_n1[gpi * 6 + k] = eps1[k];
    if (p.iter > 0) {
      if (bd.geonl) {
#pragma unroll
        for (int k = 0; k < 9; ++k) a.rot_n1[gpi * 9 + k] = R1[k];
      }
#pragma unroll
      for (int k = 0; k < 11; ++k) a.hist1[hoff + k] = hist1[k];
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
    // b-bar (rknifv vol_terms/vol_avg at n+1, gpifv1 with bmod): B-bar^T
    // {T} = B^T {T} + beta tr(T) (v - g), i.e. each point's pressure part
    // beta tr(T) is replaced by the element's mean, added back as
    // cb det[J_{n+1}] on the diagonal, cb = beta sum_gp w det[J] tr(T) /
    // sum_gp det[J]
    const double j1 = update_coords ? dfn1 * dj0 : dj0;
    double pdiag = 0.0;
    if (bd.bbar) {
      const double trs = S[0] + S[1] + S[2];
      double s1 = w * j1 * trs, s0 = j1;
#pragma unroll
      for (int off = 1; off < NG; off <<= 1) {
        s1 += __shfl_xor_sync(gmask, s1, off);
        s0 += __shfl_xor_sync(gmask, s0, off);
      }
      const double ptr = a.bbar_beta * trs;
      S[0] -= ptr; S[1] -= ptr; S[2] -= ptr;
      pdiag = a.bbar_beta * (s1 * (1.0 / s0)) * j1;
    }
    double P[9];
    if (update_coords) {
      double Fi[9];
      inverse3(F1, dfn1, Fi);
      const double wdj = w * j1;
      const double T[9] = {S[0] * wdj + pdiag, S[3] * wdj, S[5] * wdj, S[3] * wdj, S[1] * wdj + pdiag,
                           S[4] * wdj, S[5] * wdj, S[4] * wdj, S[2] * wdj + pdiag};
      // P_rc = sum_k T_rk Fi_ck
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) P[r + 3 * c] = T[r] * Fi[c] + T[r + 3] * Fi[c + 3] + T[r + 6] * Fi[c + 6];
      vol = wdj;
    } else {
      const double wdj = w * j1;
      P[0] = S[0] * wdj + pdiag; P[1] = S[3] * wdj; P[2] = S[5] * wdj;
      P[3] = S[3] * wdj; P[4] = S[1] * wdj + pdiag; P[5] = S[4] * wdj;
      P[6] = S[5] * wdj; P[7] = S[4] * wdj; P[8] = S[2] * wdj + pdiag;
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

}  // namespace hex8r
using hex8r::recover_item_hex8;

// kUmat: the instantiation for blocks of material model 8 (UMAT); the
// others run mm01
template <class E, int LPE, int EPC, bool kUmat = false>
__device__ __noinline__ void recover_item_gen(const RecoverArgs& a, const IterParams& p, int cidx,
                                                 unsigned char* smem) {
  constexpr int NN = E::NN, NG = E::NG, TOT = E::TOTDOF;
  constexpr int NT = LPE * EPC;
  constexpr int GEO = 3 * NN + 1;
  constexpr int DN = NG * 3 * NN + NG;
  static_assert(NT == kRecoverThreads, "recovery items run on kRecoverThreads threads");
  static_assert(NG <= LPE && (LPE & (LPE - 1)) == 0 && LPE <= 32, "one Gauss point per lane, power-of-two lanes");
  RecoverSmem<E, EPC>& S = *reinterpret_cast<RecoverSmem<E, EPC>*>(smem);
  double* sdn = S.dn;
  auto& sce = S.ce;
  auto& sue = S.ue;
  auto& sdu = S.du;
  auto& sfe = S.fe;
  auto& sred = S.red;

  const int tid = threadIdx.x;
  const int ge = tid / LPE;
  const int g = tid % LPE;
  const Chunk ch = a.chunks[cidx];
  const BlockDesc bd = a.blocks[ch.blk];
  const bool active = ge < ch.n;
  const bool gp_active = active && g < NG;
  const int i = ch.i0 + ge;
  const bool dirty = *a.geo_dirty != 0;

  for (int k = tid; k < DN; k += NT) sdn[k] = a.dn[E::SLOT][k];
  if (active) {
    const long long dbase = bd.einf_off + (long long)i * TOT;
    for (int node = g; node < NN; node += LPE) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const int j = d * NN + node;
        if (dirty) sce[ge][j] = a.c[a.cdest[dbase + j] - 1];
        const int eidx = a.edest[dbase + j] - 1;
        sue[ge][j] = a.u[eidx];
        sdu[ge][j] = a.du[eidx];
      }
    }
  }
  __syncthreads();

  double vol = 0.0, en = 0.0, pw = 0.0;
  if (gp_active) {
    const int eg = bd.felem + i;
    const MatProps mp = a.mat[eg];
    const double w = sdn[NG * 3 * NN + g];
    const double wf = E::TET ? w * (1.0 / 6.0) : w;   // gpifv1 weight
    const double* ue = &sue[ge][0];
    const double* du = &sdu[ge][0];
    const bool update_coords = bd.geonl && !(p.step == 1 && p.iter == 0);
    const long long gpi = bd.gp_off + (long long)i * NG + g;
    const long long hoff = bd.hist_off + ((long long)i * NG + g) * kHistMM01;

    // undeformed geometry (jacob1 on the initial coordinates), cached
    double* geo = a.geo + bd.geo_off + ((long long)i * NG + g) * GEO;
    if (dirty) {
      const double* dnx = sdn + (g * 3 + 0) * NN;
      const double* dne = sdn + (g * 3 + 1) * NN;
      const double* dnz = sdn + (g * 3 + 2) * NN;
      double gama0[9], dj0w;
      jacob1_ref<NN>(dnx, dne, dnz, &sce[ge][0], &sce[ge][NN], &sce[ge][2 * NN], gama0, dj0w);
      for (int n = 0; n < NN; ++n) {
        double tx, ty, tz;
        grad_ref(gama0, dnx[n], dne[n], dnz[n], tx, ty, tz);
        geo[3 * n] = tx; geo[3 * n + 1] = ty; geo[3 * n + 2] = tz;
      }
      geo[3 * NN] = dj0w;
    }
    const double* tg0 = geo;   // dN/dX per node (own writes, or the cache)
    const double dj0 = geo[3 * NN];

    // tcomp1/fcomp1 at n+1 and n+1/2, reference order (geonl blocks;
    // rstgp2 has no deformation gradient)
    double F1[9], Fh[9], R1[9], Rh[9];
    double dfn1 = 1.0, dfh = 1.0;
    if (bd.geonl) {
      double th1[9], thh[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) { th1[k] = 0.0; thh[k] = 0.0; }
      for (int n = 0; n < NN; ++n) {
        const double tx = tg0[3 * n], ty = tg0[3 * n + 1], tz = tg0[3 * n + 2];
        const double u1x = ra(ue[n], du[n]), u1y = ra(ue[NN + n], du[NN + n]),
                     u1z = ra(ue[2 * NN + n], du[2 * NN + n]);
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
#pragma unroll
      for (int k = 0; k < 9; ++k) F1[k] = Fh[k] = R1[k] = Rh[k] = (k % 4 == 0) ? 1.0 : 0.0;
    }

    // d = sym(dDu/dX Fh^-1)
    double L[9], dth[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) dth[k] = 0.0;
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
        for (int rr = 0; rr < 3; ++rr)
          L[rr + 3 * c] = dth[rr] * Fi[3 * c] + dth[rr + 3] * Fi[1 + 3 * c] + dth[rr + 6] * Fi[2 + 3 * c];
    } else {
#pragma unroll
      for (int k = 0; k < 9; ++k) L[k] = dth[k];
    }
    const double ddt[6] = {L[0], L[4], L[8], L[3] + L[1], L[7] + L[5], L[6] + L[2]};
    double uddt[6];
    if (bd.geonl) rotate_to_unrotated(Rh, ddt, uddt);
    else {
#pragma unroll
      for (int k = 0; k < 6; ++k) uddt[k] = ddt[k];
    }

    double cgn[9], hist[11], cgn1[9], hist1[11], cep21[21], eps1[6];
#pragma unroll
    for (int k = 0; k < 9; ++k) cgn[k] = a.urcs_n[gpi * 9 + k];
#pragma unroll
    for (int k = 0; k < 6; ++k) eps1[k] = a.eps_n[gpi * 6 + k] + uddt[k];
    if constexpr (!kUmat) {
#pragma unroll
      for (int k = 0; k < 11; ++k) hist[k] = a.hist[hoff + k];
    }
    if constexpr (kUmat) {   // drive_umat_update
      umat_gauss_point<NN>(a, p, ch.blk, bd, i, g, gpi, tg0, ue, F1, uddt, cgn1, cep21);
    } else if (p.nonlinear) {
      const double alpha11_first = a.hist[bd.hist_off + (long long)g * kHistMM01 + 10];
      mm01_point(mp, p.step, cgn, uddt, hist, alpha11_first, cgn1, hist1, cep21);
    } else {
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
    double* cp = a.cep + bd.cep_off + ((long long)g * bd.span + i) * 21;
#pragma unroll
    for (int k = 0; k < 21; ++k) cp[k] = cep21[k];
    if (p.iter != 0) {   // rstgp1_b: weight without the tetrahedral 1/6
      const double factor = bd.geonl ? dfn1 * dj0 * a.beta_fact * w : dj0 * a.beta_fact * w;
      en = cgn1[6] * factor;
      pw = cgn1[7] * factor;
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) a.urcs_n1[gpi * 9 + k] = cgn1[k];
#pragma unroll
    for (int k = 0; k < 6; ++k) a.eps_n1[gpi * 6 + k] = eps1[k];
    if (p.iter > 0) {
      if (bd.geonl) {
#pragma unroll
        for (int k = 0; k < 9; ++k) a.rot_n1[gpi * 9 + k] = R1[k];
      }
      if constexpr (!kUmat) {
#pragma unroll
        for (int k = 0; k < 11; ++k) a.hist1[hoff + k] = hist1[k];
      }
    }

    // element forces f_a = P dN_a/dX, P = wf det[J_{n+1}] [T] F1^-T
    double Sg[6];
    if (bd.geonl) rotate_to_spatial(R1, cgn1, Sg);
    else {
#pragma unroll
      for (int k = 0; k < 6; ++k) Sg[k] = cgn1[k];
    }
    double P[9];
    const double wdj = update_coords ? wf * (dfn1 * dj0) : wf * dj0;
    const double Tm[9] = {Sg[0] * wdj, Sg[3] * wdj, Sg[5] * wdj, Sg[3] * wdj, Sg[1] * wdj,
                          Sg[4] * wdj, Sg[5] * wdj, Sg[4] * wdj, Sg[2] * wdj};
    if (update_coords) {
      double Fi[9];
      inverse3(F1, dfn1, Fi);
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int rr = 0; rr < 3; ++rr)
          P[rr + 3 * c] = Tm[rr] * Fi[c] + Tm[rr + 3] * Fi[c + 3] + Tm[rr + 6] * Fi[c + 6];
    } else {
#pragma unroll
      for (int k = 0; k < 9; ++k) P[k] = Tm[k];
    }
    vol = wdj;
    double* fe = &sfe[ge][g][0];
    for (int n = 0; n < NN; ++n) {
      const double tx = tg0[3 * n], ty = tg0[3 * n + 1], tz = tg0[3 * n + 2];
      fe[n] = P[0] * tx + P[3] * ty + P[6] * tz;
      fe[NN + n] = P[1] * tx + P[4] * ty + P[7] * tz;
      fe[2 * NN + n] = P[2] * tx + P[5] * ty + P[8] * tz;
    }
  }
  __syncthreads();

  if (active) {
    for (int j = g; j < TOT; j += LPE) {
      double v = sfe[ge][0][j];
      for (int q = 1; q < NG; ++q) v += sfe[ge][q][j];
      a.einf[bd.einf_off + (long long)j * bd.span + i] = v;
    }
  }
#pragma unroll
  for (int off = 1; off < LPE; off <<= 1) {
    vol += __shfl_xor_sync(0xffffffffu, vol, off);
    en += __shfl_xor_sync(0xffffffffu, en, off);
    pw += __shfl_xor_sync(0xffffffffu, pw, off);
  }
  if (active && g == 0) a.evol[bd.felem + i] = vol;
  // chunk energy: the per-element sums are replicated on LPE lanes; reduce
  // one lane per element over the warp, then over warps
  double e1 = (g == 0) ? en : 0.0, p1 = (g == 0) ? pw : 0.0;
#pragma unroll
  for (int off = LPE; off < 32; off <<= 1) {
    e1 += __shfl_xor_sync(0xffffffffu, e1, off);
    p1 += __shfl_xor_sync(0xffffffffu, p1, off);
  }
  if ((tid & 31) == 0) { sred[tid >> 5][0] = e1; sred[tid >> 5][1] = p1; }
  __syncthreads();
  if (tid == 0) {
    double te = 0.0, tp = 0.0;
    for (int k = 0; k < (NT + 31) / 32; ++k) { te += sred[k][0]; tp += sred[k][1]; }
    a.partials[2 * cidx + 0] = te;
    a.partials[2 * cidx + 1] = tp;
  }
}


}  // namespace w3g
