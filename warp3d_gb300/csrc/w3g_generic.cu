// w3g_generic.cu -- tangent and recovery kernels for the 20-node brick
// (q3disop, 27 Gauss points) and the 10-node tetrahedron (4 Gauss points),
// templated on the element. Same algorithms as the 8-node kernels in
// w3g_tangent.cu / w3g_recover.cu; the work decomposition scales with the
// element:
//
//   tangent   LPE lanes per element (32 for hex20, 8 for tet10), one Gauss
//             point per lane in phase 1 (NG <= LPE), then per Gauss point
//             [D*][B_b] and {T}g_b for every node in shared memory and the
//             NN(NN+1)/2 node-pair blocks of Ke dealt round-robin to the
//             lanes (7 pairs per lane for both elements), accumulated in
//             registers with fused multiply-add chains.
//   recovery  one lane per Gauss point (LPE = 32 for hex20, 4 for tet10),
//             the reference-order kinematics chain, mm01 and the element
//             forces, summed over the element's Gauss points in shared
//             memory.
//
// Tetrahedra: [D] is scaled by 1/6 after ctran1 but the geometric
// stiffness is not (gptns1.f:222-225, kg1.f), and the internal-force
// weights carry 1/6 while the energy weights do not (gpifv1.f:43-47,
// rstgp1.f:5228-5236), as in the reference.
#include <climits>
#include "w3g_internal.cuh"
#include "w3g_elem.cuh"
#include "w3g_math.cuh"

namespace w3g {

namespace {

__host__ __device__ constexpr int low6(int r, int c) { return r >= c ? r * (r + 1) / 2 + c : c * (c + 1) / 2 + r; }

template <class E>
struct GenShape {
  static constexpr int NN = E::NN, NG = E::NG, TOT = E::TOTDOF, UT = E::UTSZ;
  static constexpr int NP = NN * (NN + 1) / 2;
  static constexpr int DN = NG * 3 * NN + NG;
  static constexpr int WORK = NG * (3 * NN + 21 + 6) + NN * 21;
  static constexpr int PER_ELEM = 3 * NN + (WORK > UT ? WORK : UT);
};

// ---------------------------------------------------------------------
// tangent
// ---------------------------------------------------------------------
template <class E, int LPE, int EPC, class T, bool kRel>
__global__ void __launch_bounds__(LPE * EPC) k_tangent_gen(TangentArgs a) {
  using S = GenShape<E>;
  constexpr int NN = S::NN, NG = S::NG, TOT = S::TOT, UT = S::UT, NP = S::NP;
  constexpr int PPL = (NP + LPE - 1) / LPE;
  static_assert(NG <= LPE, "one Gauss point per lane in phase 1");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sdn = reinterpret_cast<T*>(smem_raw);
  T* selem = sdn + S::DN;
  __shared__ unsigned char pa[NP], pb[NP];

  const int tid = threadIdx.x;
  const int ge = tid / LPE;
  const int l = tid % LPE;
  const Chunk ch = a.chunks[a.chunk0 + blockIdx.x];
  const BlockDesc bd = a.blocks[ch.blk];
  const bool active = ge < ch.n;
  const int i = ch.i0 + ge;

  for (int k = tid; k < S::DN; k += LPE * EPC) sdn[k] = (T)a.dn[k];
  if (tid == 0) {
    int k = 0;
    for (int x = 0; x < NN; ++x)
      for (int y = x; y < NN; ++y) { pa[k] = (unsigned char)x; pb[k] = (unsigned char)y; ++k; }
  }
  T* Eb = selem + ge * S::PER_ELEM;
  T* sx = Eb;
  T* sy = Eb + NN;
  T* sz = Eb + 2 * NN;
  T* sg = Eb + 3 * NN;            // [gp][a][3]
  T* sD = sg + NG * 3 * NN;       // [gp][21]
  T* sT = sD + NG * 21;           // [gp][6]
  T* sDB = sT + NG * 6;           // [a][6][3]
  T* sTg = sDB + NN * 18;         // [a][3]

  if (active) {   // dptstf gather
    const long long dbase = bd.einf_off + (long long)i * TOT;
    double ref[3] = {0.0, 0.0, 0.0};
    if (kRel) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        double v = a.c[a.cdest[dbase + d * NN] - 1];
        if (bd.geonl) { const int e = a.edest[dbase + d * NN] - 1; v = v + a.u[e] + a.du[e]; }
        ref[d] = v;
      }
    }
    for (int node = l; node < NN; node += LPE) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        double v = a.c[a.cdest[dbase + d * NN + node] - 1];
        if (bd.geonl) { const int e = a.edest[dbase + d * NN + node] - 1; v = v + a.u[e] + a.du[e]; }
        Eb[d * NN + node] = (T)(v - ref[d]);
      }
    }
  }
  __syncthreads();

  // ---- phase 1: Gauss point l ----
  if (active && l < NG) {
    const int gp = l;
    const T* dnx = sdn + (gp * 3 + 0) * NN;
    const T* dne = sdn + (gp * 3 + 1) * NN;
    const T* dnz = sdn + (gp * 3 + 2) * NN;
    const T w = sdn[NG * 3 * NN + gp];
    T gama[9], dj;
    jacobian_inverse<NN, T>(dnx, dne, dnz, sx, sy, sz, gama, dj);
    T* g = sg + gp * 3 * NN;
    for (int n = 0; n < NN; ++n)
      shape_gradient<T>(gama, dnx[n], dne[n], dnz[n], g[3 * n], g[3 * n + 1], g[3 * n + 2]);
    const T f = w * dj;
    T C[21];
    const double* cp = a.cep + bd.cep_off + ((long long)gp * bd.span + i) * 21;
#pragma unroll
    for (int k = 0; k < 21; ++k) C[k] = f * (T)cp[k];
    T* D = sD + gp * 21;
    T* Tw = sT + gp * 6;
    const long long gpi = bd.gp_off + (long long)i * NG + gp;
    if (bd.geonl) {
      T R[9], q[36], ur[6], cs[6];
#pragma unroll
      for (int k = 0; k < 9; ++k) R[k] = (T)a.rot_n1[gpi * 9 + k];
#pragma unroll
      for (int k = 0; k < 6; ++k) ur[k] = (T)a.urcs_n1[gpi * 9 + k];
      rotation_q2<T>(R, q);
      qmply<T>(q, ur, cs);
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        T tc[6];
#pragma unroll
        for (int kk = 0; kk < 6; ++kk) {
          T s = T(0);
#pragma unroll
          for (int m = 0; m < 6; ++m) s += q[6 * j + m] * C[low6(m, kk)];
          tc[kk] = s;
        }
#pragma unroll
        for (int kk = 0; kk <= j; ++kk) {
          T s = T(0);
#pragma unroll
          for (int m = 0; m < 6; ++m) s += tc[m] * q[6 * kk + m];
          D[low6(j, kk)] = s;
        }
      }
      if (a.qbar) {   // ctran1_qbar
        const T wf = dj * w, halfw = T(0.5) * wf;
        const T xx = cs[0], yy = cs[1], zz = cs[2], xy = cs[3], yz = cs[4], xz = cs[5];
        D[low6(0, 0)] -= T(2) * xx * wf;
        D[low6(1, 1)] -= T(2) * yy * wf;
        D[low6(2, 2)] -= T(2) * zz * wf;
        D[low6(3, 0)] -= xy * wf;
        D[low6(5, 0)] -= xz * wf;
        D[low6(3, 1)] -= xy * wf;
        D[low6(4, 1)] -= yz * wf;
        D[low6(4, 2)] -= yz * wf;
        D[low6(5, 2)] -= xz * wf;
        D[low6(3, 3)] -= halfw * (xx + yy);
        D[low6(4, 4)] -= halfw * (yy + zz);
        D[low6(5, 5)] -= halfw * (xx + zz);
        D[low6(4, 3)] -= wf * xz;
        D[low6(5, 3)] -= wf * yz;
        D[low6(5, 4)] -= wf * xy;
      }
#pragma unroll
      for (int k = 0; k < 6; ++k) Tw[k] = cs[k] * f;
    } else {
#pragma unroll
      for (int k = 0; k < 21; ++k) D[k] = C[k];
#pragma unroll
      for (int k = 0; k < 6; ++k) Tw[k] = T(0);
    }
    if (E::TET) {   // adjust_cnst: [D] x 1/6; {T}w (geometric stiffness) unscaled
      const T scalar = T(1.0 / 6.0);
#pragma unroll
      for (int k = 0; k < 21; ++k) D[k] = scalar * D[k];
    }
  }
  __syncthreads();

  T acc[PPL][9];
#pragma unroll
  for (int p = 0; p < PPL; ++p)
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[p][k] = T(0);

  for (int gp = 0; gp < NG; ++gp) {
    if (active) {
      const T* D = sD + gp * 21;
      const T* Tw = sT + gp * 6;
      const T* g = sg + gp * 3 * NN;
      for (int n = l; n < NN; n += LPE) {
        const T gx = g[3 * n], gy = g[3 * n + 1], gz = g[3 * n + 2];
        T* db = sDB + n * 18;
#pragma unroll
        for (int m = 0; m < 6; ++m) {
          db[m * 3 + 0] = D[low6(m, 0)] * gx + D[low6(m, 3)] * gy + D[low6(m, 5)] * gz;
          db[m * 3 + 1] = D[low6(m, 1)] * gy + D[low6(m, 3)] * gx + D[low6(m, 4)] * gz;
          db[m * 3 + 2] = D[low6(m, 2)] * gz + D[low6(m, 4)] * gy + D[low6(m, 5)] * gx;
        }
        T* tg = sTg + n * 3;
        tg[0] = Tw[0] * gx + Tw[3] * gy + Tw[5] * gz;
        tg[1] = Tw[3] * gx + Tw[1] * gy + Tw[4] * gz;
        tg[2] = Tw[5] * gx + Tw[4] * gy + Tw[2] * gz;
      }
    }
    __syncthreads();
    if (active) {
      const T* g = sg + gp * 3 * NN;
#pragma unroll
      for (int p = 0; p < PPL; ++p) {
        const int k = p * LPE + l;
        if (k < NP) {
          const int na = pa[k], nb = pb[k];
          const T ax = g[3 * na], ay = g[3 * na + 1], az = g[3 * na + 2];
          const T* db = sDB + nb * 18;
#pragma unroll
          for (int kk = 0; kk < 3; ++kk) {
            acc[p][0 * 3 + kk] = fma(ax, db[0 * 3 + kk], fma(ay, db[3 * 3 + kk], fma(az, db[5 * 3 + kk], acc[p][0 * 3 + kk])));
            acc[p][1 * 3 + kk] = fma(ay, db[1 * 3 + kk], fma(ax, db[3 * 3 + kk], fma(az, db[4 * 3 + kk], acc[p][1 * 3 + kk])));
            acc[p][2 * 3 + kk] = fma(az, db[2 * 3 + kk], fma(ay, db[4 * 3 + kk], fma(ax, db[5 * 3 + kk], acc[p][2 * 3 + kk])));
          }
          if (bd.geonl) {   // kgstiff
            const T* tg = sTg + nb * 3;
            const T gtg = ax * tg[0] + ay * tg[1] + az * tg[2];
            acc[p][0] += gtg; acc[p][4] += gtg; acc[p][8] += gtg;
          }
        }
      }
    }
    __syncthreads();
  }

  // ---- store: column-packed upper triangle ----
  T* ke = Eb + 3 * NN;
  if (active) {
    const T bf = (T)a.beta_fact;
#pragma unroll
    for (int p = 0; p < PPL; ++p) {
      const int k = p * LPE + l;
      if (k < NP) {
        const int na = pa[k], nb = pb[k];
#pragma unroll
        for (int ii = 0; ii < 3; ++ii)
#pragma unroll
          for (int kk = 0; kk < 3; ++kk) {
            if (na == nb && ii > kk) continue;
            int r = ii * NN + na, c = kk * NN + nb;
            if (r > c) { int tt = r; r = c; c = tt; }
            ke[c * (c + 1) / 2 + r] = acc[p][ii * 3 + kk] * bf;
          }
      }
    }
  }
  __syncthreads();
  using KOut = T;
  KOut* out = reinterpret_cast<KOut*>(a.estiff);
  const long long obase = bd.estiff_off + (long long)ch.i0 * UT;
  for (int e = 0; e < ch.n; ++e) {
    const T* src = selem + e * S::PER_ELEM + 3 * NN;
    for (int k = tid; k < UT; k += LPE * EPC) out[obase + (long long)e * UT + k] = src[k];
  }
}

// ---------------------------------------------------------------------
// recovery
// ---------------------------------------------------------------------
template <class E, int LPE, int EPC>
__global__ void __launch_bounds__(LPE * EPC) k_recover_gen(RecoverArgs a) {
  using S = GenShape<E>;
  constexpr int NN = S::NN, NG = S::NG, TOT = S::TOT;
  constexpr int NT = LPE * EPC;
  constexpr int GEO = 3 * NN + 1;
  static_assert(NG <= LPE && (LPE & (LPE - 1)) == 0, "one Gauss point per lane, power-of-two lanes");
  __shared__ double sdn[S::DN];
  __shared__ double sce[EPC][3 * NN];
  __shared__ double sue[EPC][TOT];
  __shared__ double sdu[EPC][TOT];
  __shared__ double sfe[EPC][NG][TOT + 1];
  __shared__ double sred[NT / 32 > 0 ? NT / 32 : 1][2];

  const int tid = threadIdx.x;
  const int ge = tid / LPE;
  const int g = tid % LPE;
  const int cidx = a.chunk0 + blockIdx.x;
  const Chunk ch = a.chunks[cidx];
  const BlockDesc bd = a.blocks[ch.blk];
  const bool active = ge < ch.n;
  const bool gp_active = active && g < NG;
  const int i = ch.i0 + ge;
  const bool dirty = *a.geo_dirty != 0;

  for (int k = tid; k < S::DN; k += NT) sdn[k] = a.dn[k];
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
    const bool update_coords = bd.geonl && !(a.step == 1 && a.iter == 0);
    const long long gpi = bd.gp_off + (long long)i * NG + g;

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

    // tcomp1/fcomp1 at n+1 and n+1/2, reference order
    double th1[9], thh[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) { th1[k] = 0.0; thh[k] = 0.0; }
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
      const double r = 1.0 / dfh;
      Fi[0] = (Fh[4] * Fh[8] - Fh[7] * Fh[5]) * r; Fi[3] = (Fh[6] * Fh[5] - Fh[3] * Fh[8]) * r;
      Fi[6] = (Fh[3] * Fh[7] - Fh[6] * Fh[4]) * r; Fi[1] = (Fh[7] * Fh[2] - Fh[1] * Fh[8]) * r;
      Fi[4] = (Fh[0] * Fh[8] - Fh[6] * Fh[2]) * r; Fi[7] = (Fh[6] * Fh[1] - Fh[0] * Fh[7]) * r;
      Fi[2] = (Fh[1] * Fh[5] - Fh[4] * Fh[2]) * r; Fi[5] = (Fh[3] * Fh[2] - Fh[0] * Fh[5]) * r;
      Fi[8] = (Fh[0] * Fh[4] - Fh[3] * Fh[1]) * r;
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
    rotate_to_unrotated(Rh, ddt, uddt);

    double cgn[9], hist[11], cgn1[9], hist1[11], cep21[21], eps1[6];
#pragma unroll
    for (int k = 0; k < 9; ++k) cgn[k] = a.urcs_n[gpi * 9 + k];
#pragma unroll
    for (int k = 0; k < 6; ++k) eps1[k] = a.eps_n[gpi * 6 + k] + uddt[k];
#pragma unroll
    for (int k = 0; k < 11; ++k) hist[k] = a.hist[gpi * kHistMM01 + k];
    if (a.nonlinear) {
      const double alpha11_first = a.hist[(bd.gp_off + g) * kHistMM01 + 10];
      mm01_point(mp, a.step, cgn, uddt, hist, alpha11_first, cgn1, hist1, cep21);
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
    if (a.iter != 0) {   // rstgp1_b: weight without the tetrahedral 1/6
      const double factor = dfn1 * dj0 * a.beta_fact * w;
      en = cgn1[6] * factor;
      pw = cgn1[7] * factor;
    }
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
      const double r = 1.0 / dfn1;
      Fi[0] = (F1[4] * F1[8] - F1[7] * F1[5]) * r; Fi[3] = (F1[6] * F1[5] - F1[3] * F1[8]) * r;
      Fi[6] = (F1[3] * F1[7] - F1[6] * F1[4]) * r; Fi[1] = (F1[7] * F1[2] - F1[1] * F1[8]) * r;
      Fi[4] = (F1[0] * F1[8] - F1[6] * F1[2]) * r; Fi[7] = (F1[6] * F1[1] - F1[0] * F1[7]) * r;
      Fi[2] = (F1[1] * F1[5] - F1[4] * F1[2]) * r; Fi[5] = (F1[3] * F1[2] - F1[0] * F1[5]) * r;
      Fi[8] = (F1[0] * F1[4] - F1[3] * F1[1]) * r;
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

template <class E, int LPE, int EPC, class T, bool kRel>
cudaError_t launch_tangent_gen(const TangentArgs& a, int nchunks, cudaStream_t s) {
  if (nchunks == 0) return cudaSuccess;
  using S = GenShape<E>;
  const size_t smem = sizeof(T) * (size_t)(S::DN + EPC * S::PER_ELEM);
  auto kern = k_tangent_gen<E, LPE, EPC, T, kRel>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  kern<<<nchunks, LPE * EPC, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_tangent_other(const DeviceModel& m, TangentArgs a, bool fp32, cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  // hex20: 32 lanes per element, 2 elements per CTA; tet10: 8 lanes, 8 elements
  if (m.type_chunks[1] > 0) {
    a.dn = m.dn_hex20;
    a.chunk0 = m.type_chunk0[1];
    e = fp32 ? launch_tangent_gen<Hex20, 32, 2, float, true>(a, m.type_chunks[1], s)
             : launch_tangent_gen<Hex20, 32, 2, double, false>(a, m.type_chunks[1], s);
    if (e != cudaSuccess) return e;
  }
  if (m.type_chunks[2] > 0) {
    a.dn = m.dn_tet10;
    a.chunk0 = m.type_chunk0[2];
    e = fp32 ? launch_tangent_gen<Tet10, 8, 8, float, true>(a, m.type_chunks[2], s)
             : launch_tangent_gen<Tet10, 8, 8, double, false>(a, m.type_chunks[2], s);
  }
  return e;
}

cudaError_t launch_recover_other(const DeviceModel& m, RecoverArgs a, cudaStream_t s) {
  if (m.type_chunks[1] > 0) {
    a.dn = m.dn_hex20;
    a.chunk0 = m.type_chunk0[1];
    k_recover_gen<Hex20, 32, 2><<<m.type_chunks[1], 64, 0, s>>>(a);
  }
  if (m.type_chunks[2] > 0) {
    a.dn = m.dn_tet10;
    a.chunk0 = m.type_chunk0[2];
    k_recover_gen<Tet10, 4, 8><<<m.type_chunks[2], 32, 0, s>>>(a);
  }
  return cudaGetLastError();
}

}  // namespace w3g
