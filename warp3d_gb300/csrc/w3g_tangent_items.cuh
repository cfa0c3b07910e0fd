// w3g_tangent_items.cuh -- one tangent work item: the element tangent
// stiffnesses (tanstf/rktstf/gptns1 with bdbtgen, ctran1 + Q-bar and
// kgstiff) of a chunk of consecutive elements of one block, on one warp.
// Called by the per-type kernels and the persistent work-queue kernel
// (w3g_tangent.cu).
//
// 8-node brick, 8 elements per item, 4 lanes per element:
//   gather   lane t loads nodes 2t, 2t+1: coordinates (cdest), u and du
//            (edest) -> x_{n+1} = (c + u) + du in shared memory (dptstf.f)
//   phase 1  (per half of the 8 Gauss points) lane t handles GP 4h+t:
//            jacobian/inverse at x_{n+1} (jacob1), shape gradients,
//            [D] = w det[J] cep (extract_D_symmetric), Cauchy stress
//            {T} = [q(R_{n+1})]{t} and [D*] = [q][D][q]^T - [Q-bar]
//            (getrm1 opt 2, qmply1, ctran1); writes gradients, [D*] and
//            w det[J] {T} to shared memory
//   phase 2  per GP: lane t forms [D*][B_a] and {T}g_a for nodes 2t, 2t+1
//            (shared memory), then accumulates 9 of the 36 node-pair
//            3x3 blocks of Ke = sum_gp B^T D* B + G^T T G in registers
//            with fused multiply-add chains. Each lane owns 2 diagonal
//            and 7 off-diagonal pairs, so every lane does the same work.
//   store    Ke is assembled in shared memory in WARP3D's column-packed
//            upper triangle and written with coalesced stores; the chunk's
//            elements are contiguous in estiff (utsz, span).
//
// 20-node brick (1 element per item, 32 lanes) and 10-node tetrahedron
// (4 elements per item, 8 lanes each), tangent_item_gen: phase 1 takes
// all Gauss points at once (one per lane), phase 2 deals the NN(NN+1)/2
// node-pair blocks round-robin to the element's lanes (7 per lane for
// both types). Tetrahedra scale [D] by 1/6 after ctran1 but not the
// geometric stiffness (gptns1.f:222-225, kg1.f), as the reference does.
//
// The FP64 instantiations are the plain form. FP32 is the precision form:
// same algorithm in float, coordinates relative to the element's first
// node (exactly representable offsets), Ke stored as float.
#pragma once
#include "w3g_internal.cuh"
#include "w3g_elem.cuh"
#include "w3g_math.cuh"

namespace w3g {

// lower-triangle index of the symmetric 6x6 (r, c), 0-based
__host__ __device__ __forceinline__ constexpr int low(int r, int c) {
  return r >= c ? r * (r + 1) / 2 + c : c * (c + 1) / 2 + r;
}

// w det[J] [D] of Gauss point gp of element i, lower triangle row-wise:
// from cep_blocks (extract_D_symmetric, gptns1.f:1174-1266) or, for mm10,
// from history1(1:36) (drive_10_cnst, gptns1.f:1371-1455; symmetric)
template <class T, int NG>
__device__ __forceinline__ void load_D21(const TangentArgs& a, const BlockDesc& bd, int i, int gp, T f, T* C) {
  if (bd.mat == W3G_MAT_CRYSTAL) {
    const double* h1 = a.hist1 + bd.hist_off + ((long long)i * NG + gp) * kHistMM10;
    int k = 0;
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
      for (int c = 0; c <= r; ++c) C[k++] = f * from_f64<T>(h1[r + 6 * c]);
  } else {
    const double* cp = a.cep + bd.cep_off + ((long long)gp * bd.span + i) * 21;
#pragma unroll
    for (int k = 0; k < 21; ++k) C[k] = f * from_f64<T>(cp[k]);
  }
}

namespace hex8t {
constexpr int NN = Hex8::NN;
constexpr int NG = Hex8::NG;
constexpr int TOT = Hex8::TOTDOF;
constexpr int UT = Hex8::UTSZ;
constexpr int kHalf = 4;                     // GPs per phase-1 pass
constexpr int kPerElem = 3 * NN              // coordinates
                         + kHalf * (3 * NN + 21 + 6)   // gradients, D*, {T}w
                         + NN * 18 + NN * 3;           // D*B per node, {T}g per node
constexpr int kDnSize = NG * 3 * NN + NG;

// b-bar blocks add per element the volume-averaged gradients v (24), and
// per node of the current Gauss point h = beta (v - g) (24) and the sums
// over the normal-strain rows of [D*] B-bar (24)
constexpr int kBbarExtra = 3 * 3 * NN;
static_assert(kHalf * (3 * NN + 21 + 6) >= NG * (3 * NN + 1), "b-bar staging must fit");

static_assert(kHalf * (3 * NN + 21 + 6) + NN * 18 + NN * 3 >= UT, "Ke staging must fit");

template <class T, bool kBbar = false>
struct TangentSmemHex8 {
  unsigned char pa[40], pb[40];     // node pairs of the 3x3 blocks (36 used)
  T dn[kDnSize];
  T elem[kChunk][kPerElem + (kBbar ? kBbarExtra : 0)];
};

// b-bar, phase 0 (rktstf's vol_terms + vol_avg, src/vol_terms.f:14-108,
// src/vol_avg.f:13-68): lane t evaluates Gauss points t and t + 4 and
// stages det[J] dN/dx and det[J]; then lane t sums nodes 2t, 2t + 1 over
// the eight points in Gauss-point order and scales by 1 / volume. stage
// holds NG x (3 NN + 1) values; v receives the 3 NN averaged gradients.
template <class T>
__device__ __forceinline__ void hex8_mean_gradients(const T* sdn, const T* sx, const T* sy, const T* sz, int t,
                                                    bool active, T* stage, T* v) {
  if (active) {
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int gp = t + 4 * k;
      const T* dnx = sdn + (gp * 3 + 0) * NN;
      const T* dne = sdn + (gp * 3 + 1) * NN;
      const T* dnz = sdn + (gp * 3 + 2) * NN;
      T gama[9], dj;
      jacobian_inverse<NN, T>(dnx, dne, dnz, sx, sy, sz, gama, dj);
      T* st = stage + gp * (3 * NN + 1);
#pragma unroll
      for (int n = 0; n < NN; ++n) {
        T gx, gy, gz;
        shape_gradient<T>(gama, dnx[n], dne[n], dnz[n], gx, gy, gz);
        st[3 * n] = gx * dj; st[3 * n + 1] = gy * dj; st[3 * n + 2] = gz * dj;
      }
      st[3 * NN] = dj;
    }
  }
  __syncwarp();
  if (active) {
    T vol = T(0);
#pragma unroll
    for (int gp = 0; gp < NG; ++gp) vol += stage[gp * (3 * NN + 1) + 3 * NN];
    const T voli = T(1) / vol;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const int j = 6 * t + k;   // nodes 2t, 2t + 1
      T s = T(0);
#pragma unroll
      for (int gp = 0; gp < NG; ++gp) s += stage[gp * (3 * NN + 1) + j];
      v[j] = s * voli;
    }
  }
  __syncwarp();
}

template <class T, class KOut, bool kRelative, bool kBbar = false>
__device__ __noinline__ void tangent_item_hex8(const TangentArgs& a, int cidx, unsigned char* smem) {
  TangentSmemHex8<T, kBbar>& S = *reinterpret_cast<TangentSmemHex8<T, kBbar>*>(smem);
  constexpr int kStride = kPerElem + (kBbar ? kBbarExtra : 0);
  T* sdn = S.dn;
  T* selem = &S.elem[0][0];
  unsigned char* pa = S.pa;
  unsigned char* pb = S.pb;

  const int lane = threadIdx.x;
  const int ge = lane >> 2;      // element within chunk
  const int t = lane & 3;
  const Chunk ch = a.chunks[cidx];
  const BlockDesc bd = a.blocks[ch.blk];
  const bool active = ge < ch.n;
  const int i = ch.i0 + ge;      // relative element in block

  for (int k = lane; k < kDnSize; k += 32) sdn[k] = (T)a.dn[0][k];
  if (lane == 0) {
    // node pairs (a <= b) of the 3x3 blocks of Ke, dealt to the 4 lanes of
    // an element: lane t takes slot p = 4p' + t. Slots 0-7 are the
    // diagonal pairs (t,t) and (t+4,t+4); the 28 off-diagonal pairs follow
    // in lexicographic order, 7 per lane.
    for (int t = 0; t < 4; ++t) {
      pa[t] = pb[t] = (unsigned char)t;
      pa[4 + t] = pb[4 + t] = (unsigned char)(t + 4);
    }
    int k = 8;
    for (int x = 0; x < NN; ++x)
      for (int y = x + 1; y < NN; ++y) {
        pa[k] = (unsigned char)x; pb[k] = (unsigned char)y;
        ++k;
      }
  }

  T* E = selem + ge * kStride;
  T* sx = E;
  T* sy = E + NN;
  T* sz = E + 2 * NN;
  T* sg = E + 3 * NN;                      // [slot][a][3]
  T* sD = sg + kHalf * 3 * NN;             // [slot][21]
  T* sT = sD + kHalf * 21;                 // [slot][6]
  T* sDB = sT + kHalf * 6;                 // [a][6][3]
  T* sTg = sDB + NN * 18;                  // [a][3]
  T* sV = E + kPerElem;                    // b-bar: [a][3] averaged gradients
  T* sH = sV + 3 * NN;                     //        [a][3] beta (v - g) at the GP
  T* sS = sH + 3 * NN;                     //        [a][3] normal-row sums of D* B-bar

  // ---- gather (dptstf) ----
  if (active) {
    const long long dbase = bd.einf_off + (long long)i * TOT;
    double ref[3] = {0.0, 0.0, 0.0};
    if (kRelative) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        int cidx = a.cdest[dbase + d * NN] - 1;
        double v = a.c[cidx];
        if (bd.geonl) {
          int eidx = a.edest[dbase + d * NN] - 1;
          v = v + a.u[eidx] + a.du[eidx];
        }
        ref[d] = v;
      }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      int node = 2 * t + h;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        int cidx = a.cdest[dbase + d * NN + node] - 1;
        double v = a.c[cidx];
        if (bd.geonl) {
          int eidx = a.edest[dbase + d * NN + node] - 1;
          v = v + a.u[eidx] + a.du[eidx];
        }
        E[d * NN + node] = from_f64<T>(v - ref[d]);
      }
    }
  }
  __syncwarp();
  if (kBbar) hex8_mean_gradients<T>(sdn, sx, sy, sz, t, active, sg, sV);
  const T beta = (T)a.bbar_beta;
  // b-bar: the geometric stiffness takes the averaged gradients at every
  // point, so it is v_a^T (sum_gp w det[J] {T}) v_b, formed once per
  // element; the stress sum accumulates in the (otherwise unused) {T}g
  // region, components 2t, 2t + 1 by lane t < 3
  if (kBbar && active && t < 3) { sTg[2 * t] = T(0); sTg[2 * t + 1] = T(0); }

  T acc[9][9];
#pragma unroll
  for (int p = 0; p < 9; ++p)
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[p][k] = T(0);

  const long long gpbase = bd.gp_off + (long long)i * NG;

  for (int half = 0; half < 2; ++half) {
    // ---- phase 1: one GP per lane ----
    if (active) {
      const int gp = half * kHalf + t;
      const T* dnx = sdn + (gp * 3 + 0) * NN;
      const T* dne = sdn + (gp * 3 + 1) * NN;
      const T* dnz = sdn + (gp * 3 + 2) * NN;
      const T w = sdn[NG * 3 * NN + gp];
      T gama[9], dj;
      jacobian_inverse<NN, T>(dnx, dne, dnz, sx, sy, sz, gama, dj);
      T* g = sg + t * 3 * NN;
#pragma unroll
      for (int n = 0; n < NN; ++n)
        shape_gradient<T>(gama, dnx[n], dne[n], dnz[n], g[3 * n], g[3 * n + 1], g[3 * n + 2]);
      const T f = w * dj;
      T C[21];
      load_D21<T, NG>(a, bd, i, gp, f, C);
      T* D = sD + t * 21;
      T* Tw = sT + t * 6;
      if (bd.geonl) {
        T R[9], q[36], ur[6], cs[6];
        const double* rp = a.rot_n1 + (gpbase + gp) * 9;
#pragma unroll
        for (int k = 0; k < 9; ++k) R[k] = from_f64<T>(rp[k]);
        const double* up = a.urcs_n1 + (gpbase + gp) * 9;
#pragma unroll
        for (int k = 0; k < 6; ++k) ur[k] = from_f64<T>(up[k]);
        rotation_q2<T>(R, q);
        qmply<T>(q, ur, cs);
        // [D*] = [q][D][q]^T, lower triangle, row by row (ctran1)
#pragma unroll
        for (int j = 0; j < 6; ++j) {
          T tc[6];
#pragma unroll
          for (int kk = 0; kk < 6; ++kk) {
            T s = T(0);
#pragma unroll
            for (int m = 0; m < 6; ++m) s += q[6 * j + m] * C[low(m, kk)];
            tc[kk] = s;
          }
#pragma unroll
          for (int kk = 0; kk <= j; ++kk) {
            T s = T(0);
#pragma unroll
            for (int m = 0; m < 6; ++m) s += tc[m] * q[6 * kk + m];
            D[low(j, kk)] = s;
          }
        }
        if (a.qbar) {   // ctran1_qbar (src/gptns1.f:1905-1967)
          const T wf = dj * w, halfw = T(0.5) * wf;
          const T xx = cs[0], yy = cs[1], zz = cs[2], xy = cs[3], yz = cs[4], xz = cs[5];
          D[low(0, 0)] -= T(2) * xx * wf;
          D[low(1, 1)] -= T(2) * yy * wf;
          D[low(2, 2)] -= T(2) * zz * wf;
          D[low(3, 0)] -= xy * wf;
          D[low(5, 0)] -= xz * wf;
          D[low(3, 1)] -= xy * wf;
          D[low(4, 1)] -= yz * wf;
          D[low(4, 2)] -= yz * wf;
          D[low(5, 2)] -= xz * wf;
          D[low(3, 3)] -= halfw * (xx + yy);
          D[low(4, 4)] -= halfw * (yy + zz);
          D[low(5, 5)] -= halfw * (xx + zz);
          D[low(4, 3)] -= wf * xz;
          D[low(5, 3)] -= wf * yz;
          D[low(5, 4)] -= wf * xy;
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) Tw[k] = cs[k] * f;
      } else {
#pragma unroll
        for (int k = 0; k < 21; ++k) D[k] = C[k];
#pragma unroll
        for (int k = 0; k < 6; ++k) Tw[k] = T(0);
      }
    }
    __syncwarp();
    if (kBbar && active && t < 3) {
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        T v = sTg[2 * t + j];
#pragma unroll
        for (int q = 0; q < kHalf; ++q) v += sT[q * 6 + 2 * t + j];
        sTg[2 * t + j] = v;
      }
    }

    // ---- phase 2 ----
    for (int s = 0; s < kHalf; ++s) {
      if (active) {
        const T* D = sD + s * 21;
        const T* Tw = sT + s * 6;
        const T* g = sg + s * 3 * NN;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int n = 2 * t + h;
          const T gx = g[3 * n], gy = g[3 * n + 1], gz = g[3 * n + 2];
          T* db = sDB + n * 18;   // db[m*3 + k]: row m of D*B_n, column k
          if (kBbar) {
            // bmod (src/bmod.f:16-205): column (n, k) of B-bar is column
            // (n, k) of B plus h_k = beta (v_k - g_k) in the three normal
            // rows, so D* B-bar_n = D* B_n + (D* m) h^T, m = (1,1,1,0,0,0)
            const T hx = beta * (sV[3 * n] - gx), hy = beta * (sV[3 * n + 1] - gy),
                    hz = beta * (sV[3 * n + 2] - gz);
            T s0 = T(0), s1 = T(0), s2 = T(0);
#pragma unroll
            for (int m = 0; m < 6; ++m) {
              const T dm = D[low(m, 0)] + D[low(m, 1)] + D[low(m, 2)];
              const T v0 = fma(dm, hx, D[low(m, 0)] * gx + D[low(m, 3)] * gy + D[low(m, 5)] * gz);
              const T v1 = fma(dm, hy, D[low(m, 1)] * gy + D[low(m, 3)] * gx + D[low(m, 4)] * gz);
              const T v2 = fma(dm, hz, D[low(m, 2)] * gz + D[low(m, 4)] * gy + D[low(m, 5)] * gx);
              db[m * 3 + 0] = v0; db[m * 3 + 1] = v1; db[m * 3 + 2] = v2;
              if (m < 3) { s0 += v0; s1 += v1; s2 += v2; }
            }
            sH[3 * n] = hx; sH[3 * n + 1] = hy; sH[3 * n + 2] = hz;
            sS[3 * n] = s0; sS[3 * n + 1] = s1; sS[3 * n + 2] = s2;
          } else {
#pragma unroll
            for (int m = 0; m < 6; ++m) {
              db[m * 3 + 0] = D[low(m, 0)] * gx + D[low(m, 3)] * gy + D[low(m, 5)] * gz;
              db[m * 3 + 1] = D[low(m, 1)] * gy + D[low(m, 3)] * gx + D[low(m, 4)] * gz;
              db[m * 3 + 2] = D[low(m, 2)] * gz + D[low(m, 4)] * gy + D[low(m, 5)] * gx;
            }
          }
          if (!kBbar) {   // kgstiff per point (b-bar: once per element, below)
            T* tg = sTg + n * 3;
            tg[0] = Tw[0] * gx + Tw[3] * gy + Tw[5] * gz;
            tg[1] = Tw[3] * gx + Tw[1] * gy + Tw[4] * gz;
            tg[2] = Tw[5] * gx + Tw[4] * gy + Tw[2] * gz;
          }
        }
      }
      __syncwarp();
      if (active) {
        const T* g = sg + s * 3 * NN;
#pragma unroll
        for (int p = 0; p < 9; ++p) {
          const int k = 4 * p + t;
          const int na = pa[k], nb = pb[k];
          const T ax = g[3 * na], ay = g[3 * na + 1], az = g[3 * na + 2];
          const T* db = sDB + nb * 18;
          // K_ab(i,k) += B_a(:,i) . (D* B_b)(:,k): rows of B_a column x are
          // (xx, xy, xz) = (gx, gy, gz), column y (yy, xy, yz) = (gy, gx, gz),
          // column z (zz, yz, xz) = (gz, gy, gx). Diagonal pairs (p < 2)
          // need only i <= k.
#pragma unroll
          for (int kk = 0; kk < 3; ++kk) {
            acc[p][0 * 3 + kk] = fma(ax, db[0 * 3 + kk], fma(ay, db[3 * 3 + kk], fma(az, db[5 * 3 + kk], acc[p][0 * 3 + kk])));
            if (p >= 2 || kk >= 1)
              acc[p][1 * 3 + kk] = fma(ay, db[1 * 3 + kk], fma(ax, db[3 * 3 + kk], fma(az, db[4 * 3 + kk], acc[p][1 * 3 + kk])));
            if (p >= 2 || kk >= 2)
              acc[p][2 * 3 + kk] = fma(az, db[2 * 3 + kk], fma(ay, db[4 * 3 + kk], fma(ax, db[5 * 3 + kk], acc[p][2 * 3 + kk])));
          }
          if (kBbar) {   // the normal rows of B-bar_a: + h_a (x) sum_m (D* B-bar_b)_m
            const T* ha = sH + 3 * na;
            const T* sb = sS + 3 * nb;
#pragma unroll
            for (int ii = 0; ii < 3; ++ii)
#pragma unroll
              for (int kk = 0; kk < 3; ++kk)
                if (p >= 2 || kk >= ii) acc[p][ii * 3 + kk] = fma(ha[ii], sb[kk], acc[p][ii * 3 + kk]);
          }
          if (!kBbar && bd.geonl) {   // kgstiff (src/kg1.f:16-110)
            const T* tg = sTg + nb * 3;
            const T gtg = ax * tg[0] + ay * tg[1] + az * tg[2];
            acc[p][0] += gtg; acc[p][4] += gtg; acc[p][8] += gtg;
          }
        }
      }
      __syncwarp();
    }
  }
  if (kBbar && bd.geonl) {
    // kgstiff with the averaged derivatives (src/kg1.f:46-54): v_a^T T v_b
    // per node pair with the element's stress sum T
    if (active) {
      T tsum[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) tsum[k] = sTg[k];
#pragma unroll
      for (int p = 0; p < 9; ++p) {
        const int k = 4 * p + t;
        const T* va = sV + 3 * pa[k];
        const T* vb = sV + 3 * pb[k];
        const T t0 = tsum[0] * vb[0] + tsum[3] * vb[1] + tsum[5] * vb[2];
        const T t1 = tsum[3] * vb[0] + tsum[1] * vb[1] + tsum[4] * vb[2];
        const T t2 = tsum[5] * vb[0] + tsum[4] * vb[1] + tsum[2] * vb[2];
        const T gtg = va[0] * t0 + va[1] * t1 + va[2] * t2;
        acc[p][0] += gtg; acc[p][4] += gtg; acc[p][8] += gtg;
      }
    }
  }

  // ---- store: column-packed upper triangle (src/setup.f:265-275) ----
  KOut* out = reinterpret_cast<KOut*>(a.estiff);
  T* ke = sg;   // staging reuses the GP region of this element
  if (active) {
    const T bf = (T)a.beta_fact;
#pragma unroll
    for (int p = 0; p < 9; ++p) {
      const int k = 4 * p + t;
      const int na = pa[k], nb = pb[k];
#pragma unroll
      for (int ii = 0; ii < 3; ++ii)
#pragma unroll
        for (int kk = 0; kk < 3; ++kk) {
          if (p < 2 && ii > kk) continue;
          int r = ii * NN + na, c = kk * NN + nb;
          if (r > c) { int tt = r; r = c; c = tt; }
          ke[c * (c + 1) / 2 + r] = acc[p][ii * 3 + kk] * bf;
        }
    }
  }
  __syncwarp();
  // elements i0..i0+n-1 are contiguous: out[estiff_off + (i0 + e)*UT + pos]
  const long long obase = bd.estiff_off + (long long)ch.i0 * UT;
  for (int e = 0; e < ch.n; ++e) {
    const T* src = selem + e * kStride + 3 * NN;
    for (int k = lane; k < UT; k += 32) out[obase + (long long)e * UT + k] = (KOut)src[k];
  }
}

// ---------------------------------------------------------------------
// Precision form: FP32 tangent with register blocking.
//
// FP32 arithmetic is 64x cheaper than FP64 on GB300, so here the limits
// are shared-memory traffic and latency, not the arithmetic pipe. Same
// 4 lanes per element and phase 1 as above; in phase 2 lane t owns the
// Ke columns of nodes b1 = t and b2 = 7 - t (pairs (a, b1), a <= t, and
// (a, b2), a <= 7 - t: 9 node pairs per lane), keeps [D*][B_b] and {T}g_b
// for both in registers and streams only the row-node gradients g_a from
// shared memory: 3 loads per 27 multiply-adds.
// ---------------------------------------------------------------------
constexpr int kPerElem32 = 3 * NN + kHalf * (3 * NN + 21 + 6) > UT ? 3 * NN + kHalf * (3 * NN + 21 + 6) : UT + 3 * NN;

template <bool kBbar = false>
struct TangentSmemHex8F32 {
  float dn[kDnSize];
  float elem[kChunk][kPerElem32 + (kBbar ? 3 * NN : 0)];   // b-bar: averaged gradients
};

template <bool kBbar = false>
__device__ __noinline__ void tangent_item_hex8_f32(const TangentArgs& a, int cidx, unsigned char* smem) {
  TangentSmemHex8F32<kBbar>& S = *reinterpret_cast<TangentSmemHex8F32<kBbar>*>(smem);
  float* sdn = S.dn;
  auto& selem = S.elem;

  const int lane = threadIdx.x;
  const int ge = lane >> 2;
  const int t = lane & 3;
  const Chunk ch = a.chunks[cidx];
  const BlockDesc bd = a.blocks[ch.blk];
  const bool active = ge < ch.n;
  const int i = ch.i0 + ge;

  for (int k = lane; k < kDnSize; k += 32) sdn[k] = (float)a.dn[0][k];
  float* E = selem[ge];
  float* sx = E;
  float* sy = E + NN;
  float* sz = E + 2 * NN;
  float* sg = E + 3 * NN;                  // [slot][a][3]
  float* sD = sg + kHalf * 3 * NN;         // [slot][21]
  float* sT = sD + kHalf * 21;             // [slot][6]
  float* sV = E + kPerElem32;              // b-bar: [a][3] averaged gradients

  // ---- gather: x_{n+1} relative to node 1 ----
  if (active) {
    const long long dbase = bd.einf_off + (long long)i * TOT;
    double ref[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      int cidx = a.cdest[dbase + d * NN] - 1;
      double v = a.c[cidx];
      if (bd.geonl) {
        int eidx = a.edest[dbase + d * NN] - 1;
        v = v + a.u[eidx] + a.du[eidx];
      }
      ref[d] = v;
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int node = 2 * t + h;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        int cidx = a.cdest[dbase + d * NN + node] - 1;
        double v = a.c[cidx];
        if (bd.geonl) {
          int eidx = a.edest[dbase + d * NN + node] - 1;
          v = v + a.u[eidx] + a.du[eidx];
        }
        E[d * NN + node] = d2f_rn(v - ref[d]);
      }
    }
  }
  __syncwarp();
  if (kBbar) hex8_mean_gradients<float>(sdn, sx, sy, sz, t, active, sg, sV);
  const float beta = (float)a.bbar_beta;

  const int b1 = t, b2 = 7 - t;
  float acc[9][9];
#pragma unroll
  for (int p = 0; p < 9; ++p)
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[p][k] = 0.f;
  const long long gpbase = bd.gp_off + (long long)i * NG;

  for (int half = 0; half < 2; ++half) {
    // ---- phase 1: one GP per lane (as in the FP64 kernel, in float) ----
    if (active) {
      const int gp = half * kHalf + t;
      const float* dnx = sdn + (gp * 3 + 0) * NN;
      const float* dne = sdn + (gp * 3 + 1) * NN;
      const float* dnz = sdn + (gp * 3 + 2) * NN;
      const float w = sdn[NG * 3 * NN + gp];
      float gama[9], dj;
      jacobian_inverse<NN, float>(dnx, dne, dnz, sx, sy, sz, gama, dj);
      float* g = sg + t * 3 * NN;
#pragma unroll
      for (int n = 0; n < NN; ++n)
        shape_gradient<float>(gama, dnx[n], dne[n], dnz[n], g[3 * n], g[3 * n + 1], g[3 * n + 2]);
      const float f = w * dj;
      float C[21];
      load_D21<float, NG>(a, bd, i, gp, f, C);
      float* D = sD + t * 21;
      float* Tw = sT + t * 6;
      if (bd.geonl) {
        float R[9], q[36], ur[6], cs[6];
        const double* rp = a.rot_n1 + (gpbase + gp) * 9;
#pragma unroll
        for (int k = 0; k < 9; ++k) R[k] = d2f_rn(rp[k]);
        const double* up = a.urcs_n1 + (gpbase + gp) * 9;
#pragma unroll
        for (int k = 0; k < 6; ++k) ur[k] = d2f_rn(up[k]);
        rotation_q2<float>(R, q);
        qmply<float>(q, ur, cs);
#pragma unroll
        for (int j = 0; j < 6; ++j) {
          float tc[6];
#pragma unroll
          for (int kk = 0; kk < 6; ++kk) {
            float sacc = 0.f;
#pragma unroll
            for (int m = 0; m < 6; ++m) sacc += q[6 * j + m] * C[low(m, kk)];
            tc[kk] = sacc;
          }
#pragma unroll
          for (int kk = 0; kk <= j; ++kk) {
            float sacc = 0.f;
#pragma unroll
            for (int m = 0; m < 6; ++m) sacc += tc[m] * q[6 * kk + m];
            D[low(j, kk)] = sacc;
          }
        }
        if (a.qbar) {
          const float wf = dj * w, halfw = 0.5f * wf;
          const float xx = cs[0], yy = cs[1], zz = cs[2], xy = cs[3], yz = cs[4], xz = cs[5];
          D[low(0, 0)] -= 2.f * xx * wf;
          D[low(1, 1)] -= 2.f * yy * wf;
          D[low(2, 2)] -= 2.f * zz * wf;
          D[low(3, 0)] -= xy * wf;
          D[low(5, 0)] -= xz * wf;
          D[low(3, 1)] -= xy * wf;
          D[low(4, 1)] -= yz * wf;
          D[low(4, 2)] -= yz * wf;
          D[low(5, 2)] -= xz * wf;
          D[low(3, 3)] -= halfw * (xx + yy);
          D[low(4, 4)] -= halfw * (yy + zz);
          D[low(5, 5)] -= halfw * (xx + zz);
          D[low(4, 3)] -= wf * xz;
          D[low(5, 3)] -= wf * yz;
          D[low(5, 4)] -= wf * xy;
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) Tw[k] = cs[k] * f;
      } else {
#pragma unroll
        for (int k = 0; k < 21; ++k) D[k] = C[k];
#pragma unroll
        for (int k = 0; k < 6; ++k) Tw[k] = 0.f;
      }
    }
    __syncwarp();

    // ---- phase 2: columns b1, b2 in registers ----
    if (active) {
      for (int s = 0; s < kHalf; ++s) {
        const float* D = sD + s * 21;
        const float* Tw = sT + s * 6;
        const float* g = sg + s * 3 * NN;
        float db1[18], db2[18], tg1[3], tg2[3], sb1[3], sb2[3];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int n = h == 0 ? b1 : b2;
          float* db = h == 0 ? db1 : db2;
          float* tg = h == 0 ? tg1 : tg2;
          float* sb = h == 0 ? sb1 : sb2;
          const float gx = g[3 * n], gy = g[3 * n + 1], gz = g[3 * n + 2];
#pragma unroll
          for (int m = 0; m < 6; ++m) {
            db[m * 3 + 0] = D[low(m, 0)] * gx + D[low(m, 3)] * gy + D[low(m, 5)] * gz;
            db[m * 3 + 1] = D[low(m, 1)] * gy + D[low(m, 3)] * gx + D[low(m, 4)] * gz;
            db[m * 3 + 2] = D[low(m, 2)] * gz + D[low(m, 4)] * gy + D[low(m, 5)] * gx;
          }
          float kx = gx, ky = gy, kz = gz;
          if (kBbar) {   // D* B-bar_n = D* B_n + (D* m) h^T (bmod)
            kx = sV[3 * n]; ky = sV[3 * n + 1]; kz = sV[3 * n + 2];
            const float hx = beta * (kx - gx), hy = beta * (ky - gy), hz = beta * (kz - gz);
            sb[0] = sb[1] = sb[2] = 0.f;
#pragma unroll
            for (int m = 0; m < 6; ++m) {
              const float dm = D[low(m, 0)] + D[low(m, 1)] + D[low(m, 2)];
              db[m * 3 + 0] = fmaf(dm, hx, db[m * 3 + 0]);
              db[m * 3 + 1] = fmaf(dm, hy, db[m * 3 + 1]);
              db[m * 3 + 2] = fmaf(dm, hz, db[m * 3 + 2]);
              if (m < 3) { sb[0] += db[m * 3 + 0]; sb[1] += db[m * 3 + 1]; sb[2] += db[m * 3 + 2]; }
            }
          }
          tg[0] = Tw[0] * kx + Tw[3] * ky + Tw[5] * kz;
          tg[1] = Tw[3] * kx + Tw[1] * ky + Tw[4] * kz;
          tg[2] = Tw[5] * kx + Tw[4] * ky + Tw[2] * kz;
        }
#pragma unroll
        for (int p = 0; p < 9; ++p) {
          const bool first = p <= t;
          const int na = first ? p : p - t - 1;
          const float ax = g[3 * na], ay = g[3 * na + 1], az = g[3 * na + 2];
#pragma unroll
          for (int kk = 0; kk < 3; ++kk) {
            const float d0 = first ? db1[0 * 3 + kk] : db2[0 * 3 + kk];
            const float d1 = first ? db1[1 * 3 + kk] : db2[1 * 3 + kk];
            const float d2 = first ? db1[2 * 3 + kk] : db2[2 * 3 + kk];
            const float d3 = first ? db1[3 * 3 + kk] : db2[3 * 3 + kk];
            const float d4 = first ? db1[4 * 3 + kk] : db2[4 * 3 + kk];
            const float d5 = first ? db1[5 * 3 + kk] : db2[5 * 3 + kk];
            acc[p][0 * 3 + kk] = fmaf(ax, d0, fmaf(ay, d3, fmaf(az, d5, acc[p][0 * 3 + kk])));
            acc[p][1 * 3 + kk] = fmaf(ay, d1, fmaf(ax, d3, fmaf(az, d4, acc[p][1 * 3 + kk])));
            acc[p][2 * 3 + kk] = fmaf(az, d2, fmaf(ay, d4, fmaf(ax, d5, acc[p][2 * 3 + kk])));
          }
          float kx = ax, ky = ay, kz = az;
          if (kBbar) {   // normal rows of B-bar_a: + h_a (x) sum_m (D* B-bar_b)_m
            kx = sV[3 * na]; ky = sV[3 * na + 1]; kz = sV[3 * na + 2];
            const float ha[3] = {beta * (kx - ax), beta * (ky - ay), beta * (kz - az)};
#pragma unroll
            for (int ii = 0; ii < 3; ++ii)
#pragma unroll
              for (int kk = 0; kk < 3; ++kk)
                acc[p][ii * 3 + kk] = fmaf(ha[ii], first ? sb1[kk] : sb2[kk], acc[p][ii * 3 + kk]);
          }
          if (bd.geonl) {
            const float t0 = first ? tg1[0] : tg2[0];
            const float t1 = first ? tg1[1] : tg2[1];
            const float t2 = first ? tg1[2] : tg2[2];
            const float gtg = kx * t0 + ky * t1 + kz * t2;
            acc[p][0] += gtg; acc[p][4] += gtg; acc[p][8] += gtg;
          }
        }
      }
    }
    __syncwarp();
  }

  // ---- store: column-packed upper triangle ----
  float* ke = E + 3 * NN;   // staging over the GP region (>= UT floats)
  if (active) {
    const float bf = (float)a.beta_fact;
#pragma unroll
    for (int p = 0; p < 9; ++p) {
      const bool first = p <= t;
      const int na = first ? p : p - t - 1;
      const int nb = first ? b1 : b2;
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
  __syncwarp();
  float* out = reinterpret_cast<float*>(a.estiff);
  const long long obase = bd.estiff_off + (long long)ch.i0 * UT;
  for (int e = 0; e < ch.n; ++e) {
    const float* src = selem[e] + 3 * NN;
    for (int k = lane; k < UT; k += 32) out[obase + (long long)e * UT + k] = src[k];
  }
}

}  // namespace hex8t
using hex8t::TangentSmemHex8;
using hex8t::TangentSmemHex8F32;
using hex8t::tangent_item_hex8;
using hex8t::tangent_item_hex8_f32;

template <class T> __device__ __forceinline__ const T* dn_table(const TangentArgs& a, int slot);
template <> __device__ __forceinline__ const double* dn_table<double>(const TangentArgs& a, int slot) {
  return a.dn[slot];
}
template <> __device__ __forceinline__ const float* dn_table<float>(const TangentArgs& a, int slot) {
  return a.dn32[slot];
}

template <class E>
struct GenTangentShape {
  static constexpr int NN = E::NN, NG = E::NG, UT = E::UTSZ;
  static constexpr int WORK = NG * (3 * NN + 21 + 6) + NN * (18 + 3);
  static constexpr int PER_ELEM = 3 * NN + (WORK > UT ? WORK : UT);
};

template <class E, int EPC, class T>
struct TangentSmemGen {
  T elem[EPC][GenTangentShape<E>::PER_ELEM];
};

template <class E, int LPE, int EPC, class T, bool kRel>
__device__ __noinline__ void tangent_item_gen(const TangentArgs& a, int cidx, unsigned char* smem) {
  constexpr int NN = E::NN, NG = E::NG, TOT = E::TOTDOF, UT = E::UTSZ;
  constexpr int NP = NN * (NN + 1) / 2;
  constexpr int PPL = (NP + LPE - 1) / LPE;
  constexpr int PER = GenTangentShape<E>::PER_ELEM;
  static_assert(LPE * EPC == kTangentThreads, "tangent items run on one warp");
  static_assert(NG <= LPE, "one Gauss point per lane in phase 1");
  T* selem = &reinterpret_cast<TangentSmemGen<E, EPC, T>*>(smem)->elem[0][0];
  const T* dn = dn_table<T>(a, E::SLOT);   // read through L1, shared by all items

  const int lane = threadIdx.x;
  const int ge = lane / LPE;
  const int l = lane % LPE;
  const Chunk ch = a.chunks[cidx];
  const BlockDesc bd = a.blocks[ch.blk];
  const bool active = ge < ch.n;
  const int i = ch.i0 + ge;

  // node pairs (x <= y) of this lane's Ke blocks: slot p is pair number
  // p*LPE + l in row-major upper-triangle order
  int pr[PPL];
#pragma unroll
  for (int p = 0; p < PPL; ++p) {
    const int k = p * LPE + l;
    if (k < NP) {
      int x = 0, r = k;
      while (r >= NN - x) { r -= NN - x; ++x; }
      pr[p] = x | ((x + r) << 8);
    } else {
      pr[p] = -1;
    }
  }

  T* Eb = selem + ge * PER;
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
        Eb[d * NN + node] = from_f64<T>(v - ref[d]);
      }
    }
  }
  __syncwarp();

  // ---- phase 1: Gauss point l ----
  if (active && l < NG) {
    const int gp = l;
    const T* dnx = dn + (gp * 3 + 0) * NN;
    const T* dne = dn + (gp * 3 + 1) * NN;
    const T* dnz = dn + (gp * 3 + 2) * NN;
    const T w = dn[NG * 3 * NN + gp];
    T gama[9], dj;
    jacobian_inverse<NN, T>(dnx, dne, dnz, sx, sy, sz, gama, dj);
    T* g = sg + gp * 3 * NN;
    for (int n = 0; n < NN; ++n)
      shape_gradient<T>(gama, dnx[n], dne[n], dnz[n], g[3 * n], g[3 * n + 1], g[3 * n + 2]);
    const T f = w * dj;
    T C[21];
    const double* cp = a.cep + bd.cep_off + ((long long)gp * bd.span + i) * 21;
#pragma unroll
    for (int k = 0; k < 21; ++k) C[k] = f * from_f64<T>(cp[k]);
    T* D = sD + gp * 21;
    T* Tw = sT + gp * 6;
    const long long gpi = bd.gp_off + (long long)i * NG + gp;
    if (bd.geonl) {
      T R[9], q[36], ur[6], cs[6];
#pragma unroll
      for (int k = 0; k < 9; ++k) R[k] = from_f64<T>(a.rot_n1[gpi * 9 + k]);
#pragma unroll
      for (int k = 0; k < 6; ++k) ur[k] = from_f64<T>(a.urcs_n1[gpi * 9 + k]);
      rotation_q2<T>(R, q);
      qmply<T>(q, ur, cs);
#pragma unroll
      for (int j = 0; j < 6; ++j) {   // [D*] = [q][D][q]^T (ctran1)
        T tc[6];
#pragma unroll
        for (int kk = 0; kk < 6; ++kk) {
          T s = T(0);
#pragma unroll
          for (int m = 0; m < 6; ++m) s += q[6 * j + m] * C[low(m, kk)];
          tc[kk] = s;
        }
#pragma unroll
        for (int kk = 0; kk <= j; ++kk) {
          T s = T(0);
#pragma unroll
          for (int m = 0; m < 6; ++m) s += tc[m] * q[6 * kk + m];
          D[low(j, kk)] = s;
        }
      }
      if (a.qbar) {   // ctran1_qbar (src/gptns1.f:1905-1967)
        const T wf = dj * w, halfw = T(0.5) * wf;
        const T xx = cs[0], yy = cs[1], zz = cs[2], xy = cs[3], yz = cs[4], xz = cs[5];
        D[low(0, 0)] -= T(2) * xx * wf;
        D[low(1, 1)] -= T(2) * yy * wf;
        D[low(2, 2)] -= T(2) * zz * wf;
        D[low(3, 0)] -= xy * wf;
        D[low(5, 0)] -= xz * wf;
        D[low(3, 1)] -= xy * wf;
        D[low(4, 1)] -= yz * wf;
        D[low(4, 2)] -= yz * wf;
        D[low(5, 2)] -= xz * wf;
        D[low(3, 3)] -= halfw * (xx + yy);
        D[low(4, 4)] -= halfw * (yy + zz);
        D[low(5, 5)] -= halfw * (xx + zz);
        D[low(4, 3)] -= wf * xz;
        D[low(5, 3)] -= wf * yz;
        D[low(5, 4)] -= wf * xy;
      }
#pragma unroll
      for (int k = 0; k < 6; ++k) Tw[k] = cs[k] * f;
    } else {
#pragma unroll
      for (int k = 0; k < 21; ++k) D[k] = C[k];
#pragma unroll
      for (int k = 0; k < 6; ++k) Tw[k] = T(0);
    }
    if (E::TET) {   // adjust_cnst (src/gpmas1.f:399-430): [D] x 1/6
      const T scalar = T(1.0 / 6.0);
#pragma unroll
      for (int k = 0; k < 21; ++k) D[k] = scalar * D[k];
    }
  }
  __syncwarp();

  T acc[PPL][9];
#pragma unroll
  for (int p = 0; p < PPL; ++p)
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[p][k] = T(0);

  for (int gp = 0; gp < NG; ++gp) {
    if (active) {   // [D*][B_n] and {T}g_n for the lane's nodes
      const T* D = sD + gp * 21;
      const T* Tw = sT + gp * 6;
      const T* g = sg + gp * 3 * NN;
      for (int n = l; n < NN; n += LPE) {
        const T gx = g[3 * n], gy = g[3 * n + 1], gz = g[3 * n + 2];
        T* db = sDB + n * 18;
#pragma unroll
        for (int m = 0; m < 6; ++m) {
          db[m * 3 + 0] = D[low(m, 0)] * gx + D[low(m, 3)] * gy + D[low(m, 5)] * gz;
          db[m * 3 + 1] = D[low(m, 1)] * gy + D[low(m, 3)] * gx + D[low(m, 4)] * gz;
          db[m * 3 + 2] = D[low(m, 2)] * gz + D[low(m, 4)] * gy + D[low(m, 5)] * gx;
        }
        T* tg = sTg + n * 3;
        tg[0] = Tw[0] * gx + Tw[3] * gy + Tw[5] * gz;
        tg[1] = Tw[3] * gx + Tw[1] * gy + Tw[4] * gz;
        tg[2] = Tw[5] * gx + Tw[4] * gy + Tw[2] * gz;
      }
    }
    __syncwarp();
    if (active) {
      const T* g = sg + gp * 3 * NN;
#pragma unroll
      for (int p = 0; p < PPL; ++p) {
        if (pr[p] >= 0) {
          const int na = pr[p] & 0xff, nb = pr[p] >> 8;
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
    __syncwarp();
  }

  // ---- store: column-packed upper triangle ----
  T* ke = Eb + 3 * NN;
  if (active) {
    const T bf = (T)a.beta_fact;
#pragma unroll
    for (int p = 0; p < PPL; ++p) {
      if (pr[p] >= 0) {
        const int na = pr[p] & 0xff, nb = pr[p] >> 8;
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
  __syncwarp();
  T* out = reinterpret_cast<T*>(a.estiff);
  const long long obase = bd.estiff_off + (long long)ch.i0 * UT;
  for (int e = 0; e < ch.n; ++e) {
    const T* src = selem + e * PER + 3 * NN;
    for (int k = lane; k < UT; k += kTangentThreads) out[obase + (long long)e * UT + k] = src[k];
  }
}

}  // namespace w3g
