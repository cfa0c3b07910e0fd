// w3g_tangent.cu -- element tangent stiffness kernels (tanstf/rktstf/
// gptns1 with bdbtgen, ctran1 + Q-bar and kgstiff) for 8-node hexahedra.
//
// Work decomposition (one warp = one CTA = one chunk of <= 8 elements of
// one block; 4 lanes per element):
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
// The FP64 instantiation is the plain form. The FP32 instantiation is the
// precision form: same algorithm with float arithmetic, coordinates taken
// relative to the element's first node (exactly representable offsets),
// Ke stored as float.
#include "w3g_internal.cuh"
#include "w3g_elem.cuh"
#include "w3g_math.cuh"

namespace w3g {

namespace {

constexpr int NN = Hex8::NN;
constexpr int NG = Hex8::NG;
constexpr int TOT = Hex8::TOTDOF;
constexpr int UT = Hex8::UTSZ;
constexpr int kHalf = 4;                     // GPs per phase-1 pass
constexpr int kPerElem = 3 * NN              // coordinates
                         + kHalf * (3 * NN + 21 + 6)   // gradients, D*, {T}w
                         + NN * 18 + NN * 3;           // D*B per node, {T}g per node
constexpr int kDnSize = NG * 3 * NN + NG;

static_assert(kHalf * (3 * NN + 21 + 6) + NN * 18 + NN * 3 >= UT, "Ke staging must fit");

// lower-triangle index of the symmetric 6x6 (r, c), 0-based
__device__ __forceinline__ constexpr int low(int r, int c) {
  return r >= c ? r * (r + 1) / 2 + c : c * (c + 1) / 2 + r;
}

template <class T, class KOut, bool kRelative>
__global__ void __launch_bounds__(32) k_tangent_hex8(TangentArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sdn = reinterpret_cast<T*>(smem_raw);
  T* selem = sdn + kDnSize;
  __shared__ unsigned char pa[36], pb[36];

  const int lane = threadIdx.x;
  const int ge = lane >> 2;      // element within chunk
  const int t = lane & 3;
  const Chunk ch = a.chunks[a.chunk0 + blockIdx.x];
  const BlockDesc bd = a.blocks[ch.blk];
  const bool active = ge < ch.n;
  const int i = ch.i0 + ge;      // relative element in block

  for (int k = lane; k < kDnSize; k += 32) sdn[k] = (T)a.dn[k];
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

  T* E = selem + ge * kPerElem;
  T* sx = E;
  T* sy = E + NN;
  T* sz = E + 2 * NN;
  T* sg = E + 3 * NN;                      // [slot][a][3]
  T* sD = sg + kHalf * 3 * NN;             // [slot][21]
  T* sT = sD + kHalf * 21;                 // [slot][6]
  T* sDB = sT + kHalf * 6;                 // [a][6][3]
  T* sTg = sDB + NN * 18;                  // [a][3]

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
        E[d * NN + node] = (T)(v - ref[d]);
      }
    }
  }
  __syncthreads();

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
      const double* cp = a.cep + bd.cep_off + ((long long)gp * bd.span + i) * 21;
#pragma unroll
      for (int k = 0; k < 21; ++k) C[k] = f * (T)cp[k];
      T* D = sD + t * 21;
      T* Tw = sT + t * 6;
      if (bd.geonl) {
        T R[9], q[36], ur[6], cs[6];
        const double* rp = a.rot_n1 + (gpbase + gp) * 9;
#pragma unroll
        for (int k = 0; k < 9; ++k) R[k] = (T)rp[k];
        const double* up = a.urcs_n1 + (gpbase + gp) * 9;
#pragma unroll
        for (int k = 0; k < 6; ++k) ur[k] = (T)up[k];
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
    __syncthreads();

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
      __syncthreads();
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
          if (bd.geonl) {   // kgstiff (src/kg1.f:16-110)
            const T* tg = sTg + nb * 3;
            const T gtg = ax * tg[0] + ay * tg[1] + az * tg[2];
            acc[p][0] += gtg; acc[p][4] += gtg; acc[p][8] += gtg;
          }
        }
      }
      __syncthreads();
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
  __syncthreads();
  // elements i0..i0+n-1 are contiguous: out[estiff_off + (i0 + e)*UT + pos]
  const long long obase = bd.estiff_off + (long long)ch.i0 * UT;
  for (int e = 0; e < ch.n; ++e) {
    const T* src = selem + e * kPerElem + 3 * NN;
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

__global__ void __launch_bounds__(32, 12) k_tangent32_hex8(TangentArgs a) {
  __shared__ float sdn[kDnSize];
  __shared__ __align__(16) float selem[kChunk][kPerElem32];

  const int lane = threadIdx.x;
  const int ge = lane >> 2;
  const int t = lane & 3;
  const Chunk ch = a.chunks[a.chunk0 + blockIdx.x];
  const BlockDesc bd = a.blocks[ch.blk];
  const bool active = ge < ch.n;
  const int i = ch.i0 + ge;

  for (int k = lane; k < kDnSize; k += 32) sdn[k] = (float)a.dn[k];
  float* E = selem[ge];
  float* sx = E;
  float* sy = E + NN;
  float* sz = E + 2 * NN;
  float* sg = E + 3 * NN;                  // [slot][a][3]
  float* sD = sg + kHalf * 3 * NN;         // [slot][21]
  float* sT = sD + kHalf * 21;             // [slot][6]

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
        E[d * NN + node] = (float)(v - ref[d]);
      }
    }
  }
  __syncwarp();

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
      const double* cp = a.cep + bd.cep_off + ((long long)gp * bd.span + i) * 21;
#pragma unroll
      for (int k = 0; k < 21; ++k) C[k] = f * (float)cp[k];
      float* D = sD + t * 21;
      float* Tw = sT + t * 6;
      if (bd.geonl) {
        float R[9], q[36], ur[6], cs[6];
        const double* rp = a.rot_n1 + (gpbase + gp) * 9;
#pragma unroll
        for (int k = 0; k < 9; ++k) R[k] = (float)rp[k];
        const double* up = a.urcs_n1 + (gpbase + gp) * 9;
#pragma unroll
        for (int k = 0; k < 6; ++k) ur[k] = (float)up[k];
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
        float db1[18], db2[18], tg1[3], tg2[3];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int n = h == 0 ? b1 : b2;
          float* db = h == 0 ? db1 : db2;
          float* tg = h == 0 ? tg1 : tg2;
          const float gx = g[3 * n], gy = g[3 * n + 1], gz = g[3 * n + 2];
#pragma unroll
          for (int m = 0; m < 6; ++m) {
            db[m * 3 + 0] = D[low(m, 0)] * gx + D[low(m, 3)] * gy + D[low(m, 5)] * gz;
            db[m * 3 + 1] = D[low(m, 1)] * gy + D[low(m, 3)] * gx + D[low(m, 4)] * gz;
            db[m * 3 + 2] = D[low(m, 2)] * gz + D[low(m, 4)] * gy + D[low(m, 5)] * gx;
          }
          tg[0] = Tw[0] * gx + Tw[3] * gy + Tw[5] * gz;
          tg[1] = Tw[3] * gx + Tw[1] * gy + Tw[4] * gz;
          tg[2] = Tw[5] * gx + Tw[4] * gy + Tw[2] * gz;
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
          if (bd.geonl) {
            const float t0 = first ? tg1[0] : tg2[0];
            const float t1 = first ? tg1[1] : tg2[1];
            const float t2 = first ? tg1[2] : tg2[2];
            const float gtg = ax * t0 + ay * t1 + az * t2;
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

template <class T, class KOut, bool kRel>
cudaError_t launch_hex8(const DeviceModel& m, const TangentArgs& a, cudaStream_t s) {
  if (m.type_chunks[0] == 0) return cudaSuccess;
  size_t smem = sizeof(T) * (size_t)(kDnSize + kChunk * kPerElem);
  auto kern = k_tangent_hex8<T, KOut, kRel>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  kern<<<m.type_chunks[0], 32, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_tangent_fp64(const DeviceModel& m, const TangentArgs& a, cudaStream_t s) {
  TangentArgs h = a;
  h.dn = m.dn_hex8;
  h.chunk0 = m.type_chunk0[0];
  cudaError_t e = launch_hex8<double, double, false>(m, h, s);
  if (e != cudaSuccess) return e;
  return launch_tangent_other(m, a, false, s);
}

cudaError_t launch_tangent_fp32(const DeviceModel& m, const TangentArgs& a, cudaStream_t s) {
  if (m.type_chunks[0] > 0) {
    TangentArgs h = a;
    h.dn = m.dn_hex8;
    h.chunk0 = m.type_chunk0[0];
    k_tangent32_hex8<<<m.type_chunks[0], 32, 0, s>>>(h);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return launch_tangent_other(m, a, true, s);
}

}  // namespace w3g
