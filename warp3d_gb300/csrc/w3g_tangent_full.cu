// w3g_tangent_full.cu -- 8-node brick tangents under asymmetric assembly
// ("assembly asymmetric on"): the full element matrix Bᵀ [D*] B + Gᵀ T G
// for a [D] that need not be symmetric (mm10 tangents are not symmetrized
// then, mm10_a.f:1165-1166), stored column-major as WARP3D's ek_full
// (span, totdof²) transposed to (totdof², span) (gptns1.f:1513-1612
// bdbt_asym, kg1.f:112-178, rktstf.f:161-165).
//
// One warp per work item (up to 8 consecutive elements of a block), the
// elements one after another:
//   gather   lanes 0-23 load one coordinate each (x(n+1) for geonl)
//   phase 1  lanes 0-7 take one Gauss point each: gradients, det[J],
//            w det[J] [D] (full 6x6: cep_blocks expanded, or history1(1:36)
//            for mm10), [D*] = [q][D][q]ᵀ with WARP3D's Q-bar terms (which
//            write the lower entries and copy them over the upper ones,
//            gptns1.f:1905-1967), w det[J] {T}; all to shared memory
//   b-bar    lanes 0-23 average one gradient component over the 8 points
//   phase 2  lane c < 24 owns column c of Ke: per point [D*] B̄_c, then
//            every row r: B̄_rᵀ ([D*] B̄_c), plus the geometric term of the
//            rows of the same direction; registers, FMA
//   store    the column-major matrix staged in shared memory, written with
//            coalesced stores
// The FP64 instantiation is the plain form, FP32 the precision form.
//
// 20-node bricks and tetrahedra under asymmetric assembly (mm01: a
// symmetric [D]) take their usual packed work items, written to a scratch
// array, and k_expand_packed mirrors each packed upper triangle into the
// full column-major matrix.
#include "w3g_tangent_items.cuh"

namespace w3g {

namespace {

constexpr int NN = Hex8::NN, NG = Hex8::NG, TOT = Hex8::TOTDOF;
constexpr int kDn = NG * 3 * NN + NG;

template <class T>
struct FullSmem {
  T dn[kDn];
  T x[3 * NN];
  T g[NG][3 * NN];
  T D[NG][36];      // [D*] row-major: D[r * 6 + c]
  T Tw[NG][6];
  T dj[NG];
  T v[3 * NN];      // b-bar: volume-averaged gradients
  T K[TOT * TOT];   // column-major staging
};

template <class T>
__global__ void __launch_bounds__(32) k_tangent_full_hex8(TangentArgs a) {
  __shared__ FullSmem<T> S;
  const int lane = threadIdx.x;
  const Chunk ch = a.chunks[a.chunk0 + blockIdx.x];
  const BlockDesc bd = a.blocks[ch.blk];
  const T beta = (T)a.bbar_beta;
  for (int k = lane; k < kDn; k += 32) S.dn[k] = (T)a.dn[0][k];
  for (int e = 0; e < ch.n; ++e) {
    const int i = ch.i0 + e;
    const long long dbase = bd.einf_off + (long long)i * TOT;
    __syncwarp();
    // ---- gather (dptstf); FP32 coordinates relative to the first node ----
    if (lane < 3 * NN) {
      const int d = lane / NN;
      double v = a.c[a.cdest[dbase + lane] - 1], ref = 0.0;
      if (bd.geonl) {
        const int ei = a.edest[dbase + lane] - 1;
        v = v + a.u[ei] + a.du[ei];
      }
      if (sizeof(T) == 4) {
        ref = a.c[a.cdest[dbase + d * NN] - 1];
        if (bd.geonl) {
          const int e0 = a.edest[dbase + d * NN] - 1;
          ref = ref + a.u[e0] + a.du[e0];
        }
      }
      S.x[lane] = from_f64<T>(v - ref);
    }
    __syncwarp();
    // ---- phase 1: one Gauss point per lane ----
    if (lane < NG) {
      const int gp = lane;
      const T* dnx = S.dn + (gp * 3 + 0) * NN;
      const T* dne = S.dn + (gp * 3 + 1) * NN;
      const T* dnz = S.dn + (gp * 3 + 2) * NN;
      const T w = S.dn[NG * 3 * NN + gp];
      T gama[9], dj;
      jacobian_inverse<NN, T>(dnx, dne, dnz, S.x, S.x + NN, S.x + 2 * NN, gama, dj);
      T* g = S.g[gp];
#pragma unroll
      for (int n = 0; n < NN; ++n) shape_gradient<T>(gama, dnx[n], dne[n], dnz[n], g[3 * n], g[3 * n + 1], g[3 * n + 2]);
      S.dj[gp] = dj;
      const T f = w * dj;
      T Dl[36];
      if (bd.mat == W3G_MAT_CRYSTAL) {   // drive_10_cnst: history1(1:36), column-major
        const double* h1 = a.hist1 + bd.hist_off + ((long long)i * NG + gp) * kHistMM10;
#pragma unroll
        for (int r = 0; r < 6; ++r)
#pragma unroll
          for (int c = 0; c < 6; ++c) Dl[r * 6 + c] = f * from_f64<T>(h1[r + 6 * c]);
      } else {                           // extract_D_symmetric
        const double* cp = a.cep + bd.cep_off + ((long long)gp * bd.span + i) * 21;
#pragma unroll
        for (int r = 0; r < 6; ++r)
#pragma unroll
          for (int c = 0; c < 6; ++c) Dl[r * 6 + c] = f * from_f64<T>(cp[low(r, c)]);
      }
      T* D = S.D[gp];
      T* Tw = S.Tw[gp];
      if (bd.geonl) {   // ctran1 (gptns1.f:1735-1969), full
        const long long gpi = bd.gp_off + (long long)i * NG + gp;
        T R[9], q[36], ur[6], cs[6];
#pragma unroll
        for (int k = 0; k < 9; ++k) R[k] = from_f64<T>(a.rot_n1[gpi * 9 + k]);
#pragma unroll
        for (int k = 0; k < 6; ++k) ur[k] = from_f64<T>(a.urcs_n1[gpi * 9 + k]);
        rotation_q2<T>(R, q);
        qmply<T>(q, ur, cs);
#pragma unroll
        for (int j = 0; j < 6; ++j) {
          T tc[6];
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            T s = T(0);
#pragma unroll
            for (int m = 0; m < 6; ++m) s += q[6 * j + m] * Dl[m * 6 + k];
            tc[k] = s;
          }
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            T s = T(0);
#pragma unroll
            for (int m = 0; m < 6; ++m) s += tc[m] * q[6 * k + m];
            D[j * 6 + k] = s;
          }
        }
        if (a.qbar) {   // ctran1_qbar: lower entries, then copied over the upper ones
          const T wf = dj * w, halfw = T(0.5) * wf;
          const T xx = cs[0], yy = cs[1], zz = cs[2], xy = cs[3], yz = cs[4], xz = cs[5];
          D[0 * 6 + 0] -= T(2) * xx * wf;
          D[1 * 6 + 1] -= T(2) * yy * wf;
          D[2 * 6 + 2] -= T(2) * zz * wf;
          D[3 * 6 + 0] -= xy * wf;
          D[5 * 6 + 0] -= xz * wf;
          D[3 * 6 + 1] -= xy * wf;
          D[4 * 6 + 1] -= yz * wf;
          D[4 * 6 + 2] -= yz * wf;
          D[5 * 6 + 2] -= xz * wf;
          D[3 * 6 + 3] -= halfw * (xx + yy);
          D[4 * 6 + 4] -= halfw * (yy + zz);
          D[5 * 6 + 5] -= halfw * (xx + zz);
          D[4 * 6 + 3] -= wf * xz;
          D[5 * 6 + 3] -= wf * yz;
          D[5 * 6 + 4] -= wf * xy;
          D[0 * 6 + 3] = D[3 * 6 + 0]; D[0 * 6 + 5] = D[5 * 6 + 0]; D[1 * 6 + 3] = D[3 * 6 + 1];
          D[1 * 6 + 4] = D[4 * 6 + 1]; D[2 * 6 + 4] = D[4 * 6 + 2]; D[2 * 6 + 5] = D[5 * 6 + 2];
          D[3 * 6 + 4] = D[4 * 6 + 3]; D[3 * 6 + 5] = D[5 * 6 + 3]; D[4 * 6 + 5] = D[5 * 6 + 4];
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) Tw[k] = cs[k] * f;
      } else {
#pragma unroll
        for (int k = 0; k < 36; ++k) D[k] = Dl[k];
#pragma unroll
        for (int k = 0; k < 6; ++k) Tw[k] = T(0);
      }
    }
    __syncwarp();
    // ---- b-bar: mean gradients (vol_terms, vol_avg) ----
    if (bd.bbar) {
      if (lane < 3 * NN) {
        T s = T(0), vol = T(0);
#pragma unroll
        for (int gp = 0; gp < NG; ++gp) {
          s += S.g[gp][lane] * S.dj[gp];
          vol += S.dj[gp];
        }
        S.v[lane] = s * (T(1) / vol);
      }
      __syncwarp();
    }
    // ---- phase 2: column c of Ke ----
    if (lane < TOT) {
      const int c = lane, ac = c % NN, dc = c / NN;
      T acc[TOT];
#pragma unroll
      for (int r = 0; r < TOT; ++r) acc[r] = T(0);
      for (int gp = 0; gp < NG; ++gp) {
        const T* g = S.g[gp];
        const T* D = S.D[gp];
        const T gx = g[3 * ac], gy = g[3 * ac + 1], gz = g[3 * ac + 2];
        T bc[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};   // B column c (blcmp1)
        if (dc == 0) { bc[0] = gx; bc[3] = gy; bc[5] = gz; }
        else if (dc == 1) { bc[1] = gy; bc[3] = gx; bc[4] = gz; }
        else { bc[2] = gz; bc[4] = gy; bc[5] = gx; }
        if (bd.bbar) {   // bmod: + beta (v - g) in the normal rows
          const T h = beta * (S.v[3 * ac + dc] - g[3 * ac + dc]);
          bc[0] += h; bc[1] += h; bc[2] += h;
        }
        T db[6];
#pragma unroll
        for (int m = 0; m < 6; ++m) {
          T s = T(0);
#pragma unroll
          for (int k = 0; k < 6; ++k) s = fma(D[m * 6 + k], bc[k], s);
          db[m] = s;
        }
        const T s012 = db[0] + db[1] + db[2];
#pragma unroll
        for (int r = 0; r < TOT; ++r) {
          const int ar = r % NN, dr = r / NN;
          const T rx = g[3 * ar], ry = g[3 * ar + 1], rz = g[3 * ar + 2];
          T kv;
          if (dr == 0) kv = fma(rx, db[0], fma(ry, db[3], rz * db[5]));
          else if (dr == 1) kv = fma(ry, db[1], fma(rx, db[3], rz * db[4]));
          else kv = fma(rz, db[2], fma(ry, db[4], rx * db[5]));
          if (bd.bbar) kv = fma(beta * (S.v[3 * ar + dr] - g[3 * ar + dr]), s012, kv);
          acc[r] += kv;
        }
        if (bd.geonl) {   // kgstiff: rows of the same direction (b-bar: averaged gradients)
          const T* Tw = S.Tw[gp];
          const T* kg = bd.bbar ? S.v : g;
          const T cx = kg[3 * ac], cy = kg[3 * ac + 1], cz = kg[3 * ac + 2];
          const T t0 = Tw[0] * cx + Tw[3] * cy + Tw[5] * cz;
          const T t1 = Tw[3] * cx + Tw[1] * cy + Tw[4] * cz;
          const T t2 = Tw[5] * cx + Tw[4] * cy + Tw[2] * cz;
#pragma unroll
          for (int r = 0; r < TOT; ++r)
            if (r / NN == dc) acc[r] += kg[3 * (r % NN)] * t0 + kg[3 * (r % NN) + 1] * t1 + kg[3 * (r % NN) + 2] * t2;
        }
      }
      const T bf = (T)a.beta_fact;
#pragma unroll
      for (int r = 0; r < TOT; ++r) S.K[c * TOT + r] = acc[r] * bf;
    }
    __syncwarp();
    T* out = reinterpret_cast<T*>(a.estiff) + bd.estiff_off + (long long)i * (TOT * TOT);
    for (int k = lane; k < TOT * TOT; k += 32) out[k] = S.K[k];
  }
}

// full column-major matrices from packed upper triangles (column-packed,
// pos = c(c+1)/2 + r for r <= c), one CTA per tangent work item
template <class T>
__global__ void __launch_bounds__(256) k_expand_packed(const Chunk* chunks, int chunk0, const BlockDesc* blocks,
                                                      const BlockDesc* blocks_packed, const T* packed, T* full) {
  const Chunk ch = chunks[chunk0 + blockIdx.x];
  const BlockDesc bd = blocks[ch.blk];
  const long long pbase = blocks_packed[ch.blk].estiff_off;
  const int tot = bd.totdof, nn = tot * tot;
  for (int e = 0; e < ch.n; ++e) {
    const int i = ch.i0 + e;
    const T* src = packed + pbase + (long long)i * bd.utsz;
    T* dst = full + bd.estiff_off + (long long)i * nn;
    for (int k = threadIdx.x; k < nn; k += blockDim.x) {
      const int c = k / tot, r = k - c * tot;
      const int lo = r < c ? r : c, hi = r < c ? c : r;
      dst[k] = src[hi * (hi + 1) / 2 + lo];
    }
  }
}

}  // namespace

cudaError_t launch_expand_packed(const DeviceModel& m, const TangentArgs& a, const void* packed, bool fp32,
                                 cudaStream_t s) {
  const int n = m.ttype_chunks[1] + m.ttype_chunks[2];
  if (n == 0) return cudaSuccess;
  const int c0 = m.ttype_chunks[1] > 0 ? m.ttype_chunk0[1] : m.ttype_chunk0[2];
  if (fp32)
    k_expand_packed<float><<<n, 256, 0, s>>>(a.chunks, c0, m.blocks, m.blocks_packed, (const float*)packed,
                                            (float*)a.estiff);
  else
    k_expand_packed<double><<<n, 256, 0, s>>>(a.chunks, c0, m.blocks, m.blocks_packed, (const double*)packed,
                                             (double*)a.estiff);
  return cudaGetLastError();
}

cudaError_t launch_tangent_full(const DeviceModel& m, const TangentArgs& a, bool fp32, cudaStream_t s) {
  if (m.ttype_chunks[0] == 0) return cudaSuccess;
  TangentArgs h = a;
  h.chunk0 = m.ttype_chunk0[0];
  if (fp32) k_tangent_full_hex8<float><<<m.ttype_chunks[0], 32, 0, s>>>(h);
  else k_tangent_full_hex8<double><<<m.ttype_chunks[0], 32, 0, s>>>(h);
  return cudaGetLastError();
}

}  // namespace w3g
