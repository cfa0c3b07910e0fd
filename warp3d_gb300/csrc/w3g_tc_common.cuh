// w3g_tc_common.cuh -- helpers shared by the tensor-core tangent kernels
// (w3g_tangent_tcg.cu, w3g_tangent_tc20.cu): shared-memory matrix
// descriptors of the K-major no-swizzle operand layout, bounded mbarrier
// waits, bulk copies, operand rounding to TF32 / BF16 on the integer
// pipes, and the small index maps of the strain-rotation algebra.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace w3g {
namespace tc {

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t sdesc(uint32_t addr, int sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((128 >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// bounded wait on an mbarrier phase; returns false when it gave up.
// `abort` (shared) ends the wait early when another thread gave up.
__device__ __forceinline__ bool wait_phase(unsigned long long* bar, uint32_t parity, long long limit,
                                           const volatile int* abort) {
  uint32_t done = 0;
  for (long long polls = 0; polls < limit; ++polls) {
    asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done) : "r"(su32(bar)), "r"(parity) : "memory");
    if (done) return true;
    if (abort && *abort) return false;
  }
  return false;
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(dst), "l"(src), "r"(bytes), "r"(bar) : "memory");
}

// leading bytes of a 1-D bulk copy started at the 16-byte boundary below p
__device__ __forceinline__ uint32_t pad_of(const double* p) { return (uint32_t)((uintptr_t)p & 15); }

// float -> TF32 (round to nearest, ties away from zero: add half a unit of
// the 10-bit mantissa to the magnitude bits, drop the low 13) and -> BF16
// (round to nearest even: the upper 16 bits after adding 0x7FFF plus the
// lowest kept bit), on the integer pipes; finite inputs (the operand
// values) only. The conversion instructions run on GB300's narrow
// conversion pipe, at a small fraction of the integer rate.
__device__ __forceinline__ uint32_t tf32_bits(float v) { return (__float_as_uint(v) + 0x1000u) & 0xFFFFE000u; }
__device__ __forceinline__ uint16_t bf16_bits(float v) {
  const uint32_t u = __float_as_uint(v);
  return (uint16_t)((u + 0x7FFFu + ((u >> 16) & 1u)) >> 16);
}

template <bool kBF16>
__device__ __forceinline__ void put(unsigned char* op, int o, float v) {
  if (kBF16) *reinterpret_cast<uint16_t*>(op + o) = bf16_bits(v);
  else *reinterpret_cast<uint32_t*>(op + o) = tf32_bits(v);
}

template <bool kBF16>
__device__ __forceinline__ float round_in(float v) {
  if (kBF16) return __uint_as_float((uint32_t)bf16_bits(v) << 16);
  return __uint_as_float(tf32_bits(v));
}

// one value of an operand (and its low part for the split forms)
template <bool kBF16, bool kSplit>
__device__ __forceinline__ void put_split(unsigned char* op, int op_bytes, int o, float v) {
  if (kSplit) {
    const float hi = round_in<kBF16>(v);
    put<kBF16>(op, o, hi);
    put<kBF16>(op + op_bytes, o, v - hi);
  } else {
    put<kBF16>(op, o, v);
  }
}

// lower-triangle index of (r, c), r >= c
__host__ __device__ constexpr int lw(int r, int c) { return r >= c ? r * (r + 1) / 2 + c : c * (c + 1) / 2 + r; }

// Voigt index of the strain pair (i, p): xx yy zz xy yz xz
__host__ __device__ constexpr int voigt(int i, int p) {
  return i == p ? i : (i + p == 1 ? 3 : (i + p == 3 ? 4 : 5));
}

// row r of the 6 x 6 strain-rotation matrix [q] of getrm1 option 2
// (gtmat1.f:803-846; the same entries as rotation_q2) from R, column-major:
// rows 0-2 the normal components of R's rows a = r, rows 3-5 the pairs
// (a, b) = (0, 1), (1, 2), (0, 2)
__device__ __forceinline__ void q_row(const float* R, int r, float* o) {
#define RX(i, j) R[(i) + 3 * (j)]
  if (r < 3) {
    const int x = r;
    o[0] = RX(x, 0) * RX(x, 0); o[1] = RX(x, 1) * RX(x, 1); o[2] = RX(x, 2) * RX(x, 2);
    o[3] = 2.f * RX(x, 0) * RX(x, 1); o[4] = 2.f * RX(x, 2) * RX(x, 1); o[5] = 2.f * RX(x, 0) * RX(x, 2);
  } else {
    const int x = r == 4 ? 1 : 0, y = r == 3 ? 1 : 2;
    o[0] = RX(x, 0) * RX(y, 0); o[1] = RX(x, 1) * RX(y, 1); o[2] = RX(x, 2) * RX(y, 2);
    o[3] = RX(x, 0) * RX(y, 1) + RX(y, 0) * RX(x, 1);
    o[4] = RX(x, 1) * RX(y, 2) + RX(x, 2) * RX(y, 1);
    o[5] = RX(x, 0) * RX(y, 2) + RX(x, 2) * RX(y, 0);
  }
#undef RX
}

// Per-point intermediates of the tangent kernels in shared memory,
// [quantity][point] floats (kS points per quantity, so that consecutive
// threads read consecutive words)
constexpr int kPtGam = 0;                 // Gamma (9)
constexpr int kPtF = kPtGam + 9;          // w det[J]
constexpr int kPtT = kPtF + 1;            // Cauchy stress at n+1 (6)
constexpr int kPtC = kPtT + 6;            // cep (21), unscaled
constexpr int kPtD = kPtC + 21;           // [D*] lower triangle (21), with w det[J]; [J] rows before phase 2
constexpr int kPtTw = kPtD + 21;          // w det[J] {T} (6)
constexpr int kPtR = kPtTw + 6;           // R at n+1, column-major (9)
constexpr int kPtU = kPtR + 9;            // unrotated stress urcs_n1 (6)
constexpr int kPtN = kPtU + 6;            // 79 quantities

template <int kS>
__device__ __forceinline__ float& pv(float* pt, int q, int p) { return pt[q * kS + p]; }

// row r of [q] (q_row) from R in the per-point arrays
template <int r, int kS>
__device__ __forceinline__ void q_row_pt(float* pt, int p, float* o) {
  constexpr int x = r < 3 ? r : (r == 4 ? 1 : 0), y = r < 3 ? r : (r == 3 ? 1 : 2);
  float R[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int j = 0; j < 3; ++j) {   // the rows of R that row r of [q] uses
    R[x + 3 * j] = pv<kS>(pt, kPtR + x + 3 * j, p);
    if (y != x) R[y + 3 * j] = pv<kS>(pt, kPtR + y + 3 * j, p);
  }
  q_row(R, r, o);
}

// Phase 2a, thread k of a point: k = 0 inverts [J] (rows in the [D*]
// slots) into Gamma and forms w det[J] (w: the Gauss weight; cofactor
// inverse, as jacobian_inverse); with finite strain every k forms the
// Cauchy stress component {T}_k = [q]_k {urcs_n1}.
template <int k, int kS>
__device__ __forceinline__ void pt_phase2a(float* pt, int p, float w, bool geonl) {
  if constexpr (k == 0) {
    const float j11 = pv<kS>(pt, kPtD + 0, p), j12 = pv<kS>(pt, kPtD + 1, p), j13 = pv<kS>(pt, kPtD + 2, p);
    const float j21 = pv<kS>(pt, kPtD + 3, p), j22 = pv<kS>(pt, kPtD + 4, p), j23 = pv<kS>(pt, kPtD + 5, p);
    const float j31 = pv<kS>(pt, kPtD + 6, p), j32 = pv<kS>(pt, kPtD + 7, p), j33 = pv<kS>(pt, kPtD + 8, p);
    const float c1 = j22 * j33 - j23 * j32, c2 = j21 * j33 - j23 * j31, c3 = j21 * j32 - j22 * j31;
    const float dj = j11 * c1 - j12 * c2 + j13 * c3, rdj = 1.f / dj;
    pv<kS>(pt, kPtGam + 0, p) = c1 * rdj;
    pv<kS>(pt, kPtGam + 1, p) = -c2 * rdj;
    pv<kS>(pt, kPtGam + 2, p) = c3 * rdj;
    pv<kS>(pt, kPtGam + 3, p) = (j32 * j13 - j12 * j33) * rdj;
    pv<kS>(pt, kPtGam + 4, p) = (j11 * j33 - j31 * j13) * rdj;
    pv<kS>(pt, kPtGam + 5, p) = (j12 * j31 - j11 * j32) * rdj;
    pv<kS>(pt, kPtGam + 6, p) = (j12 * j23 - j13 * j22) * rdj;
    pv<kS>(pt, kPtGam + 7, p) = (j13 * j21 - j11 * j23) * rdj;
    pv<kS>(pt, kPtGam + 8, p) = (j11 * j22 - j12 * j21) * rdj;
    pv<kS>(pt, kPtF, p) = w * dj;
  }
  if (geonl) {
    float o[6];
    q_row_pt<k, kS>(pt, p, o);
    float t = 0.f;
#pragma unroll
    for (int m = 0; m < 6; ++m) t += o[m] * pv<kS>(pt, kPtU + m, p);
    pv<kS>(pt, kPtT + k, p) = t;
  }
}

// Q-bar entry (j, c), c <= j, of ctran1 with qbar, without the factor
// w det[J], from the Cauchy stress (xx yy zz xy yz xz)
template <int J, int Cc, int kS>
__device__ __forceinline__ float qbar_entry(float* pt, int p) {
  constexpr int q = lw(J, Cc);
  auto t = [&](int m) { return pv<kS>(pt, kPtT + m, p); };
  if constexpr (q == 0) return 2.f * t(0);
  if constexpr (q == 2) return 2.f * t(1);
  if constexpr (q == 5) return 2.f * t(2);
  if constexpr (q == 6 || q == 7 || q == 19) return t(3);
  if constexpr (q == 11 || q == 12 || q == 18) return t(4);
  if constexpr (q == 13 || q == 15 || q == 17) return t(5);
  if constexpr (q == 9) return 0.5f * (t(0) + t(1));
  if constexpr (q == 14) return 0.5f * (t(1) + t(2));
  if constexpr (q == 20) return 0.5f * (t(0) + t(2));
  return 0.f;
}

template <int J, int kS>
__device__ __forceinline__ float qbar_entry_dispatch(int c, float* pt, int p) {
  switch (c) {
    case 0: return qbar_entry<J, 0, kS>(pt, p);
    case 1: return qbar_entry<J, 1, kS>(pt, p);
    case 2: return qbar_entry<J, 2, kS>(pt, p);
    case 3: return qbar_entry<J, 3, kS>(pt, p);
    case 4: return qbar_entry<J, 4, kS>(pt, p);
    default: return qbar_entry<J, 5, kS>(pt, p);
  }
}

template <int kS>
__device__ __forceinline__ void q_row_dispatch(int c, float* pt, int p, float* o) {
  switch (c) {
    case 0: q_row_pt<0, kS>(pt, p, o); break;
    case 1: q_row_pt<1, kS>(pt, p, o); break;
    case 2: q_row_pt<2, kS>(pt, p, o); break;
    case 3: q_row_pt<3, kS>(pt, p, o); break;
    case 4: q_row_pt<4, kS>(pt, p, o); break;
    default: q_row_pt<5, kS>(pt, p, o); break;
  }
}

// Phase 2, thread J of the point: row J of w det[J] [D*] = [q][D][q]^T -
// Q-bar (lower triangle, columns c <= J), and w det[J] {T}_J; without
// finite strain [D*] = [D] and no {T}.
template <int J, int kS>
__device__ __forceinline__ void pt_phase2(bool qbar, int flags, float* pt, int p) {
  const float f = pv<kS>(pt, kPtF, p);
  if (flags & 1) {
    // the rows of [q] this thread needs are formed from R in registers
    // (cheaper than reading them from shared memory six times over)
    float qj[6], tc[6];
    q_row_pt<J, kS>(pt, p, qj);
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      float v = 0.f;
#pragma unroll
      for (int m = 0; m < 6; ++m) v += qj[m] * pv<kS>(pt, kPtC + lw(m, c), p);
      tc[c] = v;
    }
#pragma unroll
    for (int c = 0; c <= J; ++c) {
      float qc[6];
      q_row_dispatch<kS>(c, pt, p, qc);
      float v = 0.f;
#pragma unroll
      for (int m = 0; m < 6; ++m) v += tc[m] * qc[m];
      v *= f;
      if (qbar) v -= f * qbar_entry_dispatch<J, kS>(c, pt, p);
      pv<kS>(pt, kPtD + lw(J, c), p) = v;
    }
    pv<kS>(pt, kPtTw + J, p) = pv<kS>(pt, kPtT + J, p) * f;
  } else {
#pragma unroll
    for (int c = 0; c <= J; ++c) pv<kS>(pt, kPtD + lw(J, c), p) = f * pv<kS>(pt, kPtC + lw(J, c), p);
    pv<kS>(pt, kPtTw + J, p) = 0.f;
  }
}

}  // namespace tc
}  // namespace w3g
