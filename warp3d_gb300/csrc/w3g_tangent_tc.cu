// w3g_tangent_tc.cu -- precision forms of the 8-node brick tangent on the
// fifth-generation tensor cores: Ke = sum_gp B^T [D*] B in TF32 or BF16
// operands with FP32 accumulation (tcgen05.mma, accumulator in tensor
// memory), plus the geometric stiffness G^T T G in FP32 on the CUDA cores.
//
// One CTA (8 warps) = one tile of up to 5 elements of one block. Per
// element the material part is a 24 x 24 x 48 product: with the 48
// contraction indices (Gauss point, strain component) as K,
//   A (dof x K) = B^T,   Bop (dof x K) = ([D*] B)^T,   Ke = A Bop^T.
// The tile stacks the 5 elements' dofs: M = 5 x 24 = 120 rows (+8 padding)
// and N = 128 columns, so a single MMA chain (6 k-steps of 8 for TF32, 3 of
// 16 for BF16) produces all element pairs; the 5 diagonal 24 x 24 blocks are
// the element matrices (the rest is discarded: the tensor core has the
// throughput to spare, the tangent is bound by its operands and Ke in HBM).
//
//   phase 1  per (element, Gauss point), 6 threads each (240 of 256): the
//            gradients at x(n+1), the rotation q(R), and one row each of
//            w det[J] [D*] = [q][D][q]^T - Q-bar, and w det[J] {T}, to
//            shared memory (FP32)
//   phase 2  operands written in the canonical no-swizzle K-major layout
//            (8-row x 16-byte core matrices), one 16-byte store per core
//            matrix row; geometric stiffness per node pair;
//            fence.proxy.async
//   phase 3  thread 0 issues the MMAs (tcgen05.mma.cta_group::1 with shared
//            memory descriptors) and commits to an mbarrier; all threads
//            wait (bounded)
//   phase 4  warps 0-3 read their 32 TMEM lanes (rows) with tcgen05.ld; the
//            element matrices are symmetrised, the geometric part added,
//            and each is projected onto the matrices that annihilate rigid
//            translations, K' = P K P with P = I - T T^T / 8 (T: the three
//            unit translations of the element's 8 nodes); Ke is staged in
//            shared memory and stored coalesced (FP32)
//
// The projection. The exact element tangent annihilates rigid translations
// (the shape-function gradients sum to zero at every point), so P Ke P = Ke
// in exact arithmetic; rounding the operands to 11 (TF32) or 8 (BF16)
// significant bits breaks this at the level of the format's unit roundoff,
// and the tensor core's FP32 accumulation adds a systematic bias on the
// diagonal. Assembled over the mesh, that error acts coherently on the
// near-rigid modes that only the displacement constraints hold (its energy
// grows with the element count while theirs does not), and the global
// Newton iteration stops converging on large meshes. The projection removes
// exactly that component of the error and nothing of the exact matrix.
#include <cstdint>
#include <cuda_bf16.h>
#include "w3g_internal.cuh"
#include "w3g_elem.cuh"
#include "w3g_math.cuh"
#include "w3g_tangent_items.cuh"

namespace w3g {

namespace {

constexpr int NN = Hex8::NN, NG = Hex8::NG, TOT = Hex8::TOTDOF, UT = Hex8::UTSZ;
constexpr int kTcElems = 5;            // elements per tile
constexpr int kTcRows = kTcElems * TOT;   // 120 live rows
constexpr int kRows = 128;             // M = N
constexpr int kK = NG * 6;             // 48
constexpr int kThreads = 256;
constexpr int kSubs = 6;               // threads per (element, Gauss point) in phase 1
constexpr int kTmemCols = 128;
constexpr int kKfStride = TOT + 1;     // padded row of the staged element matrices
constexpr long long kDrainLimit = 1ll << 26;  // polls waiting out MMAs in flight after a wait gave up

template <bool kBF16>
struct TcLayout {
  static constexpr int kBytes = kBF16 ? 2 : 4;
  static constexpr int kPerCore = 16 / kBytes;          // K elements per core-matrix row
  static constexpr int kChunks = kK / kPerCore;         // core matrices along K
  static constexpr int kLBO = 128;                      // next core matrix along K
  static constexpr int kSBO = kChunks * 128;            // next 8-row group
  static constexpr int kOpBytes = kRows * kK * kBytes;  // one operand
  static constexpr int kKStep = kBF16 ? 16 : 8;         // K per MMA
  static constexpr int kSteps = kK / kKStep;
  __device__ static __forceinline__ int offset(int r, int chunk) {
    return (r >> 3) * kSBO + chunk * kLBO + (r & 7) * 16;
  }
};

struct TcStatic {
  float dn[NG * 3 * NN + NG];
  float x[kTcElems][3 * NN];
  float g[kTcElems][NG][3 * NN];
  float D[kTcElems][NG][21];
  float T[kTcElems][NG][6];
  float kg[kTcElems][36];            // b-bar: det[J] per Gauss point until phase 2
  union {
    struct {                         // phase 1
      float C[kTcElems][NG][21];
      float cs[kTcElems][NG][6];
      float R[kTcElems][NG][9];
      float ur[kTcElems][NG][6];
    } p1;
    struct {                         // b-bar, phase 2
      float v[kTcElems][3 * NN];     // volume-averaged gradients
    } p2;
    struct {                         // phase 4
      float mrow[kTcRows][3];        // row means over the nodes, per column component
      float mblk[kTcElems][9];       // means of the row means, per (row, column) component
    } p4;
  } u;
  unsigned long long mbar;
  uint32_t tmem_base;
  int timeout;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// tcgen05 shared-memory matrix descriptor: start, leading (K) and stride
// (M/N) byte offsets in 16-byte units, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, int lbo, int sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor (kind::tf32 / kind::f16): FP32 accumulator, A and
// B both K-major, M = N = 128
template <bool kBF16>
__host__ __device__ constexpr uint32_t instr_desc() {
  return (1u << 4)                             // D format: F32
         | ((kBF16 ? 1u : 2u) << 7)            // A format: BF16 = 1, TF32 = 2
         | ((kBF16 ? 1u : 2u) << 10)           // B format
         | ((uint32_t)(kRows >> 3) << 17)      // N >> 3
         | ((uint32_t)(kRows >> 4) << 24);     // M >> 4
}

// one tcgen05.mma: D[tmem] (+)= A B^T over one K step, both operands in
// shared memory (K-major, no swizzle)
template <bool kBF16>
__device__ __forceinline__ void mma(uint32_t tmem, uint32_t a_addr, uint32_t b_addr, bool accumulate) {
  using L = TcLayout<kBF16>;
  const uint64_t da = smem_desc(a_addr, L::kLBO, L::kSBO);
  const uint64_t db = smem_desc(b_addr, L::kLBO, L::kSBO);
  const uint32_t idesc = instr_desc<kBF16>();
  const uint32_t acc = accumulate ? 1u : 0u;
  if (kBF16)
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
        "l"(da), "l"(db), "r"(idesc), "r"(acc));
  else
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
        "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

// Operands are rounded to the input format to nearest (the tensor core
// would otherwise drop the low mantissa bits of an FP32 operand). With
// kSplit, v = hi + lo with both parts in the input format, and the product
// of two split operands is taken as hi*hi + hi*lo + lo*hi (the lo*lo term is
// below FP32 rounding for TF32): three MMAs instead of one, and an error
// near FP32's for TF32 (about 2^-16 relative for BF16).
template <bool kBF16>
__device__ __forceinline__ float round_in(float v) {
  if (kBF16) return __bfloat162float(__float2bfloat16_rn(v));
  uint32_t t;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v));
  return __uint_as_float(t);
}

// one core-matrix row (16 bytes) of an operand: kPerCore consecutive K
// values of row r, split into hi and lo parts when kSplit
template <bool kBF16, bool kSplit>
__device__ __forceinline__ void put_chunk(unsigned char* op, int r, int chunk, const float* v) {
  using L = TcLayout<kBF16>;
  const int o = L::offset(r, chunk);
  float hi[L::kPerCore], lo[L::kPerCore];
#pragma unroll
  for (int j = 0; j < L::kPerCore; ++j) {
    hi[j] = round_in<kBF16>(v[j]);
    lo[j] = kSplit ? round_in<kBF16>(v[j] - hi[j]) : 0.f;
  }
  uint4 wh, wl;
  if (kBF16) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      h[j] = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(hi[2 * j])) |
             ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(hi[2 * j + 1])) << 16);
      l[j] = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(lo[2 * j])) |
             ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(lo[2 * j + 1])) << 16);
    }
    wh = make_uint4(h[0], h[1], h[2], h[3]);
    wl = make_uint4(l[0], l[1], l[2], l[3]);
  } else {
    wh = make_uint4(__float_as_uint(hi[0]), __float_as_uint(hi[1]), __float_as_uint(hi[2]), __float_as_uint(hi[3]));
    wl = make_uint4(__float_as_uint(lo[0]), __float_as_uint(lo[1]), __float_as_uint(lo[2]), __float_as_uint(lo[3]));
  }
  *reinterpret_cast<uint4*>(op + o) = wh;
  if (kSplit) *reinterpret_cast<uint4*>(op + 2 * L::kOpBytes + o) = wl;   // A_lo after B_hi, B_lo after A_lo
}

// row j (run-time) of the 6x6 q held in registers, without local memory
__device__ __forceinline__ void row_of(const float* q, int j, float* out) {
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    float v = q[m];
#pragma unroll
    for (int jj = 1; jj < 6; ++jj) v = j == jj ? q[6 * jj + m] : v;
    out[m] = v;
  }
}

// kBbar: the instantiation launched for models with b-bar blocks (the
// others keep the operand code without the b-bar terms)
template <bool kBF16, bool kSplit, bool kBbar>
__global__ void __launch_bounds__(kThreads, 4) k_tangent_tc_hex8(TangentArgs a, int chunk0, int* tc_timeout) {
  using L = TcLayout<kBF16>;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* opA = smem;                  // then B, then (split) A_lo, B_lo
  unsigned char* opB = smem + L::kOpBytes;
  __shared__ TcStatic S;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const Chunk ch = a.chunks[chunk0 + blockIdx.x];
  const BlockDesc bd = a.blocks[ch.blk];

  // ---- TMEM allocation (warp 0) and mbarrier ----
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem_base)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&S.mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
    S.timeout = 0;
  }
  for (int k = tid; k < NG * 3 * NN + NG; k += kThreads) S.dn[k] = a.dn32[0][k];
  // ---- gather: x(n+1) relative to node 1, one coordinate per thread ----
  if (tid < kTcElems * 3 * NN) {
    const int e = tid / (3 * NN), dn = tid % (3 * NN), d = dn / NN, node = dn % NN;
    if (e < ch.n) {
      const long long dbase = bd.einf_off + (long long)(ch.i0 + e) * TOT;
      double ref = a.c[a.cdest[dbase + d * NN] - 1];
      double v = a.c[a.cdest[dbase + d * NN + node] - 1];
      if (bd.geonl) {
        const int e0 = a.edest[dbase + d * NN] - 1, e1 = a.edest[dbase + d * NN + node] - 1;
        ref = ref + a.u[e0] + a.du[e0];
        v = v + a.u[e1] + a.du[e1];
      }
      S.x[e][dn] = d2f_rn(v - ref);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = S.tmem_base;

  // ---- phase 1: 6 threads per (element, Gauss point) ----
  const int item = tid / kSubs, sub = tid % kSubs;
  const int pe = item / NG, pgp = item % NG;
  const bool p1 = tid < kTcElems * NG * kSubs && pe < ch.n;
  float q[36];
  float f = 0.f, dj = 0.f;
  if (p1) {
    const int i = ch.i0 + pe;
    const float* dnx = S.dn + (pgp * 3 + 0) * NN;
    const float* dne = S.dn + (pgp * 3 + 1) * NN;
    const float* dnz = S.dn + (pgp * 3 + 2) * NN;
    const float w = S.dn[NG * 3 * NN + pgp];
    float gama[9];
    jacobian_inverse<NN, float>(dnx, dne, dnz, S.x[pe], S.x[pe] + NN, S.x[pe] + 2 * NN, gama, dj);
    float* g = S.g[pe][pgp];
    for (int n = sub; n < NN; n += kSubs)
      shape_gradient<float>(gama, dnx[n], dne[n], dnz[n], g[3 * n], g[3 * n + 1], g[3 * n + 2]);
    f = w * dj;
    if (kBbar && sub == 0) S.kg[pe][pgp] = dj;
    // w det[J] [D], lower triangle row-wise, entries sub, sub + 6, ... (as
    // load_D21: cep_blocks, or for mm10 history1 words 0-35)
    if (bd.mat == W3G_MAT_CRYSTAL) {
      const double* H = a.hist1 + bd.hist_off + ((long long)i * NG + pgp) * kHistMM10;
      for (int k = sub; k < 21; k += kSubs) {
        int r = 0, c = k;
        while (c > r) { c -= r + 1; ++r; }   // k = r(r+1)/2 + c, c <= r
        S.u.p1.C[pe][pgp][k] = f * d2f_rn(H[r + 6 * c]);
      }
    } else {
      const long long cb = bd.cep_off + ((long long)pgp * bd.span + i) * 21;
      for (int k = sub; k < 21; k += kSubs) S.u.p1.C[pe][pgp][k] = f * d2f_rn(a.cep[cb + k]);
    }
    if (bd.geonl) {
      // R and the unrotated stress: each value loaded and converted once
      const long long gpi = bd.gp_off + (long long)i * NG + pgp;
      S.u.p1.R[pe][pgp][sub] = d2f_rn(a.rot_n1[gpi * 9 + sub]);
      if (sub < 3) S.u.p1.R[pe][pgp][sub + 6] = d2f_rn(a.rot_n1[gpi * 9 + sub + 6]);
      S.u.p1.ur[pe][pgp][sub] = d2f_rn(a.urcs_n1[gpi * 9 + sub]);
    }
  }
  __syncthreads();
  if (p1 && bd.geonl) {
    rotation_q2<float>(S.u.p1.R[pe][pgp], q);
    float qrow[6];
    row_of(q, sub, qrow);
    const float* ur = S.u.p1.ur[pe][pgp];
    float s = 0.f;
    for (int m = 0; m < 6; ++m) s += qrow[m] * ur[m];
    S.u.p1.cs[pe][pgp][sub] = s;   // Cauchy stress component `sub`
  }
  __syncthreads();
  if (p1) {
    float* D = S.D[pe][pgp];
    const float* C = S.u.p1.C[pe][pgp];
    const int j = sub;
    if (bd.geonl) {
      // row j of q C q^T (entries kk <= j), then the Q-bar terms of row j
      float tc[6], qrow[6];
      row_of(q, j, qrow);
#pragma unroll
      for (int kk = 0; kk < 6; ++kk) {
        float s = 0.f;
#pragma unroll
        for (int m = 0; m < 6; ++m) s += qrow[m] * C[low(m, kk)];
        tc[kk] = s;
      }
#pragma unroll
      for (int kk = 0; kk < 6; ++kk) {
        float s = 0.f;
#pragma unroll
        for (int m = 0; m < 6; ++m) s += tc[m] * q[6 * kk + m];
        if (kk <= j) D[low(j, kk)] = s;
      }
      const float* cs = S.u.p1.cs[pe][pgp];
      if (a.qbar) {
        const float wf = f, halfw = 0.5f * wf;
        const float xx = cs[0], yy = cs[1], zz = cs[2], xy = cs[3], yz = cs[4], xz = cs[5];
        switch (j) {
          case 0: D[low(0, 0)] -= 2.f * xx * wf; break;
          case 1: D[low(1, 1)] -= 2.f * yy * wf; break;
          case 2: D[low(2, 2)] -= 2.f * zz * wf; break;
          case 3:
            D[low(3, 0)] -= xy * wf;
            D[low(3, 1)] -= xy * wf;
            D[low(3, 3)] -= halfw * (xx + yy);
            break;
          case 4:
            D[low(4, 1)] -= yz * wf;
            D[low(4, 2)] -= yz * wf;
            D[low(4, 3)] -= wf * xz;
            D[low(4, 4)] -= halfw * (yy + zz);
            break;
          default:
            D[low(5, 0)] -= xz * wf;
            D[low(5, 2)] -= xz * wf;
            D[low(5, 3)] -= wf * yz;
            D[low(5, 4)] -= wf * xy;
            D[low(5, 5)] -= halfw * (xx + zz);
            break;
        }
      }
      S.T[pe][pgp][j] = cs[j] * f;
    } else {
      for (int kk = 0; kk <= j; ++kk) D[low(j, kk)] = C[low(j, kk)];
      S.T[pe][pgp][j] = 0.f;
    }
  }
  __syncthreads();
  // b-bar: volume-averaged gradients (vol_terms + vol_avg), one thread per
  // (element, node, component)
  if (kBbar) {
    if (bd.bbar && tid < kTcElems * 3 * NN) {
      const int e = tid / (3 * NN), k = tid % (3 * NN);
      if (e < ch.n) {
        float sv = 0.f, vol = 0.f;
        for (int gp = 0; gp < NG; ++gp) {
          sv += S.g[e][gp][k] * S.kg[e][gp];
          vol += S.kg[e][gp];
        }
        S.u.p2.v[e][k] = sv * (1.f / vol);
      }
    }
    __syncthreads();
  }

  // ---- phase 2: operands (row = 24 e + dof, dof = 8 i + a; k = 6 gp + m).
  // Threads 0-127 write row r of A = B^T, threads 128-255 row r of
  // Bop = ([D*] B)^T, half of the Gauss points at a time from registers.
  // Column (i, a) of B has three non-zeros: strain components p0..p2 take
  // gradient components c0..c2 of node a:
  //   i = 0: (xx, xy, xz) <- (gx, gy, gz)   i = 1: (yy, xy, yz) <- (gy, gx, gz)
  //   i = 2: (zz, yz, xz) <- (gz, gy, gx)
  {
    const int r = tid & (kRows - 1);
    const bool isB = tid >= kRows;
    const int e = r / TOT, d = r % TOT, di = d / NN, na = d % NN;
    const bool live = r < kTcRows && e < ch.n;
    const int ee = live ? e : 0;
    const int p0 = di, p1 = di == 2 ? 4 : 3, p2 = di == 0 ? 5 : di == 1 ? 4 : 5;
    const int c0 = di, c1 = di == 0 ? 1 : di == 1 ? 0 : 1, c2 = di == 2 ? 0 : 2;
    int ix[6][3];   // packed [D*] index of (m, p_j)
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      ix[m][0] = low(m, p0);
      ix[m][1] = low(m, p1);
      ix[m][2] = low(m, p2);
    }
    unsigned char* op = isB ? opB : opA;
    // b-bar (bmod): column (i, a) of B-bar adds h = beta (v_ai - g_ai) to
    // the three normal rows; [D*] B-bar adds h times the row sums of the
    // first three columns of [D*]
    const bool bb = kBbar && bd.bbar != 0;
    const float beta = (float)a.bbar_beta;
    const float va = bb ? S.u.p2.v[ee][3 * na + di] : 0.f;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      float v[kK / 2];
#pragma unroll
      for (int q4 = 0; q4 < NG / 2; ++q4) {
        const int gp = (NG / 2) * h + q4;
        const float* g = S.g[ee][gp] + 3 * na;
        const float u0 = g[c0], u1 = g[c1], u2 = g[c2];
        const float hb = bb ? beta * (va - u0) : 0.f;
        const float* D = S.D[ee][gp];
#pragma unroll
        for (int m = 0; m < 6; ++m) {
          float val;
          if (isB) {
            val = D[ix[m][0]] * u0 + D[ix[m][1]] * u1 + D[ix[m][2]] * u2;
            if (kBbar) val += hb * (D[low(m, 0)] + D[low(m, 1)] + D[low(m, 2)]);
          } else {
            val = m == p0 ? u0 : m == p1 ? u1 : m == p2 ? u2 : 0.f;
            if (kBbar && m < 3) val += hb;
          }
          v[6 * q4 + m] = live ? val : 0.f;
        }
      }
#pragma unroll
      for (int c = 0; c < L::kChunks / 2; ++c)
        put_chunk<kBF16, kSplit>(op, r, (L::kChunks / 2) * h + c, v + c * L::kPerCore);
    }
  }
  // geometric stiffness per node pair (kgstiff): sum_gp g_a . ({T} g_b)
  if (tid < kTcElems * 36) {
    const int e = tid / 36, p = tid % 36;
    int na = 0, r = p;
    while (r >= NN - na) { r -= NN - na; ++na; }
    const int nb = na + r;
    float s = 0.f;
    if (e < ch.n && bd.geonl)
      for (int gp = 0; gp < NG; ++gp) {
        const float* g = kBbar && bd.bbar ? S.u.p2.v[e] : S.g[e][gp];   // b-bar: averaged gradients (kg1.f:46-54)
        const float* Tw = S.T[e][gp];
        const float bx = g[3 * nb], by = g[3 * nb + 1], bz = g[3 * nb + 2];
        const float t0 = Tw[0] * bx + Tw[3] * by + Tw[5] * bz;
        const float t1 = Tw[3] * bx + Tw[1] * by + Tw[4] * bz;
        const float t2 = Tw[5] * bx + Tw[4] * by + Tw[2] * bz;
        s += g[3 * na] * t0 + g[3 * na + 1] * t1 + g[3 * na + 2] * t2;
      }
    S.kg[e][p] = s;
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();

  // ---- phase 3: MMA chain (one thread), completion on the mbarrier ----
  // A wait limit of 0 gives up before any MMA is issued.
  const bool issue = a.wait_limit > 0;
  if (tid == 0 && issue) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t a0 = smem_u32(opA), b0 = smem_u32(opB);
    const uint32_t lo = 2 * L::kOpBytes;   // A_lo, B_lo follow A_hi, B_hi
#pragma unroll
    for (int s = 0; s < L::kSteps; ++s) {
      // one k-step = two core matrices along K
      const uint32_t ks = s * 2 * L::kLBO;
      mma<kBF16>(tmem, a0 + ks, b0 + ks, s > 0);
      if (kSplit) {
        mma<kBF16>(tmem, a0 + ks, b0 + lo + ks, true);
        mma<kBF16>(tmem, a0 + lo + ks, b0 + ks, true);
      }
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
        smem_u32(&S.mbar)));
  }
  // bounded wait on phase 0 of the mbarrier; after giving up, the MMAs
  // that were issued may still be running: they are waited out (bounded)
  // before tensor memory is read or freed
  {
    auto poll = [&](long long limit) {
      uint32_t done = 0;
      for (long long polls = 0; !done && polls < limit; ++polls)
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\nselp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(smem_u32(&S.mbar)));
      return done != 0;
    };
    if (!poll(a.wait_limit)) {
      S.timeout = 1;
      if (issue) poll(kDrainLimit);
    }
  }
  asm volatile("tcgen05.fence::after_thread_sync;");
  __syncthreads();
  const bool ok = S.timeout == 0;

  // ---- phase 4: TMEM -> element matrices (full, FP32) in shared memory ----
  // [kTcElems][24][kKfStride]: rows padded to 25 words so that column reads
  // by consecutive rows fall in distinct banks; operands are consumed
  float* kf = reinterpret_cast<float*>(opA);
  float* ke = reinterpret_cast<float*>(opA) + kTcElems * TOT * kKfStride;   // [kTcElems][UT]
  if (warp < 4 && ok) {
    const int r = 32 * warp + lane;
    const int e = r / TOT, dr = r % TOT;
    // the 32-column TMEM chunks holding this warp's elements' columns
    const int e_lo = (32 * warp) / TOT, e_hi = min(kTcElems - 1, (32 * warp + 31) / TOT);
    const int p_lo = (TOT * e_lo) / 32, p_hi = min(kRows / 32 - 1, (TOT * e_hi + TOT - 1) / 32);
    for (int pass = p_lo; pass <= p_hi; ++pass) {
      uint32_t v[32];
      const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(32 * pass);
      asm volatile(   // the load and its wait in one statement: no use of v before the wait
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
          "tcgen05.wait::ld.sync.aligned;"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
            "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
            "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
            "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
          : "r"(taddr)
          : "memory");
      if (r < kTcRows) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int dc = 32 * pass + j - TOT * e;
          if (dc >= 0 && dc < TOT) kf[(e * TOT + dr) * kKfStride + dc] = __uint_as_float(v[j]);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  // symmetrise, add the geometric part, row means over the nodes
  float krow[TOT];
  const int r = tid;
  const int e = r / TOT, dr = r % TOT, ir = dr / NN, ar = dr % NN;
  const bool row_live = r < kTcRows && e < ch.n;
  if (row_live) {
    const float* K = kf + e * TOT * kKfStride;
    float m3[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int dc = 0; dc < TOT; ++dc) {
      const int ic = dc / NN, ac = dc % NN;
      float val = 0.5f * (K[dr * kKfStride + dc] + K[dc * kKfStride + dr]);
      if (ic == ir) {
        const int lo = ar < ac ? ar : ac, hi = ar < ac ? ac : ar;
        val += S.kg[e][lo * NN - lo * (lo - 1) / 2 + (hi - lo)];
      }
      krow[dc] = val;
      m3[ic] += val;
    }
#pragma unroll
    for (int j = 0; j < 3; ++j) S.u.p4.mrow[r][j] = m3[j] * (1.f / NN);
  }
  __syncthreads();
  if (tid < kTcElems * 9) {
    const int be = tid / 9, i = (tid % 9) / 3, j = tid % 3;
    float s = 0.f;
    if (be < ch.n)
      for (int an = 0; an < NN; ++an) s += S.u.p4.mrow[be * TOT + i * NN + an][j];
    S.u.p4.mblk[be][tid % 9] = s * (1.f / NN);
  }
  __syncthreads();
  // K' = P K P: subtract the row and column means, add back the block mean
  if (row_live) {
    const float bf = (float)a.beta_fact;
    const float* mr = S.u.p4.mrow[r];
#pragma unroll
    for (int dc = 0; dc < TOT; ++dc) {
      if (dc < dr) continue;
      const int ic = dc / NN;
      const float val = krow[dc] - mr[ic] - S.u.p4.mrow[e * TOT + dc][ir] + S.u.p4.mblk[e][ir * 3 + ic];
      ke[e * UT + dc * (dc + 1) / 2 + dr] = ok ? val * bf : __int_as_float(0x7fc00000);
    }
  }
  __syncthreads();
  if (tid == 0 && !ok) atomicExch(tc_timeout, 1);
  float* out = reinterpret_cast<float*>(a.estiff);
  const long long obase = bd.estiff_off + (long long)ch.i0 * UT;
  for (int k = tid; k < ch.n * UT; k += kThreads) out[obase + k] = ke[k];
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
  }
}

// Dynamic shared memory per CTA: A and B (and their low parts when split),
// re-used in phase 4 for the full element matrices and the packed result.
// At least kMinDyn, so that with the static part no more than four CTAs fit
// in an SM's 228 KB and their 4 x 128 TMEM columns always fit in its 512:
// tcgen05.alloc then never has to wait for another CTA's columns.
constexpr int kMinDyn = 30 * 1024;
static_assert(sizeof(TcStatic) + kMinDyn + 1024 > 228 * 1024 / 5, "five CTAs could share an SM's TMEM");
// the split forms (four operands, 96 KB) fit two CTAs in an SM's 228 KB
// only while the static part, rounded to 1 KB, stays within 17 KB
static_assert(sizeof(TcStatic) <= 17 * 1024, "split-form tiles would drop to one CTA per SM");
static_assert((kTcElems * TOT * kKfStride + kTcElems * UT) * 4 <= kMinDyn, "phase-4 staging exceeds shared memory");

template <bool kBF16, bool kSplit>
size_t tc_smem() {
  const size_t need = (kSplit ? 4 : 2) * (size_t)TcLayout<kBF16>::kOpBytes;
  return need > (size_t)kMinDyn ? need : (size_t)kMinDyn;
}
static_assert(kTcElems * NG * kSubs <= kThreads && kTcRows <= kThreads, "tile larger than the CTA");

template <bool kBF16, bool kSplit>
cudaError_t set_smem() {
  cudaError_t e = cudaFuncSetAttribute(k_tangent_tc_hex8<kBF16, kSplit, false>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_smem<kBF16, kSplit>());
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_tangent_tc_hex8<kBF16, kSplit, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)tc_smem<kBF16, kSplit>());
}

template <bool kBF16, bool kSplit>
void launch(const DeviceModel& m, const TangentArgs& h, int* tc_timeout, cudaStream_t s) {
  if (m.has_bbar)
    k_tangent_tc_hex8<kBF16, kSplit, true><<<m.ntcchunks, kThreads, tc_smem<kBF16, kSplit>(), s>>>(h, 0, tc_timeout);
  else
    k_tangent_tc_hex8<kBF16, kSplit, false><<<m.ntcchunks, kThreads, tc_smem<kBF16, kSplit>(), s>>>(h, 0, tc_timeout);
}

}  // namespace

cudaError_t init_tangent_tc_kernels() {
  cudaError_t e = set_smem<false, false>();
  if (e == cudaSuccess) e = set_smem<true, false>();
  if (e == cudaSuccess) e = set_smem<false, true>();
  if (e == cudaSuccess) e = set_smem<true, true>();
  return e;
}

cudaError_t launch_tangent_tc_hex8(const DeviceModel& m, const TangentArgs& a, bool bf16, bool split,
                                   int* tc_timeout, cudaStream_t s) {
  if (m.ntcchunks == 0) return cudaSuccess;
  TangentArgs h = a;
  h.chunks = m.tcchunks;
  if (bf16) split ? launch<true, true>(m, h, tc_timeout, s) : launch<true, false>(m, h, tc_timeout, s);
  else split ? launch<false, true>(m, h, tc_timeout, s) : launch<false, false>(m, h, tc_timeout, s);
  return cudaGetLastError();
}

}  // namespace w3g
