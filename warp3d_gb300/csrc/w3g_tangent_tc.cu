// w3g_tangent_tc.cu -- precision form of the 8-node brick tangent on the
// fifth-generation tensor cores: Ke = sum_gp B^T [D*] B in TF32 or BF16
// operands with FP32 accumulation (tcgen05.mma, accumulator in tensor
// memory), plus the geometric stiffness G^T T G in FP32 on the CUDA cores.
//
// One CTA (4 warps) = one tile of up to 5 elements of one block. Per
// element the material part is a 24 x 24 x 48 product: with the 48
// contraction indices (Gauss point, strain component) as K,
//   A (dof x K) = B^T,   Bop (dof x K) = ([D*] B)^T,   Ke = A Bop^T.
// The tile stacks the 5 elements' dofs: M = 5 x 24 = 120 rows (+8 padding)
// and N = 128 columns, so a single MMA chain (6 k-steps of 8 for TF32, 3 of
// 16 for BF16) produces all element pairs; the 5 diagonal 24 x 24 blocks are
// the element matrices (the rest is discarded: the tensor core has the
// throughput to spare, the tangent is bound by its operands and Ke in HBM).
//
//   phase 1  (40 threads) per (element, Gauss point) as in the FP32 kernel:
//            gradients at x(n+1), w det[J] [D*] = [q][D][q]^T - Q-bar, and
//            w det[J] {T}, to shared memory (FP32)
//   phase 2  (128 threads) operands written in the canonical no-swizzle
//            K-major layout (8-row x 16-byte core matrices), geometric
//            stiffness per node pair; fence.proxy.async
//   phase 3  thread 0 issues the MMAs (tcgen05.mma.cta_group::1 with shared
//            memory descriptors) and commits to an mbarrier; all threads
//            wait (bounded)
//   phase 4  each warp reads its 32 TMEM lanes (rows) with tcgen05.ld,
//            keeps the element's upper triangle, adds the geometric part,
//            stages Ke in shared memory and stores it coalesced (FP32)
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
constexpr int kRows = 128;             // M = N
constexpr int kK = NG * 6;             // 48
constexpr int kThreads = 128;
constexpr int kTmemCols = 128;
constexpr long long kWaitLimit = 1ll << 22;   // mbarrier polls before giving up

template <bool kBF16>
struct TcLayout {
  static constexpr int kBytes = kBF16 ? 2 : 4;
  static constexpr int kPerCore = 16 / kBytes;          // K elements per core-matrix row
  static constexpr int kLBO = 128;                      // next core matrix along K
  static constexpr int kSBO = (kK / kPerCore) * 128;    // next 8-row group
  static constexpr int kOpBytes = kRows * kK * kBytes;  // one operand
  static constexpr int kKStep = kBF16 ? 16 : 8;         // K per MMA
  static constexpr int kSteps = kK / kKStep;
  __device__ static __forceinline__ int offset(int r, int k) {
    return (r >> 3) * kSBO + (k / kPerCore) * kLBO + (r & 7) * 16 + (k % kPerCore) * kBytes;
  }
};

struct TcStatic {
  float dn[NG * 3 * NN + NG];
  float x[kTcElems][3 * NN];
  float g[kTcElems][NG][3 * NN];
  float D[kTcElems][NG][21];
  float T[kTcElems][NG][6];
  float kg[kTcElems][36];
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

// Operands are rounded to the input format to nearest (the tensor core
// would otherwise drop the low mantissa bits of an FP32 operand). With
// kSplit, v = hi + lo with both parts in the input format, and the product
// of two split operands is taken as hi*hi + hi*lo + lo*hi (the lo*lo term is
// below FP32 rounding for TF32): three MMAs instead of one, and an error
// near FP32's for TF32 (about 2^-16 relative for BF16).
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

template <bool kBF16>
__device__ __forceinline__ float round_in(float v) {
  if (kBF16) return __bfloat162float(__float2bfloat16_rn(v));
  uint32_t t;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v));
  return __uint_as_float(t);
}

template <bool kBF16, bool kSplit>
__device__ __forceinline__ void put(unsigned char* op, int r, int k, float v) {
  const int o = TcLayout<kBF16>::offset(r, k);
  const float hi = round_in<kBF16>(v);
  if (kBF16) *reinterpret_cast<__nv_bfloat16*>(op + o) = __float2bfloat16_rn(hi);
  else *reinterpret_cast<float*>(op + o) = hi;
  if (kSplit) {
    unsigned char* lo_op = op + 2 * TcLayout<kBF16>::kOpBytes;   // A_lo after B_hi, B_lo after A_lo
    const float lo = round_in<kBF16>(v - hi);
    if (kBF16) *reinterpret_cast<__nv_bfloat16*>(lo_op + o) = __float2bfloat16_rn(lo);
    else *reinterpret_cast<float*>(lo_op + o) = lo;
  }
}

template <bool kBF16, bool kSplit>
__global__ void __launch_bounds__(kThreads) k_tangent_tc_hex8(TangentArgs a, int chunk0, int* tc_timeout) {
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
  for (int k = tid; k < NG * 3 * NN + NG; k += kThreads) S.dn[k] = (float)a.dn[0][k];
  // ---- gather: x(n+1) relative to node 1 of each element ----
  for (int idx = tid; idx < kTcElems * NN; idx += kThreads) {
    const int e = idx / NN, node = idx % NN;
    if (e < ch.n) {
      const long long dbase = bd.einf_off + (long long)(ch.i0 + e) * TOT;
      for (int d = 0; d < 3; ++d) {
        double ref = a.c[a.cdest[dbase + d * NN] - 1];
        double v = a.c[a.cdest[dbase + d * NN + node] - 1];
        if (bd.geonl) {
          const int e0 = a.edest[dbase + d * NN] - 1, e1 = a.edest[dbase + d * NN + node] - 1;
          ref = ref + a.u[e0] + a.du[e0];
          v = v + a.u[e1] + a.du[e1];
        }
        S.x[e][d * NN + node] = (float)(v - ref);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = S.tmem_base;

  // ---- phase 1: one (element, Gauss point) per thread ----
  if (tid < kTcElems * NG) {
    const int e = tid / NG, gp = tid % NG;
    if (e < ch.n) {
      const int i = ch.i0 + e;
      const float* dnx = S.dn + (gp * 3 + 0) * NN;
      const float* dne = S.dn + (gp * 3 + 1) * NN;
      const float* dnz = S.dn + (gp * 3 + 2) * NN;
      const float w = S.dn[NG * 3 * NN + gp];
      float gama[9], dj;
      jacobian_inverse<NN, float>(dnx, dne, dnz, S.x[e], S.x[e] + NN, S.x[e] + 2 * NN, gama, dj);
      float* g = S.g[e][gp];
      for (int n = 0; n < NN; ++n)
        shape_gradient<float>(gama, dnx[n], dne[n], dnz[n], g[3 * n], g[3 * n + 1], g[3 * n + 2]);
      const float f = w * dj;
      float C[21];
      load_D21<float, NG>(a, bd, i, gp, f, C);
      float* D = S.D[e][gp];
      float* Tw = S.T[e][gp];
      if (bd.geonl) {
        const long long gpi = bd.gp_off + (long long)i * NG + gp;
        float R[9], q[36], ur[6], cs[6];
        for (int k = 0; k < 9; ++k) R[k] = (float)a.rot_n1[gpi * 9 + k];
        for (int k = 0; k < 6; ++k) ur[k] = (float)a.urcs_n1[gpi * 9 + k];
        rotation_q2<float>(R, q);
        qmply<float>(q, ur, cs);
        for (int j = 0; j < 6; ++j) {
          float tc[6];
          for (int kk = 0; kk < 6; ++kk) {
            float s = 0.f;
            for (int m = 0; m < 6; ++m) s += q[6 * j + m] * C[low(m, kk)];
            tc[kk] = s;
          }
          for (int kk = 0; kk <= j; ++kk) {
            float s = 0.f;
            for (int m = 0; m < 6; ++m) s += tc[m] * q[6 * kk + m];
            D[low(j, kk)] = s;
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
        for (int k = 0; k < 6; ++k) Tw[k] = cs[k] * f;
      } else {
        for (int k = 0; k < 21; ++k) D[k] = C[k];
        for (int k = 0; k < 6; ++k) Tw[k] = 0.f;
      }
    }
  }
  __syncthreads();

  // ---- phase 2: operands (row = 24 e + dof, dof = 8 i + a; k = 6 gp + m) ----
  for (int idx = tid; idx < kRows * kK; idx += kThreads) {
    const int r = idx / kK, k = idx % kK;
    const int e = r / TOT;
    float va = 0.f, vb = 0.f;
    if (r < kTcElems * TOT && e < ch.n) {
      const int d = r % TOT, di = d / NN, na = d % NN;
      const int gp = k / 6, m = k % 6;
      const float* g = S.g[e][gp];
      const float gx = g[3 * na], gy = g[3 * na + 1], gz = g[3 * na + 2];
      const float* D = S.D[e][gp];
      if (di == 0) {
        va = m == 0 ? gx : m == 3 ? gy : m == 5 ? gz : 0.f;
        vb = D[low(m, 0)] * gx + D[low(m, 3)] * gy + D[low(m, 5)] * gz;
      } else if (di == 1) {
        va = m == 1 ? gy : m == 3 ? gx : m == 4 ? gz : 0.f;
        vb = D[low(m, 1)] * gy + D[low(m, 3)] * gx + D[low(m, 4)] * gz;
      } else {
        va = m == 2 ? gz : m == 4 ? gy : m == 5 ? gx : 0.f;
        vb = D[low(m, 2)] * gz + D[low(m, 4)] * gy + D[low(m, 5)] * gx;
      }
    }
    put<kBF16, kSplit>(opA, r, k, va);
    put<kBF16, kSplit>(opB, r, k, vb);
  }
  // geometric stiffness per node pair (kgstiff): sum_gp g_a . ({T} g_b)
  for (int idx = tid; idx < kTcElems * 36; idx += kThreads) {
    const int e = idx / 36, p = idx % 36;
    int na = 0, r = p;
    while (r >= NN - na) { r -= NN - na; ++na; }
    const int nb = na + r;
    float s = 0.f;
    if (e < ch.n && bd.geonl)
      for (int gp = 0; gp < NG; ++gp) {
        const float* g = S.g[e][gp];
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
  if (tid == 0) {
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
  // bounded wait on phase 0 of the mbarrier
  {
    uint32_t done = 0;
    long long polls = 0;
    while (!done && polls < kWaitLimit) {
      asm volatile(
          "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\nselp.u32 %0, 1, 0, p;\n}"
          : "=r"(done)
          : "r"(smem_u32(&S.mbar)));
      ++polls;
    }
    if (!done) S.timeout = 1;
  }
  asm volatile("tcgen05.fence::after_thread_sync;");
  __syncthreads();
  const bool ok = S.timeout == 0;

  // ---- phase 4: TMEM -> upper triangles (+ geometric part) -> Ke ----
  float* ke = reinterpret_cast<float*>(opA);   // operands are consumed
  const int r = 32 * warp + lane;
  const int e = r / TOT, dr = r % TOT, ir = dr / NN, ar = dr % NN;
  const float bf = (float)a.beta_fact;
#pragma unroll
  for (int pass = 0; pass < kRows / 32; ++pass) {
    uint32_t v[32];
    const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(32 * pass);
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
    if (r < kTcElems * TOT && e < ch.n) {
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int col = 32 * pass + j;
        const int dc = col - TOT * e;
        if (dc >= dr && dc < TOT) {
          const int ic = dc / NN, ac = dc % NN;
          float val = __uint_as_float(v[j]);
          if (ic == ir) {
            const int lo = ar < ac ? ar : ac, hi = ar < ac ? ac : ar;
            val += S.kg[e][lo * NN - lo * (lo - 1) / 2 + (hi - lo)];
          }
          ke[e * UT + dc * (dc + 1) / 2 + dr] = ok ? val * bf : __int_as_float(0x7fc00000);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
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

// Dynamic shared memory per CTA: A and B (and their low parts when split).
// At least 40 KB, so that no more than four CTAs share an SM and their
// 4 x 128 TMEM columns always fit in the SM's 512: tcgen05.alloc then never
// has to wait for another CTA's columns.
template <bool kBF16, bool kSplit>
size_t tc_smem() {
  const size_t need = (kSplit ? 4 : 2) * (size_t)TcLayout<kBF16>::kOpBytes;
  return need > 40 * 1024 ? need : 40 * 1024;
}

template <bool kBF16, bool kSplit>
cudaError_t set_smem() {
  return cudaFuncSetAttribute(k_tangent_tc_hex8<kBF16, kSplit>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)tc_smem<kBF16, kSplit>());
}

template <bool kBF16, bool kSplit>
void launch(const DeviceModel& m, const TangentArgs& h, int* tc_timeout, cudaStream_t s) {
  k_tangent_tc_hex8<kBF16, kSplit><<<m.ntcchunks, kThreads, tc_smem<kBF16, kSplit>(), s>>>(h, 0, tc_timeout);
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
