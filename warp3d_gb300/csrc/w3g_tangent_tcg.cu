// w3g_tangent_tcg.cu -- precision forms of the 8-node brick tangent on the
// fifth-generation tensor cores as ONE GEMM over all elements: the
// gradient-pair form.
//
// WARP3D's material and geometric stiffness (gptns1.f bdbtgen :1628,
// kg1.f :16) of an element is
//   Ke[(i,a),(j,b)] = sum_gp  g_a^T X^ij g_b,
//   X^ij[p][q] = [D*](v(i,p), v(j,q)) + delta_ij {T}[p][q]
// for dof (i,a) = displacement component i of node a, spatial gradients
// g_a = Gamma n_a (Gamma = J^-1, n_a = dN_a/dxi at the Gauss point) and
// v(i,p) the Voigt index of the strain pair (i,p) (xx yy zz xy yz xz, the
// engineering shears of blcmp1). Moving Gamma to the material side,
//   Ke[(i,a),(j,b)] = sum_{gp,r,s}  n_a[r] n_b[s]  H^ij_gp[r][s],
//   H^ij = Gamma^T X^ij Gamma   (3 x 3 per Gauss point and pair i <= j),
// where n_a[r] n_b[s] depends only on the element type and Gauss point:
// the contraction is a product of a CONSTANT operator M (node pair (a,b) x
// (r, s, gp), 64 x 72) with a per-element vector H (72 values per pair
// (i,j)): Ke of every element of the model is one GEMM
//   D[(e, ij), (a, b)] = sum_k H[(e, ij), k] M[(a, b), k],   K = 72,
// run here as M = 128 rows (8 row slots x 16 elements, row = slot*16 +
// element, 6 slots used), N = 64, on tcgen05.mma with an FP32 accumulator
// in tensor memory.
//
// Why this form: the per-element CUDA-core work shrinks to the Gauss-point
// quantities ([D*] = [q][D][q]^T - Q-bar, Gamma, {T}, H: ~600 FP32 FMA per
// point instead of the ~2,700 of B^T[D*]B + G^T T G), and the tensor core
// does the node-pair contraction at full tile utilisation. Rounding M to
// TF32 or BF16 keeps Ke's rigid-translation null space EXACTLY: for the
// trilinear brick dN_b/dxi_s at a Gauss point changes sign, and only sign,
// between the two nodes mirrored in xi_s, and round-to-nearest is odd, so
// every column sum over b of the rounded M is exactly zero. Rounding H only
// perturbs the material point values, which keeps that property too; what
// remains is the FP32 accumulation (as in the FP32 CUDA-core kernel), so
// no projection onto the translation-free matrices is needed.
//
// The kernel is persistent (one CTA per SM) and pipelined:
//   warp 8 (producer)  per tile, into a ring of shared-memory stages:
//                      1-D bulk copies (cp.async.bulk, completion counted
//                      in bytes on the stage's mbarrier) of the tile's
//                      contiguous slabs -- cep (21, span, ngp) for each of
//                      the 8 Gauss points, rot_n1 and urcs_n1 (9, ngp,
//                      span) -- and 8-byte cp.async gathers of the nodal
//                      coordinates, u and du through cdest/edest, which
//                      arrive on the same mbarrier
//   warps 0-7          per tile: two threads per (element, Gauss point)
//   (consumers)        form Gamma, [D*], {T} and H^ij (three pairs each)
//                      into the A operand (K-major, no swizzle); thread 0
//                      issues the MMA chain (M is built once per CTA as
//                      the B operand); the accumulator is read with
//                      tcgen05.ld, each element's packed upper triangle
//                      (utsz, span layout, setup.f:265-275) is staged in
//                      shared memory and written with one bulk copy to
//                      global memory (cp.async.bulk.global.shared::cta)
// Every wait is bounded (TangentArgs::wait_limit polls). A wait that gives
// up sets the CTA's abort flag: no further MMA is issued, the copies still
// in flight are waited for (again bounded), the tiles not finished get NaN
// Ke, the tensor memory is freed and the host sees W3G_EFATAL. A wait
// limit of 0 makes the first wait (for the first tile's copies, before any
// MMA) give up at once: the status path without a GPU fault.
#include <cstdint>
#include <cuda_bf16.h>
#include "w3g_internal.cuh"
#include "w3g_elem.cuh"
#include "w3g_math.cuh"

namespace w3g {

namespace {

constexpr int NN = Hex8::NN, NG = Hex8::NG, TOT = Hex8::TOTDOF, UT = Hex8::UTSZ;
constexpr int kTile = 16;                    // elements per tile
constexpr int kSlots = 8;                    // A rows per element (6 pairs i <= j used)
constexpr int kM = kTile * kSlots;           // 128
constexpr int kN = NN * NN;                  // 64 node pairs (a, b)
constexpr int kKLive = 9 * NG;               // 72 = (r, s, gp)
constexpr int kParts = 2;                    // threads per (element, Gauss point)
constexpr int kConsumers = 128 * kParts;     // warps 0-7
constexpr int kThreads = kConsumers + 32;    // + producer warp 8
constexpr int kTmemCols = 64;
constexpr long long kDrainLimit = 1ll << 26; // polls when waiting out copies / MMAs after an abort

// stage layout (bytes): cep slabs of the 8 Gauss points, rot_n1, urcs_n1
// (each copied from a 16-byte-aligned start, so up to 8 leading bytes are
// not the tile's), then the gathered nodal values
constexpr int kCepSlab = kTile * 21 * 8 + 16;     // 2704
constexpr int kGpSlab = kTile * NG * 9 * 8 + 16;  // 9232
constexpr int kStCep = 0;
constexpr int kStRot = kStCep + NG * kCepSlab;
constexpr int kStUrcs = kStRot + kGpSlab;
constexpr int kStXc = kStUrcs + kGpSlab;
constexpr int kStXu = kStXc + kTile * TOT * 8;
constexpr int kStXdu = kStXu + kTile * TOT * 8;
constexpr int kStage = kStXdu + kTile * TOT * 8;  // 49312
static_assert(kStage % 128 == 0 || kStage % 16 == 0, "stage alignment");

template <bool kBF16, bool kSplit>
struct Form {
  static constexpr int kBytes = kBF16 ? 2 : 4;
  static constexpr int kPerCore = 16 / kBytes;                   // K values per core-matrix row
  static constexpr int kK = kBF16 ? 80 : 72;                      // K padded to the MMA step
  static constexpr int kChunks = kK / kPerCore;
  static constexpr int kSBO = kChunks * 128;                      // next 8-row group
  static constexpr int kKStep = kBF16 ? 16 : 8;
  static constexpr int kSteps = kK / kKStep;
  static constexpr int kOpA = kM * kK * kBytes;                   // one A operand
  static constexpr int kOpB = kN * kK * kBytes;                   // one B operand
  static constexpr int kStages = (kSplit && !kBF16) ? 2 : 3;
  static constexpr int kOffB = 0;
  static constexpr int kOffA = kOffB + (kSplit ? 2 : 1) * kOpB;
  static constexpr int kOffStage = kOffA + (kSplit ? 2 : 1) * kOpA;
  static constexpr int kSmem = kOffStage + kStages * kStage;
  // byte offset of (row, k) in a K-major no-swizzle operand
  __device__ static __forceinline__ int off(int row, int k) {
    return (row >> 3) * kSBO + (k / kPerCore) * 128 + (row & 7) * 16 + (k % kPerCore) * kBytes;
  }
};
static_assert(kTile * UT * 4 <= Form<true, false>::kOpA, "Ke staging must fit in the A operand");

struct TcgStatic {
  float dn[NG * 3 * NN + NG];          // dN/dxi per Gauss point (float) + weights
  float x[kTile][TOT + 1];             // x(n+1) relative to node 1 of each element (rows padded: banks)
  float dx[kTile * NG][21];            // [D*] lower triangle per (element, Gauss point): the two halves' rows
  TcgTile hdr[3];                      // the tile in each stage, written by the producer before its arrival
  unsigned long long full[3], empty[3], mma;
  uint32_t tmem_base;
  // a bounded wait gave up: the producer's flag is written by the producer
  // only, the consumers' only by consumers before a named barrier, so that
  // every consumer takes the same branch after that barrier
  int pabort, cabort;
  int issued;                          // tiles whose copies the producer issued
  int done;                            // tiles the consumers finished (Ke stored)
};

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t sdesc(uint32_t addr, int sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((128 >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor: FP32 accumulator, A/B K-major, M = 128, N = 64
template <bool kBF16>
__host__ __device__ constexpr uint32_t idesc() {
  return (1u << 4) | ((kBF16 ? 1u : 2u) << 7) | ((kBF16 ? 1u : 2u) << 10) | ((uint32_t)(kN >> 3) << 17) |
         ((uint32_t)(kM >> 4) << 24);
}

template <bool kBF16>
__device__ __forceinline__ void mma(uint32_t tmem, uint64_t da, uint64_t db, bool acc) {
  const uint32_t id = idesc<kBF16>(), a = acc ? 1u : 0u;
  if (kBF16)
    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                 ::"r"(tmem), "l"(da), "l"(db), "r"(id), "r"(a));
  else
    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}"
                 ::"r"(tmem), "l"(da), "l"(db), "r"(id), "r"(a));
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

template <bool kBF16>
__device__ __forceinline__ void put(unsigned char* op, int o, float v) {
  if (kBF16) *reinterpret_cast<__nv_bfloat16*>(op + o) = __float2bfloat16_rn(v);
  else {
    uint32_t t;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v));
    *reinterpret_cast<uint32_t*>(op + o) = t;
  }
}

template <bool kBF16>
__device__ __forceinline__ float round_in(float v) {
  if (kBF16) return __bfloat162float(__float2bfloat16_rn(v));
  uint32_t t;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v));
  return __uint_as_float(t);
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

// rows of [D*] formed by part H of a Gauss point's two threads: {0, 3, 5}
// and {1, 2, 4} (11 and 10 lower-triangle entries)
__host__ __device__ constexpr int row_of_part(int h, int jj) {
  return h == 0 ? (jj == 0 ? 0 : jj == 1 ? 3 : 5) : (jj == 0 ? 1 : jj == 1 ? 2 : 4);
}

// One part (H = 0, 1) of the Gauss-point work of (element pe, point pg)
// of a tile: Gamma, w det[J], the three rows of [D*] = [q][D][q]^T - Q-bar
// this part owns (row_of_part; the other rows come from the other part
// through shared memory), {T}, and H^ij = Gamma^T X^ij Gamma for the
// part's three pairs (slots 3H .. 3H + 2 of 00 01 02 11 12 22), written
// into the A operand. Both parts reach the same named barrier (the
// exchange) whether their element is live or not.
template <bool kBF16, bool kSplit, int H>
__device__ __forceinline__ void point_h(const TangentArgs& a, const TcgTile& tl, const unsigned char* st,
                                        TcgStatic& T, int pe, int pg, bool live, unsigned char* opA) {
  using F = Form<kBF16, kSplit>;
  const int item = pe * NG + pg;
  float gam[9], f = 0.f, Tw[6];
  if (live) {
    const int i = tl.i0 + pe;
    const float* dnx = T.dn + (pg * 3 + 0) * NN;
    const float* dne = T.dn + (pg * 3 + 1) * NN;
    const float* dnz = T.dn + (pg * 3 + 2) * NN;
    const float w = T.dn[NG * 3 * NN + pg];
    float dj;
    jacobian_inverse<NN, float>(dnx, dne, dnz, T.x[pe], T.x[pe] + NN, T.x[pe] + 2 * NN, gam, dj);
    f = w * dj;
    // w det[J] [D], lower triangle row-wise (cep, or mm10 history1(1:36))
    float C[21];
    if (tl.flags & 2) {
      const double* Hh = a.hist1 + tl.hist_off + ((long long)i * NG + pg) * kHistMM10;
#pragma unroll
      for (int r = 0, q = 0; r < 6; ++r)
#pragma unroll
        for (int c = 0; c <= r; ++c, ++q) C[q] = f * (float)Hh[r + 6 * c];
    } else {
      const double* cp = reinterpret_cast<const double*>(
          st + kStCep + pg * kCepSlab + pad_of(a.cep + tl.cep_off + ((long long)pg * tl.span + tl.i0) * 21));
#pragma unroll
      for (int q = 0; q < 21; ++q) C[q] = f * (float)cp[pe * 21 + q];
    }
    if (tl.flags & 1) {
      const long long g0 = (tl.gp_off + (long long)tl.i0 * NG) * 9;
      const double* rp = reinterpret_cast<const double*>(st + kStRot + pad_of(a.rot_n1 + g0)) + (pe * NG + pg) * 9;
      const double* up = reinterpret_cast<const double*>(st + kStUrcs + pad_of(a.urcs_n1 + g0)) + (pe * NG + pg) * 9;
      float R[9], q[36], cs[6];
#pragma unroll
      for (int m = 0; m < 9; ++m) R[m] = (float)rp[m];
#pragma unroll
      for (int r = 0; r < 6; ++r) q_row(R, r, q + 6 * r);
#pragma unroll
      for (int r = 0; r < 6; ++r) {
        float v = 0.f;
#pragma unroll
        for (int m = 0; m < 6; ++m) v += q[6 * r + m] * (float)up[m];
        cs[r] = v;                                   // Cauchy stress at n+1
      }
#pragma unroll
      for (int jj = 0; jj < 3; ++jj) {
        const int j = row_of_part(H, jj);
        float tc[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) {
          float v = 0.f;
#pragma unroll
          for (int m = 0; m < 6; ++m) v += q[6 * j + m] * C[lw(m, c)];
          tc[c] = v;
        }
#pragma unroll
        for (int c = 0; c <= j; ++c) {
          float v = 0.f;
#pragma unroll
          for (int m = 0; m < 6; ++m) v += tc[m] * q[6 * c + m];
          if (a.qbar) {   // Q-bar terms of row j (ctran1 with qbar)
            const float xx = cs[0], yy = cs[1], zz = cs[2], xy = cs[3], yz = cs[4], xz = cs[5];
            const float hw = 0.5f * f;
            if (j == 0 && c == 0) v -= 2.f * xx * f;
            if (j == 1 && c == 1) v -= 2.f * yy * f;
            if (j == 2 && c == 2) v -= 2.f * zz * f;
            if (j == 3 && (c == 0 || c == 1)) v -= xy * f;
            if (j == 3 && c == 3) v -= hw * (xx + yy);
            if (j == 4 && (c == 1 || c == 2)) v -= yz * f;
            if (j == 4 && c == 3) v -= f * xz;
            if (j == 4 && c == 4) v -= hw * (yy + zz);
            if (j == 5 && (c == 0 || c == 2)) v -= xz * f;
            if (j == 5 && c == 3) v -= f * yz;
            if (j == 5 && c == 4) v -= f * xy;
            if (j == 5 && c == 5) v -= hw * (xx + zz);
          }
          T.dx[item][lw(j, c)] = v;
        }
      }
#pragma unroll
      for (int m = 0; m < 6; ++m) Tw[m] = cs[m] * f;
    } else {
#pragma unroll
      for (int jj = 0; jj < 3; ++jj) {
        const int j = row_of_part(H, jj);
#pragma unroll
        for (int c = 0; c <= j; ++c) T.dx[item][lw(j, c)] = C[lw(j, c)];
      }
#pragma unroll
      for (int m = 0; m < 6; ++m) Tw[m] = 0.f;
    }
  }
  asm volatile("bar.sync 1, %0;" ::"n"(kConsumers) : "memory");   // both parts' rows of [D*] in T.dx
  if (!live) return;
  float Dl[21];
#pragma unroll
  for (int z = 0; z < 21; ++z) Dl[z] = T.dx[item][z];
#pragma unroll
  for (int pp = 0; pp < 3; ++pp) {
    const int slot = 3 * H + pp;            // pairs 00 01 02 11 12 22
    const int ii = slot < 3 ? 0 : (slot < 5 ? 1 : 2);
    const int jj = slot < 3 ? slot : (slot == 3 ? 1 : 2);
    float X[3][3];
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        float v = Dl[lw(voigt(ii, p), voigt(jj, q))];
        if (ii == jj) v += Tw[voigt(p, q)];
        X[p][q] = v;
      }
    float Y[3][3];
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int s2 = 0; s2 < 3; ++s2)
        Y[p][s2] = X[p][0] * gam[3 * s2] + X[p][1] * gam[3 * s2 + 1] + X[p][2] * gam[3 * s2 + 2];
    // A operand row (slot, element pe), k = (r*3 + s)*8 + gp
    const int row = slot * kTile + pe;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int s2 = 0; s2 < 3; ++s2)
        put_split<kBF16, kSplit>(opA, F::kOpA, F::off(row, (3 * r + s2) * 8 + pg),
                                 gam[3 * r] * Y[0][s2] + gam[3 * r + 1] * Y[1][s2] + gam[3 * r + 2] * Y[2][s2]);
  }
}

template <bool kBF16, bool kSplit>
__global__ void __launch_bounds__(kThreads, 1) k_tangent_tcg_hex8(TangentArgs a, const TcgTile* tiles, int ntiles,
                                                                   int* tc_timeout) {
  using F = Form<kBF16, kSplit>;
  constexpr int S = F::kStages;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* opB = smem + F::kOffB;
  unsigned char* opA = smem + F::kOffA;
  unsigned char* stages = smem + F::kOffStage;
  __shared__ TcgStatic T;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long limit = a.wait_limit;
  volatile int* pabort = &T.pabort;
  volatile int* cabort = &T.cabort;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&T.tmem_base)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(&T.full[s])), "r"(33));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(&T.empty[s])), "r"(1));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(&T.mma)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;");
    T.pabort = 0;
    T.cabort = 0;
    T.issued = 0;
    T.done = 0;
  }
  for (int k = tid; k < NG * 3 * NN + NG; k += kThreads) T.dn[k] = a.dn32[0][k];
  // the constant operator M (B operand): row a*8 + b, k = (r*3 + s)*8 + gp,
  // products formed in double and rounded once (split: hi + lo)
  for (int idx = tid; idx < kN * F::kK; idx += kThreads) {
    const int row = idx / F::kK, k = idx % F::kK;
    float v = 0.f;
    if (k < kKLive) {
      const int ab = row, rs = k >> 3, gp = k & 7;
      const int an = ab >> 3, bn = ab & 7, r = rs / 3, s = rs % 3;
      const double* dn = a.dn[0];
      v = (float)(dn[(gp * 3 + r) * NN + an] * dn[(gp * 3 + s) * NN + bn]);
    }
    put_split<kBF16, kSplit>(opB, F::kOpB, F::off(row, k), v);
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = T.tmem_base;

  if (warp == kConsumers / 32) {
    // ================= producer =================
    constexpr int kPerLane = kTile * TOT / 32;   // 12 gathered dofs per lane and tile
    TcgTile nxt = tiles[blockIdx.x];
    int k = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++k) {
      const TcgTile tl = nxt;
      if (t + (int)gridDim.x < ntiles) nxt = tiles[t + gridDim.x];   // next tile's record, in flight meanwhile
      // this tile's dof indices, all loads issued before the first copy
      const long long dbase = tl.einf_off + (long long)tl.i0 * TOT;
      const int nv = tl.n * TOT;
      const bool geonl = tl.flags & 1;
      int ci[kPerLane], ei[kPerLane];
#pragma unroll
      for (int j = 0; j < kPerLane; ++j) {
        const int q = lane + 32 * j;
        ci[j] = q < nv ? a.cdest[dbase + q] - 1 : 0;
        ei[j] = q < nv && geonl ? a.edest[dbase + q] - 1 : 0;
      }
      const int s = k % S, use = k / S;
      if (use > 0 && !wait_phase(&T.empty[s], (use - 1) & 1, limit, cabort)) {
        if (lane == 0) *pabort = 1;
        break;
      }
      if (*cabort) break;
      unsigned char* st = stages + s * kStage;
      const uint32_t bar = su32(&T.full[s]);
      if (lane == 0) {
        T.hdr[s] = tl;   // published by the arrival below (release)
        uint32_t tx = 0;
        // byte total first (expect_tx must not trail the copies' completion)
        for (int pass = 0; pass < 2; ++pass) {
          if (pass == 1)
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(tx) : "memory");
          uint32_t txc = 0;
          auto range = [&](const double* src, long long n, uint32_t dst) {
            const uintptr_t p = (uintptr_t)src, p16 = p & ~(uintptr_t)15;
            const uint32_t bytes = (uint32_t)(((p - p16) + n * 8 + 15) & ~15ull);
            if (pass == 1) bulk_g2s(dst, (const void*)p16, bytes, bar);
            txc += bytes;
          };
          if (!(tl.flags & 2))
            for (int gp = 0; gp < NG; ++gp)
              range(a.cep + tl.cep_off + ((long long)gp * tl.span + tl.i0) * 21, (long long)tl.n * 21,
                    su32(st + kStCep + gp * kCepSlab));
          if (geonl) {
            const long long g0 = (tl.gp_off + (long long)tl.i0 * NG) * 9;
            range(a.rot_n1 + g0, (long long)tl.n * NG * 9, su32(st + kStRot));
            range(a.urcs_n1 + g0, (long long)tl.n * NG * 9, su32(st + kStUrcs));
          }
          tx = txc;
        }
      }
      // gathers of the nodal values (u and du only for finite strain)
      double* xc = reinterpret_cast<double*>(st + kStXc);
      double* xu = reinterpret_cast<double*>(st + kStXu);
      double* xdu = reinterpret_cast<double*>(st + kStXdu);
#pragma unroll
      for (int j = 0; j < kPerLane; ++j) {
        const int q = lane + 32 * j;
        if (q < nv) {
          asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(su32(xc + q)), "l"(a.c + ci[j]) : "memory");
          if (geonl) {
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(su32(xu + q)), "l"(a.u + ei[j]) : "memory");
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(su32(xdu + q)), "l"(a.du + ei[j]) : "memory");
          }
        }
      }
      asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(bar) : "memory");
      if (lane == 0) T.issued = k + 1;
    }
  } else {
    // ================= consumers =================
    // warps 0-3 and 4-7 take the two parts of every (element, Gauss
    // point): the part is uniform over a warp. A warp holds 8 elements x 4
    // Gauss points, lane = element (low 3 bits) + 8 x point, so that its
    // stores into an A row slot (rows slot*16 + element) fall in 32
    // distinct banks
    const int h = warp >> 2;
    const int pe = (lane & 7) + 8 * (warp & 1), pg = (lane >> 3) + 4 * ((warp >> 1) & 1);
    int k = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++k) {
      const int s = k % S;
      const unsigned char* st = stages + s * kStage;
      if (!wait_phase(&T.full[s], (k / S) & 1, limit, pabort)) *cabort = 1;
      // previous tile's Ke store must have read the staging (A region)
      if (tid == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
      asm volatile("bar.sync 1, %0;" ::"n"(kConsumers) : "memory");
      if (*cabort) break;
      // the tile record, read from shared memory where needed; what the
      // epilogue needs is copied before the stage (and record) is released
      const TcgTile& tl = T.hdr[s];
      const int tn = tl.n;
      float* const out = reinterpret_cast<float*>(a.estiff) + tl.estiff_off + (long long)tl.i0 * UT;
      // element coordinates at n+1 relative to node 1
      for (int q = tid; q < tl.n * TOT; q += kConsumers) {
        const int e = q / TOT, d = q % TOT, q0 = e * TOT + (d / NN) * NN;
        const double* xc = reinterpret_cast<const double*>(st + kStXc);
        double v = xc[q], ref = xc[q0];
        if (tl.flags & 1) {
          const double* xu = reinterpret_cast<const double*>(st + kStXu);
          const double* xdu = reinterpret_cast<const double*>(st + kStXdu);
          v = v + xu[q] + xdu[q];
          ref = ref + xu[q0] + xdu[q0];
        }
        T.x[e][d] = (float)(v - ref);
      }
      asm volatile("bar.sync 1, %0;" ::"n"(kConsumers) : "memory");
      // the Gauss-point work, written into the A operand (the previous
      // tile's MMAs are complete and its Ke store has read the region)
      const bool live = pe < tl.n;
      if (h == 0) point_h<kBF16, kSplit, 0>(a, tl, st, T, pe, pg, live, opA);
      else point_h<kBF16, kSplit, 1>(a, tl, st, T, pe, pg, live, opA);
      if (kBF16) {   // the K padding (72..79) must be finite zeros: the staging reuses the region
        for (int row = tid; row < kM; row += kConsumers)
          for (int kk = kKLive; kk < F::kK; ++kk) {
            put<kBF16>(opA, F::off(row, kk), 0.f);
            if (kSplit) put<kBF16>(opA + F::kOpA, F::off(row, kk), 0.f);
          }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("bar.sync 1, %0;" ::"n"(kConsumers) : "memory");
      if (tid == 0) {
        // stage consumed: hand it back to the producer
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(&T.empty[s])) : "memory");
        asm volatile("tcgen05.fence::after_thread_sync;");
        // descriptors advanced in the start-address field (16-byte units):
        // one k-step = two core matrices along K = 256 bytes
        const uint64_t da = sdesc(su32(opA), F::kSBO), db = sdesc(su32(opB), F::kSBO);
#pragma unroll 1
        for (int ks = 0; ks < F::kSteps; ++ks) {
          const uint64_t o = (uint64_t)ks * (256 >> 4);
          mma<kBF16>(tmem, da + o, db + o, ks > 0);
          if (kSplit) {
            mma<kBF16>(tmem, da + o, db + o + (F::kOpB >> 4), true);
            mma<kBF16>(tmem, da + o + (F::kOpA >> 4), db + o, true);
          }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            su32(&T.mma)) : "memory");
      }
      if (!wait_phase(&T.mma, k & 1, limit, nullptr)) {
        // the MMAs may still be running: wait them out before tensor
        // memory is read or freed
        *cabort = 1;
        wait_phase(&T.mma, k & 1, kDrainLimit, nullptr);
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      asm volatile("bar.sync 1, %0;" ::"n"(kConsumers) : "memory");
      if (*cabort) break;
      // accumulator -> packed Ke in the staging (the A region: the MMAs are done)
      {
        float* ke = reinterpret_cast<float*>(opA);
        // warp w: lane quadrant w % 4, columns 32 * (w / 4) .. + 31
        const bool ld_warp = warp < 8;
        const int quad = warp & 3, half = (warp >> 2) & 1;
        const int row = 32 * quad + lane, e = row & (kTile - 1), slot = row >> 4;
        const uint32_t taddr = tmem + ((uint32_t)(32 * quad) << 16) + (uint32_t)(32 * half);
        if (ld_warp) {
          const int ii = slot < 3 ? 0 : (slot < 5 ? 1 : 2);
          const int jj = slot < 3 ? slot : (slot == 3 ? 1 : 2);
          const bool keep = slot < 6 && e < tn;
          const float bf = (float)a.beta_fact;
#pragma unroll
          for (int p16 = 0; p16 < 2; ++p16) {
            uint32_t v[16];   // the load and its wait in one statement
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                "tcgen05.wait::ld.sync.aligned;"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15])
                : "r"(taddr + 16 * p16)
                : "memory");
            // the MMAs are complete: the staging may overwrite the A operand
            if (keep) {
#pragma unroll
              for (int c = 0; c < 16; ++c) {
                const int ab = 32 * half + 16 * p16 + c, an = ab >> 3, bn = ab & 7;
                if (ii == jj && an > bn) continue;
                const int d1 = ii * NN + an, d2 = jj * NN + bn;
                ke[e * UT + d2 * (d2 + 1) / 2 + d1] = __uint_as_float(v[c]) * bf;
              }
            }
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("bar.sync 1, %0;" ::"n"(kConsumers) : "memory");
      {
        const uint32_t bytes = (uint32_t)tn * UT * 4;
        if (((uintptr_t)out & 15) == 0) {
          if (tid == 0) {
            asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(out), "r"(su32(opA)),
                         "r"(bytes) : "memory");
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
          }
        } else {   // block offset not 16-byte aligned (after a block of another element type)
          const float* ke = reinterpret_cast<const float*>(opA);
          for (int q = tid; q < tn * UT; q += kConsumers) out[q] = ke[q];
          asm volatile("bar.sync 1, %0;" ::"n"(kConsumers) : "memory");
        }
      }
      if (tid == 0) T.done = k + 1;
    }
    if (tid == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
  }
  __syncthreads();
  if (T.pabort || T.cabort) {
    // wait out the copies the producer issued for tiles the consumers did
    // not take, then NaN for every tile of this CTA not finished
    if (tid == 0) {
      for (int q = T.done; q < T.issued; ++q) wait_phase(&T.full[q % S], (q / S) & 1, kDrainLimit, nullptr);
      atomicExch(tc_timeout, 1);
    }
    __syncthreads();
    int q = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++q) {
      if (q < T.done) continue;
      const TcgTile tl = tiles[t];
      float* out = reinterpret_cast<float*>(a.estiff) + tl.estiff_off + (long long)tl.i0 * UT;
      for (int z = tid; z < tl.n * UT; z += kThreads) out[z] = __int_as_float(0x7fc00000);
    }
  }
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
  }
}

template <bool kBF16, bool kSplit>
constexpr int smem_bytes() { return Form<kBF16, kSplit>::kSmem; }

template <bool kBF16, bool kSplit>
cudaError_t set_attr() {
  return cudaFuncSetAttribute(k_tangent_tcg_hex8<kBF16, kSplit>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              smem_bytes<kBF16, kSplit>());
}

template <bool kBF16, bool kSplit>
void launch(const DeviceModel& m, const TangentArgs& a, int* tc_timeout, cudaStream_t s) {
  const int grid = m.ntcgtiles < m.nsm ? m.ntcgtiles : m.nsm;
  k_tangent_tcg_hex8<kBF16, kSplit><<<grid, kThreads, smem_bytes<kBF16, kSplit>(), s>>>(a, m.tcgtiles, m.ntcgtiles,
                                                                                         tc_timeout);
}

static_assert(Form<false, false>::kSmem + sizeof(TcgStatic) <= 227 * 1024, "TF32 form exceeds shared memory");
static_assert(Form<false, true>::kSmem + sizeof(TcgStatic) <= 227 * 1024, "TF32x3 form exceeds shared memory");
static_assert(Form<true, false>::kSmem + sizeof(TcgStatic) <= 227 * 1024, "BF16 form exceeds shared memory");
static_assert(Form<true, true>::kSmem + sizeof(TcgStatic) <= 227 * 1024, "BF16x3 form exceeds shared memory");
static_assert(Form<false, false>::kOffStage % 16 == 0 && kStage % 16 == 0, "stages must be 16-byte aligned");

}  // namespace

cudaError_t init_tangent_tcg_kernels() {
  cudaError_t e = set_attr<false, false>();
  if (e == cudaSuccess) e = set_attr<true, false>();
  if (e == cudaSuccess) e = set_attr<false, true>();
  if (e == cudaSuccess) e = set_attr<true, true>();
  return e;
}

cudaError_t launch_tangent_tcg_hex8(const DeviceModel& m, const TangentArgs& a, bool bf16, bool split,
                                    int* tc_timeout, cudaStream_t s) {
  if (m.ntcgtiles == 0) return cudaSuccess;
  if (bf16) split ? launch<true, true>(m, a, tc_timeout, s) : launch<true, false>(m, a, tc_timeout, s);
  else split ? launch<false, true>(m, a, tc_timeout, s) : launch<false, false>(m, a, tc_timeout, s);
  return cudaGetLastError();
}

}  // namespace w3g
