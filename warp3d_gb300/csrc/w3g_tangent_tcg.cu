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
// perturbs the material point values, which keeps that property too, as
// long as the diagonal pairs' H^ii stay exactly symmetric after rounding
// (only the upper triangle of Ke is stored, the lower one is its mirror):
// they are formed for r <= s and written to both positions. The tensor
// cores' FP32 accumulation does not keep it: its error has a mean along
// the translations, the same in every element, so the epilogue projects
// the translations out of every node-pair block.
//
// The kernel is persistent (one CTA per SM) and pipelined:
//   warp 24 (producer) per tile, into a ring of shared-memory stages:
//                      1-D bulk copies (cp.async.bulk, completion counted
//                      in bytes on the stage's mbarrier) of the tile's
//                      contiguous slabs -- cep (21, span, ngp) for each of
//                      the 8 Gauss points, rot_n1 and urcs_n1 (9, ngp,
//                      span) -- and 8-byte cp.async gathers of the nodal
//                      coordinates, u and du through cdest/edest, which
//                      arrive on the same mbarrier
//   warps 0-23         per tile: six threads per (element, Gauss point),
//   (consumers)        k = 0..5, in three phases separated by CTA
//                      barriers, the point's intermediates in shared
//                      memory (one float per point and quantity, points
//                      consecutive: conflict-free): (1) k = 0 forms Gamma
//                      and w det[J]; every k converts a share of cep to
//                      float and forms row k of the strain rotation [q]
//                      and {T}_k; (2) k forms row k of [D*] = [q][D][q]^T -
//                      Q-bar (lower triangle); (3) k forms H^ij = Gamma^T
//                      X^ij Gamma of pair k (00 01 02 11 12 22) into the A
//                      operand (K-major, no swizzle); thread 0 issues the
//                      MMA chain (M is built once per CTA as the B
//                      operand); warps 0-15 read the accumulator with
//                      tcgen05.ld, project the translations out, and each
//                      element's packed upper triangle (utsz, span layout,
//                      setup.f:265-275) is staged in shared memory and
//                      written with one bulk copy to global memory
//                      (cp.async.bulk.global.shared::cta).
//                      Six short threads per point instead of two long
//                      ones: 24 warps hide the arithmetic and shared-
//                      memory latencies that 8 warps at 168 registers
//                      could not
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
#include "w3g_tc_common.cuh"

namespace w3g {

namespace {

using namespace tc;

constexpr int NN = Hex8::NN, NG = Hex8::NG, TOT = Hex8::TOTDOF, UT = Hex8::UTSZ;
constexpr int kTile = 16;                    // elements per tile
constexpr int kSlots = 8;                    // A rows per element (6 pairs i <= j used)
constexpr int kM = kTile * kSlots;           // 128
constexpr int kN = NN * NN;                  // 64 node pairs (a, b)
constexpr int kKLive = 9 * NG;               // 72 = (r, s, gp)
constexpr int kRows = 6;                     // threads per (element, Gauss point)
constexpr int kPoints = kTile * NG;          // 128 (element, Gauss point) per tile
constexpr int kConsumers = kPoints * kRows;  // 768: warps 0-23
constexpr int kThreads = kConsumers + 32;    // + producer warp 24
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

constexpr int kPtBytes = kPtN * kPoints * 4;
// epilogue scratch inside the point scratch: per accumulator row, the four
// column quarters' shares of 8 sums (row-fastest: a warp's 32 rows in
// distinct banks)
static_assert(4 * 8 * 128 * 4 <= kPtBytes, "epilogue scratch must fit the point scratch");

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
  static constexpr int kStages = (kSplit && !kBF16) ? 1 : 2;
  static constexpr int kOffB = 0;
  static constexpr int kOffA = kOffB + (kSplit ? 2 : 1) * kOpB;
  static constexpr int kOffPt = kOffA + (kSplit ? 2 : 1) * kOpA;
  static constexpr int kOffStage = kOffPt + kPtBytes;
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
  alignas(16) TcgTile hdr[2];          // the tile in each stage, copied in with the stage's data
  // the producer's dof-index slabs (cdest, edest) of two tiles: the next
  // tile's are copied in while this one's gathers are issued
  alignas(16) int idx[2][2][kTile * TOT + 4];
  unsigned long long full[2], empty[2], mma, ibar[2];
  uint32_t tmem_base;
  // a bounded wait gave up: the producer's flag is written by the producer
  // only, the consumers' only by consumers before a named barrier, so that
  // every consumer takes the same branch after that barrier
  int pabort, cabort;
  int issued;                          // tiles whose copies the producer issued
  int ifetch, iwait;                   // index slabs requested / waited for by the producer
  int done;                            // tiles the consumers finished (Ke stored)
};

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


// row of lower-triangle index q (q = r (r + 1) / 2 + c, c <= r)
__host__ __device__ constexpr int lw_row(int q) { return q < 1 ? 0 : q < 3 ? 1 : q < 6 ? 2 : q < 10 ? 3 : q < 15 ? 4 : 5; }

// the point's quantity q in the per-point arrays (kPoints points)
__device__ __forceinline__ float& pv(float* pt, int q, int p) { return tc::pv<kPoints>(pt, q, p); }

// Phase 1 of the Gauss-point work of point p = (element e, Gauss point gp)
// of a tile, thread k = 0..5 of the point: k < 3 forms row k of the
// Jacobian [J]; every k converts its share of the point's double inputs to
// float, each value once: cep entries 4k .. 4k+3 (mm10: history1(1:36))
// and, with finite strain, R entries k and k + 6 and urcs_n1 entry k.
template <int k>
__device__ __forceinline__ void tcg_phase1(const TangentArgs& a, const TcgTile& tl, const unsigned char* st,
                                           const TcgStatic& T, float* pt, int p, int e, int gp) {
  const int i = tl.i0 + e;
  if constexpr (k < 3) {   // row k of [J] = sum_a dN_a/dxi_k x_a (into the [D*] slots, free until phase 2)
    const float* dn = T.dn + (gp * 3 + k) * NN;
    float j0 = 0.f, j1 = 0.f, j2 = 0.f;
#pragma unroll
    for (int n = 0; n < NN; ++n) {
      const float w = dn[n];
      j0 += w * T.x[e][n];
      j1 += w * T.x[e][NN + n];
      j2 += w * T.x[e][2 * NN + n];
    }
    pv(pt, kPtD + 3 * k, p) = j0;
    pv(pt, kPtD + 3 * k + 1, p) = j1;
    pv(pt, kPtD + 3 * k + 2, p) = j2;
  }
  constexpr int q0 = 4 * k, q1 = q0 + 4 < 21 ? q0 + 4 : 21;
  if (tl.flags & 2) {
    const double* Hh = a.hist1 + tl.hist_off + ((long long)i * NG + gp) * kHistMM10;
#pragma unroll
    for (int q = q0; q < q1; ++q) pv(pt, kPtC + q, p) = d2f_rn(Hh[lw_row(q) + 6 * (q - lw_row(q) * (lw_row(q) + 1) / 2)]);
  } else {
    const double* cp = reinterpret_cast<const double*>(
        st + kStCep + gp * kCepSlab + pad_of(a.cep + tl.cep_off + ((long long)gp * tl.span + tl.i0) * 21)) + e * 21;
#pragma unroll
    for (int q = q0; q < q1; ++q) pv(pt, kPtC + q, p) = d2f_rn(cp[q]);
  }
  if (tl.flags & 1) {
    const long long g0 = (tl.gp_off + (long long)tl.i0 * NG) * 9;
    const double* rp = reinterpret_cast<const double*>(st + kStRot + pad_of(a.rot_n1 + g0)) + (e * NG + gp) * 9;
    const double* up = reinterpret_cast<const double*>(st + kStUrcs + pad_of(a.urcs_n1 + g0)) + (e * NG + gp) * 9;
    pv(pt, kPtR + k, p) = d2f_rn(rp[k]);
    if constexpr (k + 6 < 9) pv(pt, kPtR + k + 6, p) = d2f_rn(rp[k + 6]);
    pv(pt, kPtU + k, p) = d2f_rn(up[k]);
  }
}

// phases 2a and 2 of the per-point work (w3g_tc_common.cuh) on this
// kernel's point arrays
template <int k>
__device__ __forceinline__ void tcg_phase2a(const TcgStatic& T, float* pt, int p, int gp, bool geonl) {
  tc::pt_phase2a<k, kPoints>(pt, p, T.dn[NG * 3 * NN + gp], geonl);
}

template <int J>
__device__ __forceinline__ void tcg_phase2(const TangentArgs& a, int flags, float* pt, int p) {
  tc::pt_phase2<J, kPoints>(a.qbar != 0, flags, pt, p);
}

// per pair slot (00 01 02 11 12 22) and entry (r, q) of X^ij: the per-point
// array holding [D*](v(i,r), v(j,q)), and for i = j the one holding
// {T}[r][q] (w det[J] {T}, Voigt index v(r, q))
struct PairIdx {
  unsigned char d[6][9], tw[9];
};
__host__ __device__ constexpr PairIdx make_pair_idx() {
  PairIdx t{};
  for (int sl = 0; sl < 6; ++sl) {
    const int ii = sl < 3 ? 0 : (sl < 5 ? 1 : 2), jj = sl < 3 ? sl : (sl == 3 ? 1 : 2);
    for (int r = 0; r < 3; ++r)
      for (int q = 0; q < 3; ++q) t.d[sl][3 * r + q] = (unsigned char)(kPtD + lw(voigt(ii, r), voigt(jj, q)));
  }
  for (int r = 0; r < 3; ++r)
    for (int q = 0; q < 3; ++q) t.tw[3 * r + q] = (unsigned char)(kPtTw + voigt(r, q));
  return t;
}
__constant__ PairIdx c_pair = make_pair_idx();

// Phase 3, thread `slot` of the point: H^ij = Gamma^T X^ij Gamma for pair
// slot of 00 01 02 11 12 22, X^ij[r][q] = [D*](v(i,r), v(j,q)) + delta_ij
// {T}[r][q], into A operand row (slot, element e), k = (r*3 + s)*8 + gp.
// One code path for the six pairs (indices from a table): specialised
// copies let the compiler hoist the union of their loads and spill.
// 16 accumulator columns of the warp's lane quadrant (the load and its wait
// in one statement)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* out) {
  uint32_t v[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int c = 0; c < 16; ++c) out[c] = __uint_as_float(v[c]);
}

template <bool kBF16, bool kSplit>
__device__ __forceinline__ void tcg_phase3(float* pt, int p, int e, int gp, int slot, unsigned char* opA) {
  using F = Form<kBF16, kSplit>;
  const bool diag = slot == 0 || slot == 3 || slot == 5;
  float gam[9], X[9];
#pragma unroll
  for (int m = 0; m < 9; ++m) gam[m] = pv(pt, kPtGam + m, p);
#pragma unroll
  for (int m = 0; m < 9; ++m) {
    float v = pv(pt, c_pair.d[slot][m], p);
    if (diag) v += pv(pt, c_pair.tw[m], p);
    X[m] = v;
  }
  const int row = slot * kTile + e;
  // one column s of H at a time: y = X Gamma_s, H[r][s] = Gamma_r . y. For
  // i = j, H is symmetric: only r <= s is formed and written to both (r, s)
  // and (s, r), so that the rounded operand stays exactly symmetric --
  // otherwise an entry and its mirror can round to different TF32 / BF16
  // values, and the packed upper triangle (mirrored below the diagonal)
  // loses the exact rigid-translation null space of the node sums
#pragma unroll
  for (int s2 = 0; s2 < 3; ++s2) {
    float y[3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
      y[r] = X[3 * r] * gam[3 * s2] + X[3 * r + 1] * gam[3 * s2 + 1] + X[3 * r + 2] * gam[3 * s2 + 2];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      if (diag && r > s2) continue;
      const float h = gam[3 * r] * y[0] + gam[3 * r + 1] * y[1] + gam[3 * r + 2] * y[2];
      put_split<kBF16, kSplit>(opA, F::kOpA, F::off(row, (3 * r + s2) * 8 + gp), h);
      if (diag && r < s2) put_split<kBF16, kSplit>(opA, F::kOpA, F::off(row, (3 * s2 + r) * 8 + gp), h);
    }
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
    for (int b = 0; b < 2; ++b)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(&T.ibar[b])), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;");
    T.pabort = 0;
    T.cabort = 0;
    T.issued = 0;
    T.done = 0;
    T.ifetch = 0;
    T.iwait = 0;
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
    // The dof indices of the tile after this one are bulk-copied into
    // shared memory (T.idx, on T.ibar) while this tile's gathers are
    // issued, so that no gather waits for an index load from DRAM; the
    // consumers get the tile record by a cp.async into the stage header,
    // on the stage's mbarrier. Index slab copies start at the 16-byte
    // boundary below the slab (the arrays carry 16 bytes of slack at the
    // end); `off` is the slab's first index within the copy.
    constexpr int kPerLane = kTile * TOT / 32;   // 12 gathered dofs per lane and tile
    auto fetch_idx = [&](int t, int b) -> int {  // lane 0: returns the offset of the slab in T.idx[b]
      const TcgTile* r = tiles + t;
      const long long dbase = r->einf_off + (long long)r->i0 * TOT;
      const int nv = r->n * TOT;
      const bool fs = r->flags & 1;
      const uintptr_t pc = (uintptr_t)(a.cdest + dbase), pe_ = (uintptr_t)(a.edest + dbase);
      const uintptr_t pc16 = pc & ~(uintptr_t)15, pe16 = pe_ & ~(uintptr_t)15;
      const uint32_t bytes = (uint32_t)(((pc - pc16) + nv * 4 + 15) & ~15ull);   // same offset for both arrays
      const uint32_t bar = su32(&T.ibar[b]);
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(fs ? 2 * bytes : bytes)
                   : "memory");
      // the slab's previous contents were read (generic proxy) by the
      // gathers of two tiles ago; order those reads before the copy
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      bulk_g2s(su32(&T.idx[b][0][0]), (const void*)pc16, bytes, bar);
      if (fs) bulk_g2s(su32(&T.idx[b][1][0]), (const void*)pe16, bytes, bar);
      T.ifetch += 1;
      return (int)((pc - pc16) >> 2);
    };
    int off_next = 0;
    if (lane == 0) off_next = fetch_idx(blockIdx.x, 0);
    int k = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++k) {
      const int b = k & 1;
      const int off = __shfl_sync(0xffffffffu, off_next, 0);
      const int nv = tiles[t].n * TOT;   // the record line is in cache: read for the index copy
      const bool geonl = tiles[t].flags & 1;
      if (!wait_phase(&T.ibar[b], (k >> 1) & 1, limit, cabort)) {
        if (lane == 0) *pabort = 1;
        break;
      }
      if (lane == 0) T.iwait = k + 1;
      // the next tile's indices, in flight while this tile is issued (the
      // other slab's indices were consumed by the previous tile's gathers)
      if (lane == 0 && t + (int)gridDim.x < ntiles) off_next = fetch_idx(t + gridDim.x, b ^ 1);
      int ci[kPerLane], ei[kPerLane];
#pragma unroll
      for (int j = 0; j < kPerLane; ++j) {
        const int q = lane + 32 * j;
        ci[j] = q < nv ? T.idx[b][0][off + q] - 1 : 0;
        ei[j] = q < nv && geonl ? T.idx[b][1][off + q] - 1 : 0;
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
        const TcgTile tl = tiles[t];   // the record line is in cache (fetched one tile ago)
        // the record into the stage header, complete when the stage is
        for (int c = 0; c < 4; ++c)
          asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(su32(&T.hdr[s]) + 16 * c),
                       "l"(reinterpret_cast<const char*>(tiles + t) + 16 * c) : "memory");
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
    // warp w: thread k = w % 6 of points p = lane + 32 (w / 6); point p is
    // (element (lane & 7) + 8 (g & 1), Gauss point (lane >> 3) + 4 (g >> 1))
    // with g = w / 6, so that the 32 lanes of a warp write their A operand
    // values (rows slot*16 + element, k = .. + Gauss point) into 32
    // distinct banks and read the per-point arrays consecutively
    const int g = warp / kRows, kr = warp % kRows;
    const int p = lane + 32 * g, pe = (lane & 7) + 8 * (g & 1), pg = (lane >> 3) + 4 * (g >> 1);
    float* pt = reinterpret_cast<float*>(smem + F::kOffPt);
    int k = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++k) {
      const int s = k % S;
      const unsigned char* st = stages + s * kStage;
      if (!wait_phase(&T.full[s], (k / S) & 1, limit, pabort)) *cabort = 1;
      // previous tile's Ke store must have read the staging (A region)
      if (tid == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
      asm volatile("bar.sync 1, %0;" ::"n"(kConsumers) : "memory");
      if (*cabort) break;
      // the tile record (the stage, record included, is handed back to the
      // producer once phase 1 has read it)
      const TcgTile tl = T.hdr[s];
      const int tn = tl.n;
      float* const out = reinterpret_cast<float*>(a.estiff) + tl.estiff_off + (long long)tl.i0 * UT;
      // element coordinates at n+1 relative to node 1
      for (int q = tid; q < tn * TOT; q += kConsumers) {
        const int e = q / TOT, d = q % TOT, q0 = e * TOT + (d / NN) * NN;
        const double* xc = reinterpret_cast<const double*>(st + kStXc);
        double v = xc[q], ref = xc[q0];
        if (tl.flags & 1) {
          const double* xu = reinterpret_cast<const double*>(st + kStXu);
          const double* xdu = reinterpret_cast<const double*>(st + kStXdu);
          v = v + xu[q] + xdu[q];
          ref = ref + xu[q0] + xdu[q0];
        }
        T.x[e][d] = d2f_rn(v - ref);
      }
      asm volatile("bar.sync 1, %0;" ::"n"(kConsumers) : "memory");
      const bool live = pe < tn;
      if (live) {
        switch (kr) {
          case 0: tcg_phase1<0>(a, tl, st, T, pt, p, pe, pg); break;
          case 1: tcg_phase1<1>(a, tl, st, T, pt, p, pe, pg); break;
          case 2: tcg_phase1<2>(a, tl, st, T, pt, p, pe, pg); break;
          case 3: tcg_phase1<3>(a, tl, st, T, pt, p, pe, pg); break;
          case 4: tcg_phase1<4>(a, tl, st, T, pt, p, pe, pg); break;
          default: tcg_phase1<5>(a, tl, st, T, pt, p, pe, pg); break;
        }
      }
      asm volatile("bar.sync 1, %0;" ::"n"(kConsumers) : "memory");
      // stage consumed: hand it back to the producer
      if (tid == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(&T.empty[s])) : "memory");
      if (live) {
        const bool geonl = tl.flags & 1;
        switch (kr) {
          case 0: tcg_phase2a<0>(T, pt, p, pg, geonl); break;
          case 1: tcg_phase2a<1>(T, pt, p, pg, geonl); break;
          case 2: tcg_phase2a<2>(T, pt, p, pg, geonl); break;
          case 3: tcg_phase2a<3>(T, pt, p, pg, geonl); break;
          case 4: tcg_phase2a<4>(T, pt, p, pg, geonl); break;
          default: tcg_phase2a<5>(T, pt, p, pg, geonl); break;
        }
      }
      asm volatile("bar.sync 1, %0;" ::"n"(kConsumers) : "memory");
      if (live) {
        switch (kr) {
          case 0: tcg_phase2<0>(a, tl.flags, pt, p); break;
          case 1: tcg_phase2<1>(a, tl.flags, pt, p); break;
          case 2: tcg_phase2<2>(a, tl.flags, pt, p); break;
          case 3: tcg_phase2<3>(a, tl.flags, pt, p); break;
          case 4: tcg_phase2<4>(a, tl.flags, pt, p); break;
          default: tcg_phase2<5>(a, tl.flags, pt, p); break;
        }
      }
      asm volatile("bar.sync 1, %0;" ::"n"(kConsumers) : "memory");
      // H into the A operand (the previous tile's MMAs are complete and its
      // Ke store has read the region)
      if (live) tcg_phase3<kBF16, kSplit>(pt, p, pe, pg, kr, opA);
      if constexpr (kBF16) {   // the K padding (72..79) must be finite zeros: the staging reuses the region
        for (int z = tid; z < kM * (F::kK - kKLive); z += kConsumers) {
          const int row = z / (F::kK - kKLive), kk = kKLive + z % (F::kK - kKLive);
          put<kBF16>(opA, F::off(row, kk), 0.f);
          if (kSplit) put<kBF16>(opA + F::kOpA, F::off(row, kk), 0.f);
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("bar.sync 1, %0;" ::"n"(kConsumers) : "memory");
      if (tid == 0) {
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
      // accumulator -> Ke. The tensor cores' FP32 accumulation is not
      // sign-symmetric: its error has a mean, the same in every element,
      // along the rigid translations, which a plastic mesh's softest modes
      // do not tolerate (Newton stalls or K_ff turns indefinite). So each
      // node-pair block leaves with the translations projected out,
      // K' = P S P, P = I - 11^T / 8, S the block as stored (a diagonal
      // block's upper triangle mirrored); the exact Ke has these null
      // vectors, so the projection only removes error.
      // Warp w < 16 reads TMEM lane quadrant w % 4 (the quadrant a warp may
      // access), columns 16 (w / 4) .. + 15: rows x = 2 (w / 4), + 1 of its
      // lane's block. (1) Each thread publishes its share q_b of the block's
      // column sums (off-diagonal blocks) or of the row sums of S (diagonal
      // blocks: the upper part of its rows, the mirrored part of the rows
      // below), b = 0..7, in the point scratch (free until the next tile's
      // phase 1); its own rows' sums stay in registers. (2) After one
      // barrier it adds its lane's four shares, reloads its accumulator
      // values and packs S_xb - (r_x + c_b) / 8 + (sum of S) / 64, times
      // beta_fact, into the staging (the A region: the MMAs are done).
      float* part = reinterpret_cast<float*>(smem + F::kOffPt);   // [4 column quarters][8][kM rows]
      const int quad = warp & 3, cq = warp >> 2;
      const int row = 32 * quad + lane, e = row & (kTile - 1), slot = row >> 4;
      const int ii = slot < 3 ? 0 : (slot < 5 ? 1 : 2);
      const int jj = slot < 3 ? slot : (slot == 3 ? 1 : 2);
      const bool diag = ii == jj;
      const uint32_t taddr = tmem + ((uint32_t)(32 * quad) << 16) + (uint32_t)(16 * cq);
      float rs0 = 0.f, rs1 = 0.f;   // row sums of rows 2 cq, 2 cq + 1 (off-diagonal blocks)
      if (warp < 16) {
        float v[16];
        tmem_ld16(taddr, v);
        float q[8];
#pragma unroll
        for (int b = 0; b < 8; ++b) {
          const int x0 = 2 * cq, x1 = 2 * cq + 1;
          // diagonal: S_xb = K_xb for b >= x contributes to r_x (below);
          // for b > x it is also S_bx and contributes to r_b
          q[b] = diag ? (b > x0 ? v[b] : 0.f) + (b > x1 ? v[8 + b] : 0.f) : v[b] + v[8 + b];
          rs0 += diag && b < x0 ? 0.f : v[b];
          rs1 += diag && b < x1 ? 0.f : v[8 + b];
        }
        if (diag) {   // the thread's own rows enter the shared sums
#pragma unroll
          for (int b = 0; b < 8; ++b) q[b] += b == 2 * cq ? rs0 : (b == 2 * cq + 1 ? rs1 : 0.f);
        }
#pragma unroll
        for (int b = 0; b < 8; ++b) part[(cq * 8 + b) * kM + row] = q[b];
      }
      asm volatile("bar.sync 1, %0;" ::"n"(kConsumers) : "memory");
      if (warp < 16) {
        // the load is warp-collective (.sync.aligned): every lane of the
        // warp executes it, whatever its row
        float v[16];
        tmem_ld16(taddr, v);
        if (slot < 6 && e < tn) {
          float* ke = reinterpret_cast<float*>(opA);
          const float bf = (float)a.beta_fact;
          float sb[8], tot = 0.f;
#pragma unroll
          for (int b = 0; b < 8; ++b) {
            sb[b] = part[b * kM + row] + part[(8 + b) * kM + row] + part[(16 + b) * kM + row] +
                    part[(24 + b) * kM + row];
            tot += sb[b];
          }
          // diagonal: sb = row sums of S (= its column sums); off-diagonal:
          // sb = column sums, rs = the thread's row sums
          const float r0 = diag ? sb[2 * cq] : rs0, r1 = diag ? sb[2 * cq + 1] : rs1;
          const float t64 = 0.015625f * tot;
#pragma unroll
          for (int c = 0; c < 16; ++c) {
            const int an = 2 * cq + (c >> 3), bn = c & 7;
            if (diag && an > bn) continue;
            const int d1 = ii * NN + an, d2 = jj * NN + bn;
            const float kp = v[c] - 0.125f * ((c < 8 ? r0 : r1) + sb[bn]) + t64;
            ke[e * UT + d2 * (d2 + 1) / 2 + d1] = kp * bf;
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
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
      for (int q = T.iwait; q < T.ifetch; ++q) wait_phase(&T.ibar[q & 1], (q >> 1) & 1, kDrainLimit, nullptr);
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
