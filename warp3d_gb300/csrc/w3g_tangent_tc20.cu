// w3g_tangent_tc20.cu -- precision forms of the 20-node brick tangent on the
// fifth-generation tensor cores.
//
// WARP3D's material and geometric stiffness of a q3disop element (gptns1.f
// bdbtgen :1628, kg1.f :16) is, per pair of displacement components
// i <= j and nodes a, b,
//   Ke_ij[a][b] = sum_gp n_a^T H^ij_gp n_b,   H^ij = Gamma^T X^ij Gamma,
// with n_a = dN_a/dxi at the Gauss point, Gamma = J^-1 and X^ij[p][q] =
// [D*](v(i,p), v(j,q)) + delta_ij {T}[p][q] (the same point quantities as
// the 8-node brick's gradient-pair kernel). Splitting the node sums,
//   Ke_ij[a][b] = sum_{gp,r} n_a[r](gp) Y[(ij,b), (gp,r)],
//   Y[(ij,b), (gp,r)] = sum_s H^ij_gp[r][s] n_b[s](gp),
// every element's tangent is ONE product of its Y (120 rows (pair, node b)
// x K = 81 (Gauss point, r)) with the CONSTANT operator N_A[a, (gp, r)] =
// n_a[r](gp) of the element type: an MMA of M = 128 (120 used), N = 32 (20
// used), K = 81 (padded to 88 for TF32, 96 for BF16), FP32 accumulation in
// 32 TMEM columns. The CUDA cores form the Gauss-point quantities and Y
// (~1,900 multiply-adds per point, against ~8,000 for B^T D* B + G^T T G).
//
// Operand precision: rounding N_A or Y to TF32 or BF16 does NOT keep the
// exact rigid-translation null space here (the 27-point rule has no mirror
// symmetry of dN/dxi between nodes), and the tensor cores' FP32
// accumulation adds an error with a mean along the translations; the
// epilogue therefore projects the translations out of every node-pair
// block, which leaves them at the FP32 rounding level whatever the operand
// rounding. TF32 requests round both operands once (one MMA per k-step);
// BF16 requests round Y once and split the constant N_A, x = hi + lo in
// the input format (Y*hi + Y*lo: two MMAs; see launch_tangent_tc_hex20);
// the X3 forms split both and accumulate hi*hi + hi*lo + lo*hi (three
// MMAs).
//
// One CTA of 8 warps per record of up to 8 elements of a block, elements in
// turn, two CTAs per SM (one for TF32x3, by shared memory):
//   (0) the element's coordinates at n+1 relative to its node 1 (cdest /
//       edest gathers);
//   (1)-(3) warp k = thread k of every Gauss point (lane = point):
//       [J] rows and the float conversion of cep, R, urcs_n1 (each value
//       once); Gamma, w det J, {T}; row k of w det J [D*]; H of pair k
//       (exactly symmetric for i = j) into shared memory;
//   (4) threads 0-119, one per row (pair, node b): the 81 values of Y,
//       split and written into the A operand (K-major, no swizzle);
//   (5) thread 0 issues the 3 x K/k-step MMAs and commits to an mbarrier;
//   (6) warps 0-3 read the accumulator (tcgen05.ld, each warp its lane
//       quadrant) into shared memory; the rigid translations are projected
//       out of every node-pair block, scaled by beta_fact and the packed
//       upper triangle (utsz = 1830, setup.f:265-275) stored coalesced as
//       FP32.
// The one wait (for the MMAs) is bounded by TangentArgs::wait_limit; a wait
// that gives up drains the MMAs (bounded), fills NaN Ke for every element of
// the CTA not finished and sets the timeout flag (W3G_EFATAL). A limit of 0
// gives up before the first MMA is issued.
#include <cstdint>
#include "w3g_internal.cuh"
#include "w3g_elem.cuh"
#include "w3g_math.cuh"
#include "w3g_tc_common.cuh"

namespace w3g {

namespace {

using namespace tc;

constexpr int NN = Hex20::NN, NG = Hex20::NG, TOT = Hex20::TOTDOF, UT = Hex20::UTSZ;
constexpr int kPts = 32;                 // point slots per quantity (27 used)
constexpr int kThreads = 8 * 32;         // warps 0-5: thread k of every Gauss point; 6-7: prefetch
constexpr int kM = 128;                  // MMA rows: (pair, node b), 120 used
constexpr int kCols = 32;                // MMA columns: node a, 20 used
constexpr int kKLive = 3 * NG;           // 81: (Gauss point, r)
constexpr int kRowsLive = 6 * NN;        // 120
constexpr int kTmemCols = 32;
constexpr long long kDrainLimit = 1ll << 26;

// an element's inputs, prefetched by warps 6-7 while the element before is
// processed (8-byte cp.async: gathered nodal values, the 27 cep rows, the
// element's contiguous R and stress slabs)
struct Tc20Inputs {
  double c[TOT], u[TOT], du[TOT];
  double cep[NG * 21];
  double rot[NG * 9], urcs[NG * 9];
};

template <bool kBF16, bool kSplit>
struct Op {
  static constexpr int kBytes = kBF16 ? 2 : 4;
  static constexpr int kPerCore = 16 / kBytes;              // K values per core-matrix row
  static constexpr int kKStep = kBF16 ? 16 : 8;
  static constexpr int kK = (kKLive + kKStep - 1) / kKStep * kKStep;   // 96 / 88
  static constexpr int kSteps = kK / kKStep;
  // next 8-row group: 16 bytes more than the group's K extent, so that the
  // stores of 32 consecutive rows fall into distinct banks
  static constexpr int kSBO = (kK / kPerCore) * 128 + 16;
  static constexpr int kOpA = (kM / 8) * kSBO;              // hi part; the lo part follows (split)
  static constexpr int kOpB = (kCols / 8) * kSBO;
  static constexpr int kParts = kSplit ? 2 : 1;             // A operand parts
  static constexpr bool kSplitB = kSplit || kBF16;          // N_A as hi + lo
  static constexpr int kPartsB = kSplitB ? 2 : 1;
  static constexpr int kPerSm = (kBF16 || !kSplit) ? 2 : 1;   // CTAs per SM (shared memory)
  static constexpr int kOffB = 0;
  static constexpr int kOffA = kOffB + kPartsB * kOpB;
  static constexpr int kOffIn = kOffA + kParts * kOpA;           // two Tc20Inputs: this and the next element
  static constexpr int kSmem = kOffIn + 2 * (int)sizeof(Tc20Inputs);
  // byte offset of (row, k) in a K-major no-swizzle operand
  __device__ static __forceinline__ int off(int row, int k) {
    return (row >> 3) * kSBO + (k / kPerCore) * 128 + (row & 7) * 16 + (k % kPerCore) * kBytes;
  }
};

// where an element of the CTA's sequence lives
struct Tc20Elem {
  long long cep_off, gp_off, estiff_off, einf_off;
  int i, span, flags, pad;
};

struct Tc20Static {
  float dn[NG * 3 * NN + NG];          // dN/dxi per Gauss point (float) + weights
  float x[TOT];                        // x(n+1) relative to node 1
  float pt[kPtN * kPts];               // per-point intermediates
  float H[NG][6][9];                   // H^ij per point and pair
  float ke[UT];                        // packed Ke of the element in the epilogue
  unsigned long long mma;
  uint32_t tmem_base;
  int abort;                           // a wait gave up (written before a barrier)
  int fail_n;                          // sequence index of the first element not stored
};

// instruction descriptor: FP32 accumulator, A/B K-major, M = 128, N = 32
template <bool kBF16>
__host__ __device__ constexpr uint32_t idesc20() {
  return (1u << 4) | ((kBF16 ? 1u : 2u) << 7) | ((kBF16 ? 1u : 2u) << 10) | ((uint32_t)(kCols >> 3) << 17) |
         ((uint32_t)(kM >> 4) << 24);
}

template <bool kBF16>
__device__ __forceinline__ void mma20(uint32_t tmem, uint64_t da, uint64_t db, bool acc) {
  const uint32_t id = idesc20<kBF16>(), a = acc ? 1u : 0u;
  if (kBF16)
    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                 ::"r"(tmem), "l"(da), "l"(db), "r"(id), "r"(a));
  else
    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}"
                 ::"r"(tmem), "l"(da), "l"(db), "r"(id), "r"(a));
}

__device__ __forceinline__ float& pv20(float* pt, int q, int g) { return pv<kPts>(pt, q, g); }

// Phase 1, thread k of Gauss point g: k < 3 forms row k of [J] (into the
// [D*] slots); every k converts its share of the point's staged double
// inputs to float: cep entries 4k .. 4k+3 and, with finite strain, R
// entries k and k + 6 and urcs_n1 entry k.
template <int k>
__device__ __forceinline__ void tc20_phase1(const Tc20Inputs& in, bool geonl, Tc20Static& T, int g) {
  float* pt = T.pt;
  if constexpr (k < 3) {
    const float* dn = T.dn + (g * 3 + k) * NN;
    float j0 = 0.f, j1 = 0.f, j2 = 0.f;
#pragma unroll
    for (int n = 0; n < NN; ++n) {
      const float w = dn[n];
      j0 += w * T.x[n];
      j1 += w * T.x[NN + n];
      j2 += w * T.x[2 * NN + n];
    }
    pv20(pt, kPtD + 3 * k, g) = j0;
    pv20(pt, kPtD + 3 * k + 1, g) = j1;
    pv20(pt, kPtD + 3 * k + 2, g) = j2;
  }
  constexpr int q0 = 4 * k, q1 = q0 + 4 < 21 ? q0 + 4 : 21;
#pragma unroll
  for (int q = q0; q < q1; ++q) pv20(pt, kPtC + q, g) = d2f_rn(in.cep[g * 21 + q]);
  if (geonl) {
    pv20(pt, kPtR + k, g) = d2f_rn(in.rot[g * 9 + k]);
    if constexpr (k + 6 < 9) pv20(pt, kPtR + k + 6, g) = d2f_rn(in.rot[g * 9 + k + 6]);
    pv20(pt, kPtU + k, g) = d2f_rn(in.urcs[g * 9 + k]);
  }
}

// Phase 3, thread `slot` of point g: H^ij = Gamma^T X^ij Gamma for pair
// slot (00 01 02 11 12 22); for i = j only r <= s is formed and mirrored,
// so that H^ii is exactly symmetric.
__device__ __forceinline__ void tc20_phase3(Tc20Static& T, int g, int slot) {
  float* pt = T.pt;
  const int ii = slot < 3 ? 0 : (slot < 5 ? 1 : 2);
  const int jj = slot < 3 ? slot : (slot == 3 ? 1 : 2);
  const bool diag = ii == jj;
  float gam[9], X[9];
#pragma unroll
  for (int m = 0; m < 9; ++m) gam[m] = pv20(pt, kPtGam + m, g);
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      float v = pv20(pt, kPtD + lw(voigt(ii, r), voigt(jj, q)), g);
      if (diag) v += pv20(pt, kPtTw + voigt(r, q), g);
      X[3 * r + q] = v;
    }
  float* h = T.H[g][slot];
#pragma unroll
  for (int s2 = 0; s2 < 3; ++s2) {
    float y[3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
      y[r] = X[3 * r] * gam[3 * s2] + X[3 * r + 1] * gam[3 * s2 + 1] + X[3 * r + 2] * gam[3 * s2 + 2];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      if (diag && r > s2) continue;
      const float v = gam[3 * r] * y[0] + gam[3 * r + 1] * y[1] + gam[3 * r + 2] * y[2];
      h[3 * r + s2] = v;
      if (diag && r < s2) h[3 * s2 + r] = v;
    }
  }
}

// the CTA's elements in sequence: records blockIdx.x, blockIdx.x + grid, ...
// and their elements in turn; advances (t, e) and fills the descriptor
__device__ __forceinline__ bool tc20_next(const TcgTile* tiles, int ntiles, int& t, int& e, Tc20Elem& d) {
  while (t < ntiles) {
    const TcgTile r = tiles[t];
    if (e < r.n) {
      d.cep_off = r.cep_off; d.gp_off = r.gp_off; d.estiff_off = r.estiff_off; d.einf_off = r.einf_off;
      d.i = r.i0 + e; d.span = r.span; d.flags = r.flags;
      ++e;
      return true;
    }
    t += gridDim.x;
    e = 0;
  }
  return false;
}

// warps 6-7 (64 threads, index p): the element's inputs into `in`, 8-byte
// cp.async (the completion is waited for by the same threads)
__device__ __forceinline__ void tc20_prefetch(const TangentArgs& a, const Tc20Elem& d, Tc20Inputs& in, int p) {
  const long long dbase = d.einf_off + (long long)d.i * TOT;
  const bool geonl = d.flags & 1;
  for (int q = p; q < TOT; q += 64) {
    const int ci = a.cdest[dbase + q] - 1;
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(su32(in.c + q)), "l"(a.c + ci) : "memory");
    if (geonl) {
      const int ei = a.edest[dbase + q] - 1;
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(su32(in.u + q)), "l"(a.u + ei) : "memory");
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(su32(in.du + q)), "l"(a.du + ei) : "memory");
    }
  }
  for (int q = p; q < NG * 21; q += 64) {
    const int g = q / 21, m = q % 21;
    const double* src = a.cep + d.cep_off + ((long long)g * d.span + d.i) * 21 + m;
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(su32(in.cep + q)), "l"(src) : "memory");
  }
  if (geonl) {
    const long long g0 = (d.gp_off + (long long)d.i * NG) * 9;
    for (int q = p; q < NG * 9; q += 64) {
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(su32(in.rot + q)), "l"(a.rot_n1 + g0 + q)
                   : "memory");
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(su32(in.urcs + q)), "l"(a.urcs_n1 + g0 + q)
                   : "memory");
    }
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
}

// accumulator of one element -> packed Ke in T.ke, with the rigid
// translations projected out of every node-pair block: K' = P S P,
// P = I - 11^T / 20, S the block as stored (a diagonal block's upper
// triangle mirrored). The tensor cores' FP32 accumulation is not
// sign-symmetric, so its error has a mean along the translations, the same
// in every element, which the soft modes of a yielded mesh do not
// tolerate; the exact Ke has these null vectors, so the projection only
// removes error. raw: shared memory free during the epilogue (the start
// of the A operand: the element's MMAs are done; the next element's Y
// rewrites every value of the live rows, K padding included) for the 120
// accumulator rows (pair, node b) x node a, then the row and column sums
// of each pair.
// Every thread of the CTA takes part (two barriers).
__device__ __forceinline__ void tc20_epilogue(uint32_t tmem, int warp, int lane, int tid, Tc20Static& T, float* raw,
                                              float bf) {
  constexpr int kLd = NN + 1;            // odd row stride: a warp's 32 rows in distinct banks
  float* sums = raw + kRowsLive * kLd;   // per pair slot: r_a (20), c_b (20)
  if (warp < 4) {   // warp w reads lane quadrant w
    const int row = 32 * warp + lane;
    const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16);
    uint32_t v[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%32];\n"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%33];\n"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]),
          "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
          "=r"(v[30]), "=r"(v[31])
        : "r"(taddr), "r"(taddr + 16)
        : "memory");
    if (row < kRowsLive) {
#pragma unroll
      for (int an = 0; an < NN; ++an) raw[row * kLd + an] = __uint_as_float(v[an]);
    }
  }
  __syncthreads();
  // K_ab of pair slot p sits in row (p, b), column a
  if (tid < 6 * 2 * NN) {
    const int slot = tid / (2 * NN), q = tid % (2 * NN);
    const bool diag = slot == 0 || slot == 3 || slot == 5;
    const float* r = raw + slot * NN * kLd;
    float acc = 0.f;
#pragma unroll 4
    for (int t = 0; t < NN; ++t) {
      const int an = q < NN ? q : t, b = q < NN ? t : q - NN;
      acc += diag && an > b ? r[an * kLd + b] : r[b * kLd + an];
    }
    sums[slot * 2 * NN + q] = acc;
  }
  __syncthreads();
  if (warp < 4) {
    const int row = 32 * warp + lane;
    if (row < kRowsLive) {
      const int slot = row / NN, b = row % NN;
      const int ii = slot < 3 ? 0 : (slot < 5 ? 1 : 2);
      const int jj = slot < 3 ? slot : (slot == 3 ? 1 : 2);
      const int d2 = jj * NN + b;
      const float* sm = sums + slot * 2 * NN;
      float tot = 0.f;
#pragma unroll
      for (int t = 0; t < NN; ++t) tot += sm[t];
      const float cb = sm[NN + b] - 0.05f * tot;
#pragma unroll
      for (int an = 0; an < NN; ++an) {
        if (ii == jj && an > b) continue;
        const int d1 = ii * NN + an;
        const float kp = raw[row * kLd + an] - 0.05f * (sm[an] + cb);
        T.ke[d2 * (d2 + 1) / 2 + d1] = kp * bf;
      }
    }
  }
}

template <bool kBF16, bool kSplit>
__global__ void __launch_bounds__(kThreads, Op<kBF16, kSplit>::kPerSm) k_tangent_tc_hex20(
    TangentArgs a, const TcgTile* tiles, int ntiles, int* tc_timeout) {
  using O = Op<kBF16, kSplit>;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* opB = smem + O::kOffB;
  unsigned char* opA = smem + O::kOffA;
  Tc20Inputs* inb = reinterpret_cast<Tc20Inputs*>(smem + O::kOffIn);
  __shared__ Tc20Static T;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long limit = a.wait_limit;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&T.tmem_base)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(&T.mma)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;");
    T.abort = 0;
    T.fail_n = -1;
  }
  const double* dnd = a.dn[Hex20::SLOT];
  for (int k = tid; k < NG * 3 * NN + NG; k += kThreads) T.dn[k] = (float)dnd[k];
  // the constant operator N_A (B operand): row a, k = gp*3 + r, hi and lo
  // parts of the double value; rows a >= 20 and k >= 81 zero
  for (int idx = tid; idx < kCols * O::kK; idx += kThreads) {
    const int row = idx / O::kK, k = idx % O::kK;
    double v = 0.0;
    if (row < NN && k < kKLive) v = dnd[k * NN + row];   // k = gp*3 + r
    const float hi = round_in<kBF16>((float)v);
    put<kBF16>(opB, O::off(row, k), hi);
    if (O::kSplitB) put<kBF16>(opB + O::kOpB, O::off(row, k), (float)(v - (double)hi));
  }
  // A rows 120..127 and the K padding stay zero (finite) for every element
  for (int idx = tid; idx < kM * O::kK; idx += kThreads) {
    const int row = idx / O::kK, k = idx % O::kK;
    if (row >= kRowsLive || k >= kKLive) {
      put<kBF16>(opA, O::off(row, k), 0.f);
      if (kSplit) put<kBF16>(opA + O::kOpA, O::off(row, k), 0.f);
    }
  }
  // the first element's inputs
  int nt = blockIdx.x, ne = 0;   // position of the next element in the sequence
  Tc20Elem cur, prev{}, nxt;
  bool have = tc20_next(tiles, ntiles, nt, ne, cur);
  if (have && warp >= 6) {
    tc20_prefetch(a, cur, inb[0], tid - 192);
    asm volatile("cp.async.wait_all;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = T.tmem_base;
  const float bf = (float)a.beta_fact;
  const int g = lane, kr = warp;   // phases 1-3: Gauss point, thread of the point

  // element n: its point phases overlap the MMAs of element n - 1, whose
  // epilogue follows; then Y of n into the A operand and its MMAs
  int n = 0;
  for (; have; ++n) {
    const Tc20Inputs& in = inb[n & 1];
    const bool more = tc20_next(tiles, ntiles, nt, ne, nxt);
    if (more && warp >= 6) tc20_prefetch(a, nxt, inb[(n + 1) & 1], tid - 192);
    // (0) coordinates at n+1 relative to node 1
    if (tid < TOT) {
      const int d0 = (tid / NN) * NN;
      double v = in.c[tid], ref = in.c[d0];
      if (cur.flags & 1) {
        v = v + in.u[tid] + in.du[tid];
        ref = ref + in.u[d0] + in.du[d0];
      }
      T.x[tid] = d2f_rn(v - ref);
    }
    __syncthreads();
    // (1) [J] rows, conversions
    const bool geonl = cur.flags & 1;
    if (warp < 6 && g < NG) {
      switch (kr) {
        case 0: tc20_phase1<0>(in, geonl, T, g); break;
        case 1: tc20_phase1<1>(in, geonl, T, g); break;
        case 2: tc20_phase1<2>(in, geonl, T, g); break;
        case 3: tc20_phase1<3>(in, geonl, T, g); break;
        case 4: tc20_phase1<4>(in, geonl, T, g); break;
        default: tc20_phase1<5>(in, geonl, T, g); break;
      }
    }
    __syncthreads();
    // (2a) Gamma, w det J, {T}
    if (warp < 6 && g < NG) {
      const float w = T.dn[NG * 3 * NN + g];
      switch (kr) {
        case 0: pt_phase2a<0, kPts>(T.pt, g, w, geonl); break;
        case 1: pt_phase2a<1, kPts>(T.pt, g, w, geonl); break;
        case 2: pt_phase2a<2, kPts>(T.pt, g, w, geonl); break;
        case 3: pt_phase2a<3, kPts>(T.pt, g, w, geonl); break;
        case 4: pt_phase2a<4, kPts>(T.pt, g, w, geonl); break;
        default: pt_phase2a<5, kPts>(T.pt, g, w, geonl); break;
      }
    }
    __syncthreads();
    // (2) rows of w det J [D*]
    if (warp < 6 && g < NG) {
      const bool qb = a.qbar != 0;
      switch (kr) {
        case 0: pt_phase2<0, kPts>(qb, cur.flags, T.pt, g); break;
        case 1: pt_phase2<1, kPts>(qb, cur.flags, T.pt, g); break;
        case 2: pt_phase2<2, kPts>(qb, cur.flags, T.pt, g); break;
        case 3: pt_phase2<3, kPts>(qb, cur.flags, T.pt, g); break;
        case 4: pt_phase2<4, kPts>(qb, cur.flags, T.pt, g); break;
        default: pt_phase2<5, kPts>(qb, cur.flags, T.pt, g); break;
      }
    }
    __syncthreads();
    // (3) H per point and pair
    if (warp < 6 && g < NG) tc20_phase3(T, g, kr);
    // the next element's inputs have landed (read after the loop's next barrier)
    if (warp >= 6) asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();
    // (6) of element n - 1: its MMAs done, accumulator -> packed Ke -> global
    if (n > 0) {
      if (!wait_phase(&T.mma, (n - 1) & 1, limit, nullptr)) {
        // the MMAs may still be running: wait them out before tensor memory
        // is read or freed
        T.abort = 1;
        wait_phase(&T.mma, (n - 1) & 1, kDrainLimit, nullptr);
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      __syncthreads();
      if (T.abort) {
        if (tid == 0) T.fail_n = n - 1;
        break;
      }
      tc20_epilogue(tmem, warp, lane, tid, T, reinterpret_cast<float*>(opA), bf);
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      float* out = reinterpret_cast<float*>(a.estiff) + prev.estiff_off + (long long)prev.i * UT;
      for (int z = tid; z < UT; z += kThreads) out[z] = T.ke[z];
    }
    // (4) Y of element n into the A operand (element n - 1's MMAs are
    // complete): 240 threads, one per row (pair, node b) and half of the
    // Gauss points; the second half also rewrites the row's K padding with
    // zeros (the epilogue's scratch overwrote it in the first rows, and a
    // bit pattern that decodes as Inf or NaN would turn 0 x pad into NaN)
    if (tid < 2 * kRowsLive) {
      const int row = tid % kRowsLive, half = tid / kRowsLive;
      const int slot = row / NN, b = row % NN;
      const int g0 = half ? 14 : 0, g1 = half ? NG : 14;
#pragma unroll 2
      for (int gp = g0; gp < g1; ++gp) {
        const float* h = T.H[gp][slot];
        const float n0 = T.dn[(gp * 3 + 0) * NN + b], n1 = T.dn[(gp * 3 + 1) * NN + b],
                    n2 = T.dn[(gp * 3 + 2) * NN + b];
#pragma unroll
        for (int r = 0; r < 3; ++r)
          put_split<kBF16, kSplit>(opA, O::kOpA, O::off(row, gp * 3 + r), h[3 * r] * n0 + h[3 * r + 1] * n1 + h[3 * r + 2] * n2);
      }
      if (half)
        for (int k = kKLive; k < O::kK; ++k) put_split<kBF16, kSplit>(opA, O::kOpA, O::off(row, k), 0.f);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (limit == 0) {   // give up before any MMA (the status path without a fault)
      if (tid == 0) { T.abort = 1; T.fail_n = n; }
      break;
    }
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint64_t da = sdesc(su32(opA), O::kSBO), db = sdesc(su32(opB), O::kSBO);
      const uint64_t dal = da + (O::kOpA >> 4), dbl = db + (O::kOpB >> 4);
#pragma unroll 1
      for (int ks = 0; ks < O::kSteps; ++ks) {
        const uint64_t o = (uint64_t)ks * (256 >> 4);   // one k-step = two core matrices along K
        mma20<kBF16>(tmem, da + o, db + o, ks > 0);
        if (O::kSplitB) mma20<kBF16>(tmem, da + o, dbl + o, true);
        if (kSplit) mma20<kBF16>(tmem, dal + o, db + o, true);
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          su32(&T.mma)) : "memory");
    }
    prev = cur;
    cur = nxt;
    have = more;
  }
  // the last element's epilogue
  if (!T.abort && n > 0) {
    if (!wait_phase(&T.mma, (n - 1) & 1, limit, nullptr)) {
      T.abort = 1;
      wait_phase(&T.mma, (n - 1) & 1, kDrainLimit, nullptr);
    }
    asm volatile("tcgen05.fence::after_thread_sync;");
    __syncthreads();
    if (T.abort) {
      if (tid == 0) T.fail_n = n - 1;
    } else {
      tc20_epilogue(tmem, warp, lane, tid, T, reinterpret_cast<float*>(opA), bf);
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      float* out = reinterpret_cast<float*>(a.estiff) + prev.estiff_off + (long long)prev.i * UT;
      for (int z = tid; z < UT; z += kThreads) out[z] = T.ke[z];
    }
  }
  if (warp >= 6) asm volatile("cp.async.wait_all;" ::: "memory");   // no copy outlives the CTA
  __syncthreads();
  if (T.abort) {
    // NaN for every element of the CTA's sequence from the first one not stored
    if (tid == 0) atomicExch(tc_timeout, 1);
    int t = blockIdx.x, e = 0, k = 0;
    Tc20Elem d;
    while (tc20_next(tiles, ntiles, t, e, d)) {
      if (k++ < T.fail_n) continue;
      float* out = reinterpret_cast<float*>(a.estiff) + d.estiff_off + (long long)d.i * UT;
      for (int z = tid; z < UT; z += kThreads) out[z] = __int_as_float(0x7fc00000);
    }
  }
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
  }
}

template <bool kBF16, bool kSplit>
cudaError_t set_attr20() {
  return cudaFuncSetAttribute(k_tangent_tc_hex20<kBF16, kSplit>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              Op<kBF16, kSplit>::kSmem);
}

template <bool kBF16, bool kSplit>
cudaError_t launch20(const DeviceModel& m, const TangentArgs& a, int* tc_timeout, cudaStream_t s) {
  using O = Op<kBF16, kSplit>;
  // as many CTAs as fit (1-2 per SM by shared memory), records taken in turn
  const int grid = m.ntc20tiles < m.nsm * O::kPerSm ? m.ntc20tiles : m.nsm * O::kPerSm;
  k_tangent_tc_hex20<kBF16, kSplit><<<grid, kThreads, O::kSmem, s>>>(a, m.tc20tiles, m.ntc20tiles, tc_timeout);
  return cudaGetLastError();
}

template <bool kBF16, bool kSplit>
constexpr bool fits() {
  using O = Op<kBF16, kSplit>;
  return O::kPerSm * (O::kSmem + (int)sizeof(Tc20Static)) <= 226 * 1024 && O::kOffA % 16 == 0 &&
         O::kOffIn % 16 == 0 && (kRowsLive * (NN + 1) + 12 * NN) * 4 <= O::kOpA;
}
static_assert(fits<false, false>() && fits<false, true>() && fits<true, false>() && fits<true, true>(),
              "shared memory: operands, staging and CTAs per SM; the epilogue scratch in the A operand");
static_assert(UT * 4 <= 8 * 1024, "Ke staging");

}  // namespace

cudaError_t init_tangent_tc20_kernels() {
  cudaError_t e = set_attr20<false, false>();
  if (e == cudaSuccess) e = set_attr20<false, true>();
  if (e == cudaSuccess) e = set_attr20<true, false>();
  return e == cudaSuccess ? set_attr20<true, true>() : e;
}

// BF16 requests split the constant N_A (hi + lo, two MMAs per k-step) and
// round Y once: with N_A rounded once as well (Ke error ~2e-3, the same
// operator error in every element) the Newton solve of the mixed
// hex8/hex20/tet10 bars diverged and met an indefinite K_ff in its first
// step. TF32 rounds both once (the FP32 tangent's iterations on the same
// problem; a split N_A would leave room for one CTA per SM only).
cudaError_t launch_tangent_tc_hex20(const DeviceModel& m, const TangentArgs& a, bool bf16, bool split,
                                    int* tc_timeout, cudaStream_t s) {
  if (m.ntc20tiles == 0) return cudaSuccess;
  if (bf16) return split ? launch20<true, true>(m, a, tc_timeout, s) : launch20<true, false>(m, a, tc_timeout, s);
  return split ? launch20<false, true>(m, a, tc_timeout, s) : launch20<false, false>(m, a, tc_timeout, s);
}

}  // namespace w3g
