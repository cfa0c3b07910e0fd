// w3g_noalloc.cu -- internal-force assembly for callers that cannot
// allocate device memory.
//
// Some host codes that would call this library never call cudaMalloc
// themselves: a Fortran solver whose device arrays come from a memory
// pool or from CUDA Fortran managed declarations owned elsewhere, or a
// code that runs with device allocation forbidden after start-up (a
// fixed memory budget, a context shared with a framework that owns the
// allocator). Such a caller already holds its element internal forces
// and dof map on the device and wants the nodal vector, without a
// w3g_context (whose creation allocates the resident element state).
//
// w3g_assemble_ifv_noalloc scatters einfvec into ifv and sums |einfvec|
// (WARP3D's addifv, src/addifv.f:86-124) using only the caller's arrays
// plus one fixed scratch array that lives in this file: a file-scope
// static __device__ array (the block table and the per-block partial
// sums). It calls no cudaMalloc/cudaFree and no allocating library.
//
//   * the scratch array holds at most W3G_NOALLOC_MAX_BLOCKS blocks; a
//     larger model is rejected with W3G_EARG and a message;
//   * every GPU that loads the library holds the array (a few MB) until
//     the process exits;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress, with that device current) and caches it:
//     make that first call before any stream capture;
//   * all calls share the one array and it keeps the last call's
//     contents: calls whose work overlaps on the GPU (different streams
//     or threads without ordering) race on it and must be serialised by
//     the caller. The entry point rewrites every entry it reads and
//     clears the bad-index record first; ifv is zeroed by the call;
//   * every call copies the caller's tables from host memory and waits
//     for its work, so it must not be called while its stream is being
//     captured into a graph (it refuses with W3G_EARG);
//   * the cached address belongs to the device's primary context: after
//     cudaDeviceReset on that device it is stale, and the process must
//     not call this entry point on that device again;
//   * edest entries outside 1..nodof are skipped (no write outside ifv)
//     and the call returns W3G_EARG naming the first block holding one.
#include <climits>
#include <mutex>
#include <string>
#include <cuda_runtime.h>
#include "w3g_internal.cuh"

namespace {

constexpr int kMaxBlocks = W3G_NOALLOC_MAX_BLOCKS;
constexpr int kThreads = 256;

// the caller's elblks and totdof tables, the derived einfvec offsets and
// the per-block partial sums of |einfvec|
struct NoallocScratch {
  int elblks[3 * kMaxBlocks];
  int totdof[kMaxBlocks];
  long long einf_off[kMaxBlocks];
  double partial[kMaxBlocks];
  int bad_block;      // smallest 0-based block with an edest entry outside 1..nodof, or INT_MAX
};

static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

// device address of g_noalloc_scratch per device, looked up once
std::mutex g_mu;
NoallocScratch* g_addr[64] = {};

// zeroes ifv and clears the bad-index record of the previous call
__global__ void k_zero(double* v, int n, NoallocScratch* s) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) v[k] = 0.0;
  if (k == 0) s->bad_block = INT_MAX;
}

// einfvec offset of every block: exclusive prefix sum of span*totdof
__global__ void __launch_bounds__(kThreads) k_offsets(NoallocScratch* s, int nelblk) {
  __shared__ long long part[kThreads];
  const int per = (nelblk + kThreads - 1) / kThreads;
  const int b0 = threadIdx.x * per, b1 = min(nelblk, b0 + per);
  long long t = 0;
  for (int b = b0; b < b1; ++b) t += (long long)s->elblks[3 * b] * s->totdof[b];
  part[threadIdx.x] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long run = 0;
    for (int k = 0; k < kThreads; ++k) { long long v = part[k]; part[k] = run; run += v; }
  }
  __syncthreads();
  long long run = part[threadIdx.x];
  for (int b = b0; b < b1; ++b) {
    s->einf_off[b] = run;
    run += (long long)s->elblks[3 * b] * s->totdof[b];
  }
}

// one CTA per element block; OpenMP-ATOMIC-style scatter as addifv does
__global__ void __launch_bounds__(kThreads) k_scatter(NoallocScratch* s, const double* __restrict__ einf,
                                                      const int* __restrict__ edest, double* ifv, int nodof) {
  __shared__ double sw[kThreads / 32];
  const int b = blockIdx.x;
  const int span = s->elblks[3 * b], totdof = s->totdof[b];
  const long long off = s->einf_off[b];
  double sa = 0.0;
  const int n = span * totdof;
  for (int k = threadIdx.x; k < n; k += kThreads) {
    const int i = k % span;            // einfvec (span, totdof): k = j*span + i
    const int j = k / span;
    const double v = einf[off + k];
    const int dof = edest[off + (long long)i * totdof + j];
    if (dof >= 1 && dof <= nodof) atomicAdd(&ifv[dof - 1], v);
    else atomicMin(&s->bad_block, b);   // skipped: never written outside ifv
    sa += fabs(v);
  }
  for (int o = 16; o > 0; o >>= 1) sa += __shfl_xor_sync(0xffffffffu, sa, o);
  if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = sa;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) t += sw[w];
    s->partial[b] = t;
  }
}

__global__ void k_sum_partials(const NoallocScratch* s, int nelblk, double* out) {
  __shared__ double red[kThreads];
  double t = 0.0;
  for (int b = threadIdx.x; b < nelblk; b += kThreads) t += s->partial[b];
  red[threadIdx.x] = t;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

int fail(int code, const std::string& msg) {
  w3g::set_last_error("w3g_assemble_ifv_noalloc: " + msg);
  return code;
}

}  // namespace

extern "C" int w3g_assemble_ifv_noalloc(int nelblk, const int* elblks, const int* totdof, int nodof,
                                        const double* d_einfvec, const int* d_edest, double* d_ifv,
                                        double* d_sum_ifv, void* stream) {
  if (nelblk < 1 || !elblks || !totdof || nodof < 1 || !d_einfvec || !d_edest || !d_ifv || !d_sum_ifv) {
    return fail(W3G_EARG, "null or empty argument");
  }
  if (nelblk > kMaxBlocks) {
    return fail(W3G_EARG, std::to_string(nelblk) + " element blocks exceed the fixed scratch of " +
                              std::to_string(kMaxBlocks) + " blocks");
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
      return fail(W3G_EARG, "called while the stream is being captured (the call copies host tables and waits)");
    }
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    return fail(W3G_ECUDA, "no current CUDA device");
  }
  NoallocScratch* s = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {   // once per device, with that device current
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) {
        return fail(W3G_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      }
      g_addr[dev] = static_cast<NoallocScratch*>(p);
    }
    s = g_addr[dev];
  }
  // check the caller's tables, then copy them into the scratch array
  for (int b = 0; b < nelblk; ++b) {
    if (elblks[3 * b] < 1 || elblks[3 * b] > W3G_MXVL || totdof[b] < 1 || totdof[b] > 3 * 27) {
      return fail(W3G_EARG, "bad span or totdof in block " + std::to_string(b + 1));
    }
  }
  cudaError_t e = cudaMemcpyAsync(s->elblks, elblks, sizeof(int) * 3 * nelblk, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(s->totdof, totdof, sizeof(int) * nelblk, cudaMemcpyHostToDevice, st);
  int bad = INT_MAX;
  if (e == cudaSuccess) {
    k_offsets<<<1, kThreads, 0, st>>>(s, nelblk);
    k_zero<<<(nodof + kThreads - 1) / kThreads, kThreads, 0, st>>>(d_ifv, nodof, s);
    k_scatter<<<nelblk, kThreads, 0, st>>>(s, d_einfvec, d_edest, d_ifv, nodof);
    k_sum_partials<<<1, kThreads, 0, st>>>(s, nelblk, d_sum_ifv);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, &s->bad_block, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    return fail(W3G_ECUDA, cudaGetErrorString(e));
  }
  if (bad != INT_MAX) {
    return fail(W3G_EARG, "edest entry outside 1.." + std::to_string(nodof) + " in block " + std::to_string(bad + 1) +
                              " (skipped; ifv lacks those contributions)");
  }
  return 0;
}
