// w3g_solve.cu -- the global stiffness on the device and its solve.
//
// WARP3D assembles its equilibrium equations row by row from the element
// stiffnesses (drive_assemble_solve, src/drive_assemble_solve.f:654-929;
// assem_by_row / assem_a_row, src/assemble_code.f:659,785) after building
// the sparsity once (ds_setup_sparsity_local, :358), then calls a sparse
// solver. Here:
//
//   pattern   built once on the host from edest: for every equation row,
//             the (column, element-stiffness index) contributions of the
//             elements sharing the row's dof, in ascending element-vector
//             order, sorted stably by column; rows split over host threads
//   assembly  one thread per stored coefficient sums its contributions in
//             that fixed order from the resident element stiffnesses (FP64,
//             or FP32 under the precision forms): no atomics, bitwise
//             reproducible. Traffic per launch: the contribution indices
//             (4 B each), the element stiffness values they name, and the
//             coefficients (8 B each)
//   PCG       preconditioned conjugate gradient on the free dofs (the
//             inverse 3x3 diagonal block of each node, or the diagonal),
//             five kernels per iteration (SpMV with the p.Kp partial: a
//             warp per node when the three rows of every node share their
//             column pattern, else a warp per row; alpha; vector update
//             with the r.z and r.r partials,
//             beta and the stopping test, direction update) reading the
//             scalars from device memory; a batch of iterations replays as
//             one CUDA graph and the host reads the state between batches.
//             Reductions go through per-CTA partials over a fixed grid,
//             summed in a fixed order: the same inputs give the same
//             iterates bit for bit.
#include <algorithm>
#include <climits>
#include <cstring>
#include <string>
#include <thread>
#include <utility>
#include <vector>
#include "w3g_context.cuh"

using namespace w3g;

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kBatch = 16;   // CG iterations per graph replay

struct PcgScal {
  double rz, pap, alpha, beta, rr, bb, tol2;
  int done, iters, breakdown;
};

__device__ __forceinline__ double warp_sum_down(double v) {
  // tree towards lane 0 (fixed association: deterministic)
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// block sum of one value per thread, fixed order; result valid in thread 0
__device__ __forceinline__ double block_sum(double v, double* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_sum_down(v);
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < kWarps; ++k) t += sh[k];
  __syncthreads();
  return t;
}

// sum of nparts partials (stride `stride`, offset `off`) by one block
__device__ double sum_partials(const double* partials, int nparts, int stride, int off, double* sh) {
  double v = 0.0;
  for (int k = threadIdx.x; k < nparts; k += blockDim.x) v += partials[(size_t)k * stride + off];
  return block_sum(v, sh);
}

template <class T>
__global__ void __launch_bounds__(kThreads) k_assemble(long long nnz, const int* __restrict__ cptr,
                                                       const int* __restrict__ csrc, const T* __restrict__ est,
                                                       double* __restrict__ val) {
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < nnz;
       j += (long long)gridDim.x * blockDim.x) {
    // contributions in their fixed order, four gathers in flight at a time
    double s = 0.0;
    const int e = cptr[j + 1];
    for (int k = cptr[j]; k < e; k += 4) {
      int idx[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) idx[u] = k + u < e ? csrc[k + u] : -1;
      double v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = idx[u] >= 0 ? (double)est[idx[u]] : 0.0;
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (idx[u] >= 0) s += v[u];
    }
    val[j] = s;
  }
}

__global__ void __launch_bounds__(kThreads) k_dinv(int n, const int* __restrict__ diag,
                                                   const double* __restrict__ val,
                                                   const unsigned char* __restrict__ fixed, double* dinv) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double d = val[diag[i]];
    dinv[i] = (fixed[i] || d == 0.0) ? 0.0 : 1.0 / d;
  }
}

// Node-block Jacobi (three rows of a node sharing their pattern): the
// inverse of each node's 3x3 diagonal block over its free dofs (a
// constrained dof's row and column are the identity's, its entries of the
// inverse zero). A block that is not positive (det <= 0 or not finite)
// falls back to the scalar diagonal.
__global__ void __launch_bounds__(kThreads) k_binv(int nn, const int* __restrict__ diag,
                                                   const double* __restrict__ val,
                                                   const unsigned char* __restrict__ fixed, double* binv) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    double M[9];
    bool f[3];
    for (int i = 0; i < 3; ++i) f[i] = fixed[3 * k + i] != 0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        M[3 * i + j] = (f[i] || f[j]) ? (i == j ? 1.0 : 0.0) : val[diag[3 * k + i] + (j - i)];
    const double c0 = M[4] * M[8] - M[5] * M[7], c1 = M[5] * M[6] - M[3] * M[8], c2 = M[3] * M[7] - M[4] * M[6];
    const double det = M[0] * c0 + M[1] * c1 + M[2] * c2;
    double* B = binv + 9 * (long long)k;
    if (det > 0.0 && isfinite(det)) {
      const double r = 1.0 / det;
      B[0] = c0 * r;
      B[1] = (M[2] * M[7] - M[1] * M[8]) * r;
      B[2] = (M[1] * M[5] - M[2] * M[4]) * r;
      B[3] = c1 * r;
      B[4] = (M[0] * M[8] - M[2] * M[6]) * r;
      B[5] = (M[2] * M[3] - M[0] * M[5]) * r;
      B[6] = c2 * r;
      B[7] = (M[1] * M[6] - M[0] * M[7]) * r;
      B[8] = (M[0] * M[4] - M[1] * M[3]) * r;
    } else {
      for (int q = 0; q < 9; ++q) B[q] = 0.0;
      for (int i = 0; i < 3; ++i) B[4 * i] = (M[4 * i] != 0.0) ? 1.0 / M[4 * i] : 0.0;
    }
    for (int i = 0; i < 3; ++i)
      if (f[i])
        for (int j = 0; j < 3; ++j) B[3 * i + j] = B[3 * j + i] = 0.0;
  }
}

// z = B^-1 r for one node (3 dofs)
__device__ __forceinline__ void apply_binv(const double* B, const double* r, double* z) {
  z[0] = B[0] * r[0] + B[1] * r[1] + B[2] * r[2];
  z[1] = B[3] * r[0] + B[4] * r[1] + B[5] * r[2];
  z[2] = B[6] * r[0] + B[7] * r[1] + B[8] * r[2];
}

__global__ void __launch_bounds__(kThreads) k_pcg_init3(int nn, const unsigned char* __restrict__ fixed,
                                                        const double* __restrict__ b, double bscale,
                                                        const double* __restrict__ binv, double* x, double* r,
                                                        double* z, double* p, double* partials) {
  __shared__ double sh[kWarps];
  double rz = 0.0, rr = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    double rk[3], zk[3];
    for (int i = 0; i < 3; ++i) rk[i] = fixed[3 * k + i] ? 0.0 : bscale * b[3 * k + i];
    apply_binv(binv + 9 * (long long)k, rk, zk);
    for (int i = 0; i < 3; ++i) {
      x[3 * k + i] = 0.0;
      r[3 * k + i] = rk[i];
      z[3 * k + i] = zk[i];
      p[3 * k + i] = zk[i];
      rz += rk[i] * zk[i];
      rr += rk[i] * rk[i];
    }
  }
  rz = block_sum(rz, sh);
  rr = block_sum(rr, sh);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = rz;
    partials[2 * blockIdx.x + 1] = rr;
  }
}

__global__ void __launch_bounds__(kThreads) k_update3(int nn, const double* __restrict__ binv, double* x, double* r,
                                                      double* z, const double* __restrict__ p,
                                                      const double* __restrict__ q, double* partials,
                                                      const PcgScal* sc) {
  __shared__ double sh[kWarps];
  if (sc->done) return;
  const double a = sc->alpha;
  double rz = 0.0, rr = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    double rk[3], zk[3];
    for (int i = 0; i < 3; ++i) {
      const int d = 3 * k + i;
      x[d] += a * p[d];
      rk[i] = r[d] - a * q[d];
      r[d] = rk[i];
    }
    apply_binv(binv + 9 * (long long)k, rk, zk);
    for (int i = 0; i < 3; ++i) {
      z[3 * k + i] = zk[i];
      rz += rk[i] * zk[i];
      rr += rk[i] * rk[i];
    }
  }
  rz = block_sum(rz, sh);
  rr = block_sum(rr, sh);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = rz;
    partials[2 * blockIdx.x + 1] = rr;
  }
}

__global__ void __launch_bounds__(kThreads) k_pcg_init(int n, const unsigned char* __restrict__ fixed,
                                                       const double* __restrict__ b, double bscale,
                                                       const double* __restrict__ dinv, double* x, double* r,
                                                       double* z, double* p, double* partials) {
  __shared__ double sh[kWarps];
  double rz = 0.0, rr = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double ri = fixed[i] ? 0.0 : bscale * b[i];
    const double zi = dinv[i] * ri;
    x[i] = 0.0;
    r[i] = ri;
    z[i] = zi;
    p[i] = zi;
    rz += ri * zi;
    rr += ri * ri;
  }
  rz = block_sum(rz, sh);
  rr = block_sum(rr, sh);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = rz;
    partials[2 * blockIdx.x + 1] = rr;
  }
}

__global__ void __launch_bounds__(kThreads) k_pcg_init_fin(const double* partials, int nparts, double rtol,
                                                           PcgScal* sc) {
  __shared__ double sh[kWarps];
  const double rz = sum_partials(partials, nparts, 2, 0, sh);
  const double rr = sum_partials(partials, nparts, 2, 1, sh);
  if (threadIdx.x == 0) {
    sc->rz = rz;
    sc->rr = rr;
    sc->bb = rr;
    sc->tol2 = rtol * rtol * rr;
    sc->alpha = sc->beta = sc->pap = 0.0;
    sc->iters = 0;
    sc->breakdown = 0;
    sc->done = rr <= sc->tol2 ? 1 : 0;
  }
}

// q = K p on the free rows (0 on constrained rows), partial of p.q
__global__ void __launch_bounds__(kThreads) k_spmv(int n, const int* __restrict__ rowptr,
                                                   const int* __restrict__ colind, const double* __restrict__ val,
                                                   const unsigned char* __restrict__ fixed,
                                                   const double* __restrict__ p, double* __restrict__ q,
                                                   double* partials, const PcgScal* sc) {
  // eight lanes per row, four rows per warp in flight, 32 columns per pass
  // with all loads issued first, fixed-order reduction over the eight lanes
  __shared__ double sh[kWarps];
  if (sc->done) return;
  const int lane = threadIdx.x & 31, sl = lane & 7;
  const int first = (blockIdx.x * kWarps + (threadIdx.x >> 5)) * 4;
  const int ngroups = gridDim.x * kWarps * 4;
  double acc = 0.0;
  for (int base = first; base < n; base += ngroups) {
    const int row = base + (lane >> 3);
    const bool live = row < n;
    const int b = rowptr[live ? row : 0];
    const int len = live ? rowptr[row + 1] - b : 0;
    double s = 0.0;
    for (int kb = 0; kb < len; kb += 32) {
      int c[4];
      bool ok[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = kb + sl + 8 * u;
        ok[u] = k < len;
        c[u] = ok[u] ? colind[b + k] : 0;
      }
      double x[4], v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        x[u] = ok[u] ? p[c[u]] : 0.0;
        v[u] = ok[u] ? val[b + kb + sl + 8 * u] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) s += v[u] * x[u];
    }
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, 8);
    if (live && sl == 0) {
      const double qi = fixed[row] ? 0.0 : s;
      q[row] = qi;
      acc += qi * p[row];
    }
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// the same product when the three rows of each node share one column
// pattern: eight lanes per node (four nodes per warp in flight) read the
// column indices and the gathered direction once for the node's three
// rows, 32 columns per pass with all loads issued first, and reduce over
// their eight lanes in a fixed order
__global__ void __launch_bounds__(kThreads) k_spmv3(int n, const int* __restrict__ rowptr,
                                                    const int* __restrict__ colind, const double* __restrict__ val,
                                                    const unsigned char* __restrict__ fixed,
                                                    const double* __restrict__ p, double* __restrict__ q,
                                                    double* partials, const PcgScal* sc) {
  __shared__ double sh[kWarps];
  if (sc->done) return;
  const int lane = threadIdx.x & 31, sl = lane & 7;
  const int group = (blockIdx.x * kWarps + (threadIdx.x >> 5)) * 4 + (lane >> 3);
  const int ngroups = gridDim.x * kWarps * 4;
  const int nn = n / 3;
  double acc = 0.0;
  // every lane of a warp runs the same number of passes (shuffles need the
  // whole warp): the loop bound is the warp's largest node index
  const int first = group - (lane >> 3);
  for (int base = first; base < nn; base += ngroups) {
    const int node = base + (lane >> 3);
    const bool live = node < nn;
    const int r0 = 3 * (live ? node : 0);
    const int b0 = rowptr[r0], b1 = rowptr[r0 + 1], b2 = rowptr[r0 + 2];
    const int len = live ? b1 - b0 : 0;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int kb = 0; kb < len; kb += 32) {
      int c[4];
      bool ok[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = kb + sl + 8 * u;
        ok[u] = k < len;
        c[u] = ok[u] ? colind[b0 + k] : 0;
      }
      double x[4], v0[4], v1[4], v2[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = kb + sl + 8 * u;
        x[u] = ok[u] ? p[c[u]] : 0.0;
        v0[u] = ok[u] ? val[b0 + k] : 0.0;
        v1[u] = ok[u] ? val[b1 + k] : 0.0;
        v2[u] = ok[u] ? val[b2 + k] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        s0 += v0[u] * x[u];
        s1 += v1[u] * x[u];
        s2 += v2[u] * x[u];
      }
    }
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) {
      s0 += __shfl_down_sync(0xffffffffu, s0, o, 8);
      s1 += __shfl_down_sync(0xffffffffu, s1, o, 8);
      s2 += __shfl_down_sync(0xffffffffu, s2, o, 8);
    }
    if (live && sl == 0) {
      const double q0 = fixed[r0] ? 0.0 : s0, q1 = fixed[r0 + 1] ? 0.0 : s1, q2 = fixed[r0 + 2] ? 0.0 : s2;
      q[r0] = q0;
      q[r0 + 1] = q1;
      q[r0 + 2] = q2;
      acc += q0 * p[r0];
      acc += q1 * p[r0 + 1];
      acc += q2 * p[r0 + 2];
    }
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

__global__ void __launch_bounds__(kThreads) k_alpha(const double* partials, int nparts, PcgScal* sc) {
  __shared__ double sh[kWarps];
  if (sc->done) return;
  const double pap = sum_partials(partials, nparts, 1, 0, sh);
  if (threadIdx.x == 0) {
    sc->pap = pap;
    if (!(pap > 0.0) || !isfinite(pap)) {
      sc->alpha = 0.0;
      sc->breakdown = 1;
      sc->done = 1;
    } else {
      sc->alpha = sc->rz / pap;
    }
  }
}

__global__ void __launch_bounds__(kThreads) k_update(int n, const double* __restrict__ dinv, double* x, double* r,
                                                     double* z, const double* __restrict__ p,
                                                     const double* __restrict__ q, double* partials,
                                                     const PcgScal* sc) {
  __shared__ double sh[kWarps];
  if (sc->done) return;
  const double a = sc->alpha;
  double rz = 0.0, rr = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] += a * p[i];
    const double ri = r[i] - a * q[i];
    const double zi = dinv[i] * ri;
    r[i] = ri;
    z[i] = zi;
    rz += ri * zi;
    rr += ri * ri;
  }
  rz = block_sum(rz, sh);
  rr = block_sum(rr, sh);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = rz;
    partials[2 * blockIdx.x + 1] = rr;
  }
}

__global__ void __launch_bounds__(kThreads) k_beta(const double* partials, int nparts, PcgScal* sc) {
  __shared__ double sh[kWarps];
  if (sc->done) return;
  const double rz = sum_partials(partials, nparts, 2, 0, sh);
  const double rr = sum_partials(partials, nparts, 2, 1, sh);
  if (threadIdx.x == 0) {
    sc->iters += 1;
    sc->beta = sc->rz != 0.0 ? rz / sc->rz : 0.0;
    sc->rz = rz;
    sc->rr = rr;
    if (rr <= sc->tol2 || !isfinite(rr)) sc->done = 1;
  }
}

__global__ void __launch_bounds__(kThreads) k_pupdate(int n, const double* __restrict__ z, double* p,
                                                      const PcgScal* sc) {
  if (sc->done) return;
  const double bt = sc->beta;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = z[i] + bt * p[i];
}

__global__ void __launch_bounds__(kThreads) k_norms(int n, const double* __restrict__ v,
                                                    const unsigned char* __restrict__ fixed, double* partials) {
  __shared__ double sh[kWarps];
  double f = 0.0, a = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double vi = v[i];
    a += vi * vi;
    if (!fixed[i]) f += vi * vi;
  }
  f = block_sum(f, sh);
  a = block_sum(a, sh);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = f;
    partials[2 * blockIdx.x + 1] = a;
  }
}

__global__ void __launch_bounds__(kThreads) k_norms_fin(const double* partials, int nparts, double* out) {
  __shared__ double sh[kWarps];
  const double f = sum_partials(partials, nparts, 2, 0, sh);
  const double a = sum_partials(partials, nparts, 2, 1, sh);
  if (threadIdx.x == 0) {
    out[0] = f;
    out[1] = a;
  }
}

// sum over the free dofs of a_i b_i: the line search's s-value of mnralg_ls
// (s = -sum res idu, src/mnralg.f:1135-1158) with a = -res; per-CTA partials
// in a fixed order
__global__ void __launch_bounds__(kThreads) k_dot_free(int n, const double* __restrict__ a,
                                                       const double* __restrict__ b,
                                                       const unsigned char* __restrict__ fixed, double* partials) {
  __shared__ double sh[kWarps];
  double t = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (!fixed[i]) t += a[i] * b[i];
  t = block_sum(t, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

__global__ void __launch_bounds__(kThreads) k_dot_fin(const double* partials, int nparts, double* out) {
  __shared__ double sh[kWarps];
  const double t = sum_partials(partials, nparts, 1, 0, sh);
  if (threadIdx.x == 0) out[0] = t;
}

// ---- one Newton iteration as one graph (w3g_newton_iteration_dev) ----
// the solve's tolerance and iteration limit, written before each launch
struct NewtonParams {
  double rtol;
  int maxit, pad;
};

// k_pcg_init_fin with the tolerance read from the device
__global__ void __launch_bounds__(kThreads) k_pcg_init_fin_p(const double* partials, int nparts,
                                                             const NewtonParams* prm, PcgScal* sc) {
  __shared__ double sh[kWarps];
  const double rz = sum_partials(partials, nparts, 2, 0, sh);
  const double rr = sum_partials(partials, nparts, 2, 1, sh);
  if (threadIdx.x == 0) {
    const double rtol = prm->rtol;
    sc->rz = rz;
    sc->rr = rr;
    sc->bb = rr;
    sc->tol2 = rtol * rtol * rr;
    sc->alpha = sc->beta = sc->pap = 0.0;
    sc->iters = 0;
    sc->breakdown = 0;
    sc->done = rr <= sc->tol2 ? 1 : 0;
  }
}

// the loop condition of the device-side CG loop: another batch while the
// solve is neither converged nor broken down and below the iteration limit
// (every batch that runs advances iters, so the loop ends)
__global__ void k_pcg_cond(const PcgScal* sc, const NewtonParams* prm, cudaGraphConditionalHandle h) {
  cudaGraphSetConditional(h, (!sc->done && sc->iters < prm->maxit) ? 1u : 0u);
}

__global__ void __launch_bounds__(kThreads) k_add(int n, const double* __restrict__ x, double* __restrict__ y) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] += x[i];
}

// the pinned host side of one launch: parameters in, scalars out
struct NewtonHost {
  NewtonParams prm;
  PcgScal sc;
  w3g_recover_info info;
  double norms[2];
};

// what the Newton-iteration graph was built for
struct NewtonKey {
  const void *c = nullptr, *u = nullptr, *du = nullptr, *ifv = nullptr, *fixed = nullptr, *d = nullptr,
             *norms = nullptr;
  int precision = -1;
  w3g::Schedule sched{};
  long long wait_limit = 0;
  bool triplet = false;
};

}  // namespace

struct w3g_csr {
  w3g_context* ctx = nullptr;
  int n = 0;
  long long nnz = 0, ncontrib = 0;
  int *rowptr = nullptr, *colind = nullptr, *diag = nullptr, *cptr = nullptr, *csrc = nullptr;
  double* val = nullptr;
  // PCG work
  int grid = 0;
  int grid_spmv = 0;      // resident CTAs of the node matrix-product kernel (one wave)
  int grid_spmv_rows = 0; // ... of the row kernel
  bool triplet = false;   // node kernels in use (w3g_csr_set_node_blocks)
  bool pattern_triplet = false;   // dofs 3k..3k+2 of every node share their column pattern
  double* binv = nullptr;  // node-block Jacobi inverses (triplet patterns)
  double *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *dinv = nullptr;
  double* partials = nullptr;
  PcgScal* sc = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  cudaGraphExec_t batch = nullptr;
  const void* graph_fixed = nullptr;   // mask the batch graph was captured with
  // one Newton iteration as one graph
  cudaGraphExec_t newton = nullptr;
  NewtonKey newton_key;
  cudaStream_t stream2 = nullptr;      // captures the CG loop body
  NewtonParams* d_prm = nullptr;
  NewtonHost* h_newton = nullptr;      // pinned
};

namespace {

#define CKS(call)                                                                    \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess)                                                           \
      return w3g_fail(W3G_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

void csr_free(w3g_csr* m) {
  if (m->batch) cudaGraphExecDestroy(m->batch);
  if (m->newton) cudaGraphExecDestroy(m->newton);
  if (m->stream2) cudaStreamDestroy(m->stream2);
  if (m->d_prm) cudaFree(m->d_prm);
  if (m->h_newton) cudaFreeHost(m->h_newton);
  void* ptrs[] = {m->rowptr, m->colind, m->diag, m->cptr, m->csrc, m->val, m->x, m->r, m->z, m->p, m->q,
                  m->dinv, m->binv, m->partials, m->sc};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (m->ev_in) cudaEventDestroy(m->ev_in);
  if (m->ev_out) cudaEventDestroy(m->ev_out);
  if (m->stream) cudaStreamDestroy(m->stream);
}

// the CG set-up of w3g_pcg_dev (preconditioner, x = 0, r, z, p, partials)
void enqueue_pcg_init(w3g_csr* s, const unsigned char* fixed, const double* b, double b_scale, cudaStream_t st) {
  const int n = s->n, G = s->grid;
  if (s->triplet) {
    k_binv<<<G, kThreads, 0, st>>>(n / 3, s->diag, s->val, fixed, s->binv);
    k_pcg_init3<<<G, kThreads, 0, st>>>(n / 3, fixed, b, b_scale, s->binv, s->x, s->r, s->z, s->p, s->partials);
  } else {
    k_dinv<<<G, kThreads, 0, st>>>(n, s->diag, s->val, fixed, s->dinv);
    k_pcg_init<<<G, kThreads, 0, st>>>(n, fixed, b, b_scale, s->dinv, s->x, s->r, s->z, s->p, s->partials);
  }
}

// `count` CG iterations (each a no-op once the solve is done)
void enqueue_pcg_iterations(w3g_csr* s, const unsigned char* fixed, int count, cudaStream_t st) {
  const int n = s->n, G = s->grid;
  for (int it = 0; it < count; ++it) {
    const int GS = s->triplet ? s->grid_spmv : s->grid_spmv_rows;
    if (s->triplet)
      k_spmv3<<<GS, kThreads, 0, st>>>(n, s->rowptr, s->colind, s->val, fixed, s->p, s->q, s->partials, s->sc);
    else
      k_spmv<<<GS, kThreads, 0, st>>>(n, s->rowptr, s->colind, s->val, fixed, s->p, s->q, s->partials, s->sc);
    k_alpha<<<1, kThreads, 0, st>>>(s->partials, GS, s->sc);
    if (s->triplet)
      k_update3<<<G, kThreads, 0, st>>>(n / 3, s->binv, s->x, s->r, s->z, s->p, s->q, s->partials, s->sc);
    else
      k_update<<<G, kThreads, 0, st>>>(n, s->dinv, s->x, s->r, s->z, s->p, s->q, s->partials, s->sc);
    k_beta<<<1, kThreads, 0, st>>>(s->partials, G, s->sc);
    k_pupdate<<<G, kThreads, 0, st>>>(n, s->z, s->p, s->sc);
  }
}

// the part of the pattern built by one host thread: rows [r0, r1)
struct RowsPart {
  int r0 = 0, r1 = 0;
  std::vector<int> row_nnz, diag_rel, col, cnt, src;
};

// block holding element-vector entry `e` (blocks are in einf_off order)
int block_of(const std::vector<BlockDesc>& B, long long e) {
  int lo = 0, hi = (int)B.size() - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (B[mid].einf_off <= e) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

void build_rows(const std::vector<BlockDesc>& B, const std::vector<int>& ed, const std::vector<int>& ifv_ptr,
                const std::vector<long long>& ifv_src, RowsPart& P) {
  std::vector<std::pair<int, int>> pr;   // (column, element-stiffness index)
  for (int g = P.r0; g < P.r1; ++g) {
    pr.clear();
    for (int k = ifv_ptr[g]; k < ifv_ptr[g + 1]; ++k) {
      // ifv_src entries ascend in element-vector order: block, dof, element
      const long long e = ifv_src[k];
      const BlockDesc& d = B[block_of(B, e)];
      const long long rel = e - d.einf_off;
      const int r = (int)(rel / d.span), i = (int)(rel % d.span);
      const int* dofs = &ed[d.einf_off + (size_t)i * d.totdof];
      const long long base = d.estiff_off + (long long)i * d.utsz;
      for (int c = 0; c < d.totdof; ++c) {
        const int lo = std::min(r, c), hi = std::max(r, c);
        pr.emplace_back(dofs[c] - 1, (int)(base + (long long)hi * (hi + 1) / 2 + lo));
      }
    }
    if (pr.empty()) {   // a dof no element touches: an empty coefficient on the diagonal
      P.col.push_back(g);
      P.cnt.push_back(0);
      P.row_nnz.push_back(1);
      P.diag_rel.push_back(0);
      continue;
    }
    std::stable_sort(pr.begin(), pr.end(),
                     [](const std::pair<int, int>& a, const std::pair<int, int>& b) { return a.first < b.first; });
    int nz = 0, drel = -1;
    for (size_t k = 0; k < pr.size(); ++k) {
      if (k == 0 || pr[k].first != pr[k - 1].first) {
        if (pr[k].first == g) drel = nz;
        P.col.push_back(pr[k].first);
        P.cnt.push_back(0);
        ++nz;
      }
      P.cnt.back()++;
      P.src.push_back(pr[k].second);
    }
    P.row_nnz.push_back(nz);
    P.diag_rel.push_back(drel);
  }
}

int grid_for(int device) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  return std::max(1, sms) * 8;
}

}  // namespace

namespace {

// The Newton-iteration graph: the CG solve of K d = -ifv as a device-side
// loop (a conditional while node over batches of kBatch iterations, the
// condition set by k_pcg_cond: no host round trip per batch), then d = x,
// du += d, the element work of the next iteration (recovery at du, then the
// tangent; the caller launches k_begin_recover before the graph), the
// assembly of K and the residual norms.
int build_newton_graph(w3g_csr* s, const NewtonKey& k) {
  w3g_context* c = s->ctx;
  if (!s->stream2) CKS(cudaStreamCreateWithFlags(&s->stream2, cudaStreamNonBlocking));
  if (!s->d_prm) CKS(cudaMalloc(&s->d_prm, sizeof(NewtonParams)));
  if (!s->h_newton) CKS(cudaMallocHost(&s->h_newton, sizeof(NewtonHost)));
  if (s->newton) {
    CKS(cudaGraphExecDestroy(s->newton));
    s->newton = nullptr;
  }
  const int n = s->n, G = s->grid;
  const unsigned char* fixed = (const unsigned char*)k.fixed;
  cudaStream_t cs = s->stream;
  CKS(cudaStreamSynchronize(cs));
  CKS(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
  cudaStreamCaptureStatus cst;
  cudaGraph_t g = nullptr;
  cudaGraphConditionalHandle h = 0;
  cudaError_t e = cudaStreamGetCaptureInfo(cs, &cst, nullptr, &g, nullptr, nullptr, nullptr);
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, g, 0, 0);
  if (e == cudaSuccess) {
    enqueue_pcg_init(s, fixed, (const double*)k.ifv, -1.0, cs);
    k_pcg_init_fin_p<<<1, kThreads, 0, cs>>>(s->partials, G, s->d_prm, s->sc);
    k_pcg_cond<<<1, 1, 0, cs>>>(s->sc, s->d_prm, h);
    e = cudaGetLastError();
  }
  // the loop node after what is captured so far; capture continues after it
  cudaGraphNode_t wnode = nullptr;
  cudaGraph_t body = nullptr;
  if (e == cudaSuccess) {
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    e = cudaStreamGetCaptureInfo(cs, &cst, nullptr, nullptr, &deps, nullptr, &nd);
    if (e == cudaSuccess) {
      cudaGraphNodeParams prm{};
      prm.type = cudaGraphNodeTypeConditional;
      prm.conditional.handle = h;
      prm.conditional.type = cudaGraphCondTypeWhile;
      prm.conditional.size = 1;
      e = cudaGraphAddNode(&wnode, g, deps, nullptr, nd, &prm);
      if (e == cudaSuccess) body = prm.conditional.phGraph_out[0];
    }
  }
  if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(cs, &wnode, nullptr, 1, cudaStreamSetCaptureDependencies);
  // the loop body, captured into the node's graph from the second stream
  if (e == cudaSuccess)
    e = cudaStreamBeginCaptureToGraph(s->stream2, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    enqueue_pcg_iterations(s, fixed, kBatch, s->stream2);
    k_pcg_cond<<<1, 1, 0, s->stream2>>>(s->sc, s->d_prm, h);
    e = cudaGetLastError();
    cudaGraph_t bo = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(s->stream2, &bo);
    if (e == cudaSuccess) e = e2;
  }
  int nel = 0;
  if (e == cudaSuccess) {
    e = cudaMemcpyAsync((void*)k.d, s->x, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, cs);
    k_add<<<G, kThreads, 0, cs>>>(n, s->x, (double*)k.du);
    nel = w3g::enqueue_element_iteration(c, W3G_ITER_RECOVER | W3G_ITER_TANGENT, (const double*)k.c,
                                         (const double*)k.u, (const double*)k.du, (double*)k.ifv, cs);
    const int grid = (int)std::min<long long>((s->nnz + kThreads - 1) / kThreads, 16LL * G);
    if (c->precision == W3G_TANGENT_FP64)
      k_assemble<double><<<std::max(1, grid), kThreads, 0, cs>>>(s->nnz, s->cptr, s->csrc, c->s.estiff, s->val);
    else
      k_assemble<float><<<std::max(1, grid), kThreads, 0, cs>>>(s->nnz, s->cptr, s->csrc, c->s.estiff32, s->val);
    double* part = s->partials + 2 * (size_t)G;
    k_norms<<<G, kThreads, 0, cs>>>(n, (const double*)k.ifv, fixed, part);
    k_norms_fin<<<1, kThreads, 0, cs>>>(part, G, (double*)k.norms);
    if (e == cudaSuccess) e = cudaGetLastError();
  }
  cudaGraph_t gout = nullptr;
  const cudaError_t ee = cudaStreamEndCapture(cs, &gout);
  if (nel < 0) {
    if (gout) cudaGraphDestroy(gout);
    return nel;   // the element path's own error (message set)
  }
  if (e == cudaSuccess) e = ee;
  if (e == cudaSuccess) e = cudaGraphInstantiate(&s->newton, gout, 0);
  if (gout) cudaGraphDestroy(gout);
  if (e != cudaSuccess) {
    s->newton = nullptr;
    return w3g_fail(W3G_ECUDA, std::string("newton iteration graph: ") + cudaGetErrorString(e));
  }
  s->newton_key = k;
  return 0;
}

bool same_key(const NewtonKey& a, const NewtonKey& b) {
  return a.c == b.c && a.u == b.u && a.du == b.du && a.ifv == b.ifv && a.fixed == b.fixed && a.d == b.d &&
         a.norms == b.norms && a.precision == b.precision && a.wait_limit == b.wait_limit &&
         a.triplet == b.triplet && a.sched.mode == b.sched.mode &&
         a.sched.recover_ctas_per_sm == b.sched.recover_ctas_per_sm &&
         a.sched.tangent_ctas_per_sm == b.sched.tangent_ctas_per_sm &&
         a.sched.recover_grain == b.sched.recover_grain && a.sched.tangent_grain == b.sched.tangent_grain &&
         a.sched.order == b.sched.order;
}

}  // namespace

extern "C" {

int w3g_csr_create(w3g_context* c, w3g_csr** out) {
  if (!c || !out) return w3g_fail(W3G_EARG, "null argument");
  CKS(cudaSetDevice(c->device));
  const DeviceModel& m = c->m;
  const int n = m.nodof;
  if (m.estiff_total >= INT_MAX) return w3g_fail(W3G_EUNSUPPORTED, "element stiffnesses exceed 2^31 values");
  if (m.asym) return w3g_fail(W3G_EUNSUPPORTED, "the device assembly and PCG take symmetric element matrices");
  std::vector<int> ed(m.einf_total);
  std::vector<int> ifv_ptr(n + 1);
  std::vector<long long> ifv_src(m.einf_total);
  CKS(cudaMemcpy(ed.data(), m.edest, ed.size() * sizeof(int), cudaMemcpyDeviceToHost));
  CKS(cudaMemcpy(ifv_ptr.data(), m.ifv_rowptr, ifv_ptr.size() * sizeof(int), cudaMemcpyDeviceToHost));
  CKS(cudaMemcpy(ifv_src.data(), m.ifv_src, ifv_src.size() * sizeof(long long), cudaMemcpyDeviceToHost));

  // rows in parts of similar contribution counts, one host thread each
  const int nthreads = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  std::vector<RowsPart> parts(nthreads);
  {
    const long long total = ifv_ptr[n];
    int r = 0;
    for (int t = 0; t < nthreads; ++t) {
      parts[t].r0 = r;
      const long long target = total * (t + 1) / nthreads;
      while (r < n && (t == nthreads - 1 || ifv_ptr[r] < target)) ++r;
      parts[t].r1 = r;
    }
    parts[nthreads - 1].r1 = n;
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t)
      th.emplace_back(build_rows, std::cref(c->blocks), std::cref(ed), std::cref(ifv_ptr), std::cref(ifv_src),
                      std::ref(parts[t]));
    for (auto& t : th) t.join();
  }
  long long nnz = 0, ncontrib = 0;
  for (const RowsPart& P : parts) {
    nnz += (long long)P.col.size();
    ncontrib += (long long)P.src.size();
  }
  if (nnz >= INT_MAX || ncontrib >= INT_MAX) return w3g_fail(W3G_EUNSUPPORTED, "global stiffness exceeds 2^31 entries");
  for (const RowsPart& P : parts)
    for (int d : P.diag_rel)
      if (d < 0) return w3g_fail(W3G_EARG, "equation row without its diagonal coefficient");

  w3g_csr* s = new w3g_csr;
  s->ctx = c;
  s->n = n;
  s->nnz = nnz;
  s->ncontrib = ncontrib;
  s->grid = grid_for(c->device);
  std::vector<int> rowptr(n + 1), diag(n), cptr(nnz + 1);
  {
    int row = 0;
    long long z = 0, k = 0;
    rowptr[0] = 0;
    for (const RowsPart& P : parts) {
      for (size_t j = 0; j < P.row_nnz.size(); ++j) {
        diag[row] = (int)z + P.diag_rel[j];
        z += P.row_nnz[j];
        rowptr[++row] = (int)z;
      }
    }
    long long zz = 0;
    for (const RowsPart& P : parts)
      for (int cn : P.cnt) {
        cptr[zz++] = (int)k;
        k += cn;
      }
    cptr[nnz] = (int)k;
  }
  // the stored pattern of a node's three rows: identical when every dof
  // belongs to a node of three consecutive dofs (WARP3D's dstmap); the
  // matrix product then reads the column indices and x once per node
  std::vector<int> colind_all;
  colind_all.reserve((size_t)nnz);
  for (const RowsPart& P : parts) colind_all.insert(colind_all.end(), P.col.begin(), P.col.end());
  bool triplet = n % 3 == 0;
  for (int k = 0; triplet && k < n / 3; ++k) {
    const int r0 = 3 * k, len = rowptr[r0 + 1] - rowptr[r0];
    for (int d = 1; d < 3 && triplet; ++d) {
      const int rd = r0 + d;
      if (rowptr[rd + 1] - rowptr[rd] != len ||
          !std::equal(colind_all.begin() + rowptr[r0], colind_all.begin() + rowptr[r0] + len,
                      colind_all.begin() + rowptr[rd]))
        triplet = false;
    }
  }
  s->triplet = triplet;
  s->pattern_triplet = triplet;
  {
    // one wave of the product kernel: its per-CTA partials are summed in a
    // fixed order, so the grid is fixed per matrix
    int per_sm = 0, per_sm_rows = 0, sms = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)k_spmv3, kThreads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_rows, (const void*)k_spmv, kThreads, 0);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    s->grid_spmv = std::max(1, std::min(s->grid, per_sm * sms));
    s->grid_spmv_rows = std::max(1, std::min(s->grid, per_sm_rows * sms));
  }
  cudaError_t e = cudaSuccess;
  auto al = [&](auto** p, size_t count) {
    if (e == cudaSuccess) e = cudaMalloc((void**)p, std::max<size_t>(1, count) * sizeof(**p));
  };
  al(&s->rowptr, n + 1);
  al(&s->colind, nnz);
  al(&s->diag, n);
  al(&s->cptr, nnz + 1);
  al(&s->csrc, ncontrib);
  al(&s->val, nnz);
  al(&s->x, n);
  al(&s->r, n);
  al(&s->z, n);
  al(&s->p, n);
  al(&s->q, n);
  al(&s->dinv, n);
  if (triplet) al(&s->binv, 3 * (size_t)n);
  al(&s->partials, 5 * (size_t)s->grid);   // PCG partials, the norms' partials, the free dot's
  al(&s->sc, 1);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_in, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_out, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMemcpy(s->rowptr, rowptr.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(s->diag, diag.data(), n * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(s->cptr, cptr.data(), (nnz + 1) * sizeof(int), cudaMemcpyHostToDevice);
  long long ko = 0;
  if (e == cudaSuccess) e = cudaMemcpy(s->colind, colind_all.data(), nnz * sizeof(int), cudaMemcpyHostToDevice);
  for (const RowsPart& P : parts) {
    if (e == cudaSuccess && !P.src.empty())
      e = cudaMemcpy(s->csrc + ko, P.src.data(), P.src.size() * sizeof(int), cudaMemcpyHostToDevice);
    ko += (long long)P.src.size();
  }
  if (e == cudaSuccess) e = cudaMemset(s->val, 0, nnz * sizeof(double));
  if (e != cudaSuccess) {
    csr_free(s);
    delete s;
    return w3g_fail(W3G_ECUDA, std::string("w3g_csr_create: ") + cudaGetErrorString(e));
  }
  *out = s;
  return 0;
}

int w3g_csr_destroy(w3g_csr* s) {
  if (!s) return 0;
  cudaSetDevice(s->ctx->device);
  csr_free(s);
  delete s;
  return 0;
}

int w3g_csr_info(w3g_csr* s, int* n, long long* nnz, void** d_rowptr, void** d_colind, void** d_values) {
  if (!s) return w3g_fail(W3G_EARG, "null csr");
  if (n) *n = s->n;
  if (nnz) *nnz = s->nnz;
  if (d_rowptr) *d_rowptr = s->rowptr;
  if (d_colind) *d_colind = s->colind;
  if (d_values) *d_values = s->val;
  return 0;
}

int w3g_csr_assemble_dev(w3g_csr* s, void* stream) {
  if (!s) return w3g_fail(W3G_EARG, "null csr");
  w3g_context* c = s->ctx;
  CKS(cudaSetDevice(c->device));
  cudaStream_t st = (cudaStream_t)stream;
  const int grid = (int)std::min<long long>((s->nnz + kThreads - 1) / kThreads, 16LL * s->grid);
  if (c->precision == W3G_TANGENT_FP64)
    k_assemble<double><<<std::max(1, grid), kThreads, 0, st>>>(s->nnz, s->cptr, s->csrc, c->s.estiff, s->val);
  else
    k_assemble<float><<<std::max(1, grid), kThreads, 0, st>>>(s->nnz, s->cptr, s->csrc, c->s.estiff32, s->val);
  CKS(cudaGetLastError());
  return 0;
}

int w3g_csr_download(w3g_csr* s, int* rowptr, int* colind, double* values) {
  if (!s) return w3g_fail(W3G_EARG, "null csr");
  CKS(cudaSetDevice(s->ctx->device));
  CKS(cudaDeviceSynchronize());
  if (rowptr) CKS(cudaMemcpy(rowptr, s->rowptr, (s->n + 1) * sizeof(int), cudaMemcpyDeviceToHost));
  if (colind) CKS(cudaMemcpy(colind, s->colind, s->nnz * sizeof(int), cudaMemcpyDeviceToHost));
  if (values) CKS(cudaMemcpy(values, s->val, s->nnz * sizeof(double), cudaMemcpyDeviceToHost));
  return 0;
}

int w3g_pcg_dev(w3g_csr* s, const void* d_fixed, const void* d_b, double b_scale, void* d_x, double rtol, int maxit,
                void* stream, int* iters, double* relres) {
  if (!s || !d_fixed || !d_b || !d_x) return w3g_fail(W3G_EARG, "null argument");
  if (maxit < 0 || !(rtol >= 0.0)) return w3g_fail(W3G_EARG, "bad rtol / maxit");
  CKS(cudaSetDevice(s->ctx->device));
  const int n = s->n, G = s->grid;
  const unsigned char* fixed = (const unsigned char*)d_fixed;
  cudaStream_t st = s->stream;
  // ordered after the caller's stream
  CKS(cudaEventRecord(s->ev_in, (cudaStream_t)stream));
  CKS(cudaStreamWaitEvent(st, s->ev_in, 0));
  enqueue_pcg_init(s, fixed, (const double*)d_b, b_scale, st);
  k_pcg_init_fin<<<1, kThreads, 0, st>>>(s->partials, G, rtol, s->sc);
  CKS(cudaGetLastError());
  if (!s->batch || s->graph_fixed != d_fixed) {
    if (s->batch) cudaGraphExecDestroy(s->batch);
    s->batch = nullptr;
    cudaGraph_t g;
    CKS(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    enqueue_pcg_iterations(s, fixed, kBatch, st);
    CKS(cudaStreamEndCapture(st, &g));
    cudaError_t e = cudaGraphInstantiate(&s->batch, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return w3g_fail(W3G_ECUDA, std::string("pcg graph: ") + cudaGetErrorString(e));
    s->graph_fixed = d_fixed;
  }
  PcgScal h{};
  CKS(cudaMemcpyAsync(&h, s->sc, sizeof(h), cudaMemcpyDeviceToHost, st));
  CKS(cudaStreamSynchronize(st));
  while (!h.done && h.iters < maxit) {
    CKS(cudaGraphLaunch(s->batch, st));
    CKS(cudaMemcpyAsync(&h, s->sc, sizeof(h), cudaMemcpyDeviceToHost, st));
    CKS(cudaStreamSynchronize(st));
  }
  CKS(cudaMemcpyAsync(d_x, s->x, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, st));
  CKS(cudaEventRecord(s->ev_out, st));
  CKS(cudaStreamWaitEvent((cudaStream_t)stream, s->ev_out, 0));
  CKS(cudaStreamSynchronize(st));
  if (iters) *iters = h.iters;
  const double rel = h.bb > 0.0 ? std::sqrt(h.rr / h.bb) : 0.0;
  if (relres) *relres = rel;
  if (h.breakdown) return W3G_PCG_BREAKDOWN;
  return (h.rr <= h.tol2) ? 0 : W3G_PCG_MAXIT;
}

int w3g_residual_norms_dev(w3g_csr* s, const void* d_v, const void* d_fixed, void* d_out, void* stream) {
  if (!s || !d_v || !d_fixed || !d_out) return w3g_fail(W3G_EARG, "null argument");
  CKS(cudaSetDevice(s->ctx->device));
  cudaStream_t st = (cudaStream_t)stream;
  // its own partials (after the PCG's), so that it may run on any stream
  double* part = s->partials + 2 * (size_t)s->grid;
  k_norms<<<s->grid, kThreads, 0, st>>>(s->n, (const double*)d_v, (const unsigned char*)d_fixed, part);
  k_norms_fin<<<1, kThreads, 0, st>>>(part, s->grid, (double*)d_out);
  CKS(cudaGetLastError());
  return 0;
}

int w3g_free_dot_dev(w3g_csr* s, const void* d_a, const void* d_b, const void* d_fixed, void* d_out,
                     void* stream) {
  if (!s || !d_a || !d_b || !d_fixed || !d_out) return w3g_fail(W3G_EARG, "null argument");
  CKS(cudaSetDevice(s->ctx->device));
  cudaStream_t st = (cudaStream_t)stream;
  double* part = s->partials + 4 * (size_t)s->grid;
  k_dot_free<<<s->grid, kThreads, 0, st>>>(s->n, (const double*)d_a, (const double*)d_b,
                                           (const unsigned char*)d_fixed, part);
  k_dot_fin<<<1, kThreads, 0, st>>>(part, s->grid, (double*)d_out);
  CKS(cudaGetLastError());
  return 0;
}

int w3g_newton_iteration_dev(w3g_csr* s, int step, int iter, int extrapolated_du, const void* d_c,
                             const void* d_u, void* d_du, void* d_ifv, const void* d_fixed, void* d_d, double rtol,
                             int maxit, void* d_norms, void* stream, int* pcg_iters, double* pcg_relres,
                             int* recover_status, double* norms) {
  if (!s || !d_c || !d_u || !d_du || !d_ifv || !d_fixed || !d_d || !d_norms)
    return w3g_fail(W3G_EARG, "null argument");
  if (maxit < 0 || !(rtol >= 0.0)) return w3g_fail(W3G_EARG, "bad rtol / maxit");
  w3g_context* c = s->ctx;
  CKS(cudaSetDevice(c->device));
  NewtonKey k;
  k.c = d_c; k.u = d_u; k.du = d_du; k.ifv = d_ifv; k.fixed = d_fixed; k.d = d_d; k.norms = d_norms;
  k.precision = c->precision;
  k.sched = c->sched;
  k.wait_limit = c->wait_limit;
  k.triplet = s->triplet;
  if (!s->newton || !same_key(k, s->newton_key)) {
    const int r = build_newton_graph(s, k);
    if (r) return r;
  }
  cudaStream_t st = (cudaStream_t)stream;
  NewtonHost* hh = s->h_newton;
  hh->prm.rtol = rtol;
  hh->prm.maxit = maxit;
  CKS(cudaMemcpyAsync(s->d_prm, &hh->prm, sizeof(NewtonParams), cudaMemcpyHostToDevice, st));
  int r = w3g::enqueue_begin_recover(c, step, iter, extrapolated_du, st);
  if (r) return r;
  CKS(cudaGraphLaunch(s->newton, st));
  CKS(cudaMemcpyAsync(&hh->sc, s->sc, sizeof(PcgScal), cudaMemcpyDeviceToHost, st));
  CKS(cudaMemcpyAsync(&hh->info, w3g::device_recover_info(c), sizeof(w3g_recover_info), cudaMemcpyDeviceToHost,
                      st));
  CKS(cudaMemcpyAsync(hh->norms, d_norms, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  CKS(cudaStreamSynchronize(st));
  if (pcg_iters) *pcg_iters = hh->sc.iters;
  if (pcg_relres) *pcg_relres = hh->sc.bb > 0.0 ? std::sqrt(hh->sc.rr / hh->sc.bb) : 0.0;
  if (recover_status) *recover_status = hh->info.material_cut_step;
  if (norms) {
    norms[0] = hh->norms[0];
    norms[1] = hh->norms[1];
  }
  if (hh->sc.breakdown) return W3G_PCG_BREAKDOWN;
  return (hh->sc.rr <= hh->sc.tol2) ? 0 : W3G_PCG_MAXIT;
}

int w3g_csr_set_node_blocks(w3g_csr* s, int enable) {
  if (!s) return w3g_fail(W3G_EARG, "null csr");
  const bool t = enable && s->pattern_triplet;
  if (t != s->triplet) {
    s->triplet = t;
    if (s->batch) cudaGraphExecDestroy(s->batch);   // recaptured with the other kernels
    s->batch = nullptr;
  }
  return t ? 1 : 0;
}

}  // extern "C"
