// w3g_recover.cu -- launches of the recovery work items
// (w3g_recover_items.cuh) and the deterministic assembly of the element
// internal forces into the nodal vector (addifv).
//
// Two schedules over the same work items:
//   per type    one kernel per element type present, one CTA per item;
//   persistent  one kernel for all items of all types: CTAs resident on
//               every SM take the next items from a device work queue
//               (an atomic counter over the schedule order) until it is
//               empty, each item dispatched on its element type. Item
//               results do not depend on which CTA runs them or when.
//
// k_assemble_ifv: one thread per global dof sums the element
// contributions that map to it (a CSR built from edest at model creation,
// contributions in ascending einfvec order). This replaces the OpenMP
// ATOMIC scatter of addifv.f:93-98 with a deterministic gather.
#include <algorithm>
#include <climits>
#include "w3g_recover_items.cuh"

namespace w3g {

namespace {

constexpr size_t kRecoverSmem = std::max({sizeof(RecoverSmem<Hex8, 8>), sizeof(RecoverSmem<Hex20, 2>),
                                          sizeof(RecoverSmem<Tet10, 16>)});

__global__ void k_begin_recover(IterParams* params, unsigned long long* status, int step, int iter, int nonlinear) {
  params->step = step;
  params->iter = iter;
  params->nonlinear = nonlinear;
  params->pad = 0;
  status[0] = ~0ull;
}

__global__ void __launch_bounds__(kRecoverThreads) k_recover_hex8(RecoverArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const IterParams p = *a.params;
  const int cidx = a.chunk0 + blockIdx.x;
  if (umat_chunk(a, cidx)) recover_item_gen<Hex8, 8, 8, true>(a, p, cidx, smem);
  else recover_item_hex8(a, p, cidx, smem);
}

template <class E, int LPE, int EPC>
__global__ void __launch_bounds__(kRecoverThreads) k_recover_type(RecoverArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const IterParams p = *a.params;
  const int cidx = a.chunk0 + blockIdx.x;
  if (umat_chunk(a, cidx)) recover_item_gen<E, LPE, EPC, true>(a, p, cidx, smem);
  else recover_item_gen<E, LPE, EPC>(a, p, cidx, smem);
}

// persistent: the CTA takes q.grain queue entries at a time
__global__ void __launch_bounds__(kRecoverThreads) k_recover_persistent(RecoverArgs a, WorkQueue q) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int next;
  const IterParams p = *a.params;
  for (;;) {
    if (threadIdx.x == 0) next = atomicAdd(q.counter, q.grain);
    __syncthreads();
    const int w0 = next;
    __syncthreads();
    if (w0 >= q.nitems) break;
    const int w1 = min(w0 + q.grain, q.nitems);
    for (int w = w0; w < w1; ++w) {
      const int cidx = q.items[w];
      const bool um = umat_chunk(a, cidx);
      switch (a.chunks[cidx].type) {
        case 0:
          if (um) recover_item_gen<Hex8, 8, 8, true>(a, p, cidx, smem);
          else recover_item_hex8(a, p, cidx, smem);
          break;
        case 1:
          if (um) recover_item_gen<Hex20, 32, 2, true>(a, p, cidx, smem);
          else recover_item_gen<Hex20, 32, 2>(a, p, cidx, smem);
          break;
        default:
          if (um) recover_item_gen<Tet10, 4, 16, true>(a, p, cidx, smem);
          else recover_item_gen<Tet10, 4, 16>(a, p, cidx, smem);
          break;
      }
      __syncthreads();   // the next item reuses the shared memory
    }
  }
}

template <class K>
cudaError_t prepare(K kern, size_t smem) {
  if (smem <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

// the undeformed-geometry cache is valid while the coordinates equal the
// ones it was built from; a changed coordinate marks it dirty
__global__ void k_check_coords(const double* __restrict__ c, const double* __restrict__ c_geo, int n, int* dirty) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n && c[k] != c_geo[k]) *dirty = 1;
}

__global__ void k_commit_coords(const double* __restrict__ c, double* c_geo, int n, int* dirty) {
  if (*dirty == 0) return;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) c_geo[k] = c[k];
}

__global__ void k_clear_dirty(int* dirty) { *dirty = 0; }

constexpr int kAsmThreads = 256;

__global__ void __launch_bounds__(kAsmThreads) k_assemble_ifv(int nodof, const int* __restrict__ rowptr,
                                                              const long long* __restrict__ src,
                                                              const double* __restrict__ einf, double* ifv,
                                                              double* partials) {
  __shared__ double sw[kAsmThreads / 32];
  const int d = blockIdx.x * kAsmThreads + threadIdx.x;
  double s = 0.0, sa = 0.0;
  if (d < nodof) {
    for (int k = rowptr[d]; k < rowptr[d + 1]; ++k) {
      const double v = einf[src[k]];
      s += v;
      sa += fabs(v);
    }
    ifv[d] = s;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) sa += __shfl_xor_sync(0xffffffffu, sa, off);
  if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = sa;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < kAsmThreads / 32; ++k) t += sw[k];
    partials[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(256) k_finalize(int nchunks, const double* partials, int nparts,
                                                  const double* ifv_partials, const unsigned long long* status,
                                                  const BlockDesc* blocks, long long num_term,
                                                  w3g_recover_info* info) {
  __shared__ double s0[256], s1[256], s2[256];
  double e = 0.0, p = 0.0, f = 0.0;
  for (int k = threadIdx.x; k < nchunks; k += 256) { e += partials[2 * k]; p += partials[2 * k + 1]; }
  for (int k = threadIdx.x; k < nparts; k += 256) f += ifv_partials[k];
  s0[threadIdx.x] = e; s1[threadIdx.x] = p; s2[threadIdx.x] = f;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      s0[threadIdx.x] += s0[threadIdx.x + w];
      s1[threadIdx.x] += s1[threadIdx.x + w];
      s2[threadIdx.x] += s2[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const unsigned long long st = status[0];
    const bool cut = st != ~0ull;
    info->internal_energy = s0[0];
    info->plastic_work = s1[0];
    info->sum_ifv = s2[0];
    info->num_term_ifv = num_term;
    info->material_cut_step = cut ? (((st >> 20) & 0xFull) == 2 ? W3G_LOCAL_FAIL : W3G_STEP_CUT) : 0;
    info->first_bad_element = cut ? blocks[st >> 40].felem + (int)(st & 0xFFFFFull) + 1 : 0;
  }
}

}  // namespace


namespace {
int g_occ = 0;   // persistent CTAs per SM
}

cudaError_t init_recover_kernels() {
  cudaError_t e;
  if ((e = prepare(k_recover_hex8, sizeof(RecoverSmem<Hex8, 8>))) != cudaSuccess) return e;
  if ((e = prepare(k_recover_type<Hex20, 32, 2>, sizeof(RecoverSmem<Hex20, 2>))) != cudaSuccess) return e;
  if ((e = prepare(k_recover_type<Tet10, 4, 16>, sizeof(RecoverSmem<Tet10, 16>))) != cudaSuccess) return e;
  if ((e = prepare(k_recover_persistent, kRecoverSmem)) != cudaSuccess) return e;
  int n = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_recover_persistent, kRecoverThreads, kRecoverSmem);
  if (e != cudaSuccess) return e;
  g_occ = std::max(1, n);
  return cudaSuccess;
}

int persistent_recover_occupancy() { return std::max(1, g_occ); }

int recover_kernel_launches(const DeviceModel& m, const Schedule& sc) {
  int n = mm10_kernel_launches(m, sc.order == W3G_ORDER_HEAVY_FIRST);
  if (sc.mode == W3G_SCHED_PERSISTENT) return n + (m.nrchunks > 0 ? 1 : 0);
  for (int t = 0; t < kNumTypes; ++t) n += m.type_chunks[t] > 0 ? 1 : 0;
  return n;
}

cudaError_t launch_begin_recover(IterParams* params, unsigned long long* status, int step, int iter, int nonlinear,
                                 cudaStream_t s) {
  k_begin_recover<<<1, 1, 0, s>>>(params, status, step, iter, nonlinear);
  return cudaGetLastError();
}

cudaError_t launch_recover(const DeviceModel& m, const RecoverArgs& a, double* c_geo, const Schedule& sc,
                           int* counter, cudaStream_t s) {
  if (m.nchunks == 0) return cudaSuccess;
  const int nb = (m.ncoord + 255) / 256;
  k_check_coords<<<nb, 256, 0, s>>>(a.c, c_geo, m.ncoord, a.geo_dirty);
  cudaError_t e = cudaSuccess;
  if (sc.mode == W3G_SCHED_PERSISTENT) {
    if (m.nrchunks > 0) {
      const int occ = persistent_recover_occupancy();
      const int per_sm = sc.recover_ctas_per_sm > 0 ? std::min(sc.recover_ctas_per_sm, occ) : occ;
      const int grain = std::max(1, sc.recover_grain);
      const int need = (m.nrchunks + grain - 1) / grain;
      const int grid = std::max(1, std::min(m.nsm * per_sm, need));
      WorkQueue q{m.rorder[sc.order == W3G_ORDER_HEAVY_FIRST ? 1 : 0], m.nrchunks, grain, counter};
      e = cudaMemsetAsync(counter, 0, sizeof(int), s);
      if (e != cudaSuccess) return e;
      k_recover_persistent<<<grid, kRecoverThreads, kRecoverSmem, s>>>(a, q);
    }
  } else {
    const size_t s8 = sizeof(RecoverSmem<Hex8, 8>), s20 = sizeof(RecoverSmem<Hex20, 2>),
                 s10 = sizeof(RecoverSmem<Tet10, 16>);
    if (m.type_chunks[0] > 0) {
      RecoverArgs h = a;
      h.chunk0 = m.type_chunk0[0];
      k_recover_hex8<<<m.type_chunks[0], kRecoverThreads, s8, s>>>(h);
    }
    if (m.type_chunks[1] > 0) {
      RecoverArgs h = a;
      h.chunk0 = m.type_chunk0[1];
      k_recover_type<Hex20, 32, 2><<<m.type_chunks[1], kRecoverThreads, s20, s>>>(h);
    }
    if (m.type_chunks[2] > 0) {
      RecoverArgs h = a;
      h.chunk0 = m.type_chunk0[2];
      k_recover_type<Tet10, 4, 16><<<m.type_chunks[2], kRecoverThreads, s10, s>>>(h);
    }
  }
  if ((e = launch_mm10(m, a, s)) != cudaSuccess) return e;
  k_commit_coords<<<nb, 256, 0, s>>>(a.c, c_geo, m.ncoord, a.geo_dirty);
  k_clear_dirty<<<1, 1, 0, s>>>(a.geo_dirty);
  return cudaGetLastError();
}

int assemble_ifv_parts(int nodof) { return (nodof + kAsmThreads - 1) / kAsmThreads; }

cudaError_t launch_assemble_ifv(const DeviceModel& m, const double* einf, double* ifv, double* ifv_partials,
                                int nparts, cudaStream_t s) {
  if (m.nodof == 0) return cudaSuccess;
  k_assemble_ifv<<<nparts, kAsmThreads, 0, s>>>(m.nodof, m.ifv_rowptr, m.ifv_src, einf, ifv, ifv_partials);
  return cudaGetLastError();
}

cudaError_t launch_finalize(const DeviceModel& m, const double* partials, const double* ifv_partials, int nparts,
                            const unsigned long long* status, w3g_recover_info* d_info, cudaStream_t s) {
  k_finalize<<<1, 256, 0, s>>>(m.nchunks, partials, nparts, ifv_partials, status, m.blocks, m.einf_total, d_info);
  return cudaGetLastError();
}

}  // namespace w3g
