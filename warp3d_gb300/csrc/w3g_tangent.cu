// w3g_tangent.cu -- launches of the tangent work items
// (w3g_tangent_items.cuh).
//
// Two schedules over the same work items:
//   per type    one kernel per element type present, one warp-sized CTA
//               per item;
//   persistent  one kernel for all items of all types: CTAs resident on
//               every SM take the next items from a device work queue
//               (an atomic counter over the schedule order) until it is
//               empty, each item dispatched on its element type. Item
//               results do not depend on which CTA runs them or when.
#include <algorithm>
#include "w3g_tangent_items.cuh"

namespace w3g {

namespace {

// shared memory of the brick items; models with b-bar blocks launch with
// the larger b-bar layout (more per element), the others keep the smaller
// one and its occupancy
template <class T>
constexpr size_t hex8_smem(bool bbar) {
  return sizeof(T) == 8 ? (bbar ? sizeof(TangentSmemHex8<double, true>) : sizeof(TangentSmemHex8<double>))
                        : (bbar ? sizeof(TangentSmemHex8F32<true>) : sizeof(TangentSmemHex8F32<>));
}

template <class T>
constexpr size_t tangent_smem(bool bbar) {
  return std::max({hex8_smem<T>(bbar), sizeof(TangentSmemGen<Hex20, 1, T>), sizeof(TangentSmemGen<Tet10, 4, T>)});
}

// the FP32 coordinates are relative to the element's first node; b-bar
// blocks take the b-bar instantiation of the item
template <class T>
__device__ __forceinline__ void hex8_item(const TangentArgs& a, int cidx, unsigned char* smem);
template <>
__device__ __forceinline__ void hex8_item<double>(const TangentArgs& a, int cidx, unsigned char* smem) {
  if (a.blocks[a.chunks[cidx].blk].bbar) tangent_item_hex8<double, double, false, true>(a, cidx, smem);
  else tangent_item_hex8<double, double, false>(a, cidx, smem);
}
template <>
__device__ __forceinline__ void hex8_item<float>(const TangentArgs& a, int cidx, unsigned char* smem) {
  if (a.blocks[a.chunks[cidx].blk].bbar) tangent_item_hex8_f32<true>(a, cidx, smem);
  else tangent_item_hex8_f32<false>(a, cidx, smem);
}

// resident one-warp CTAs per SM for the FP32 brick tangent (registers:
// 65536 / (32 x this)); the FP64 form is bound by the FP64 pipe at any
// occupancy. Measured on 262,144 bricks: 12 -> 0.530 ms, 16 -> 0.547 ms,
// 20 -> 0.692 ms, 24 -> 0.821 ms (the 81 accumulators of a lane's node
// pairs want registers more than the kernel wants warps)
#ifndef W3G_TAN32_MIN_CTAS
#define W3G_TAN32_MIN_CTAS 12
#endif

template <class T>
__global__ void __launch_bounds__(kTangentThreads, sizeof(T) == 8 ? 1 : W3G_TAN32_MIN_CTAS)
    k_tangent_hex8(TangentArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  hex8_item<T>(a, a.chunk0 + blockIdx.x, smem);
}

template <class E, int LPE, int EPC, class T>
__global__ void __launch_bounds__(kTangentThreads) k_tangent_type(TangentArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  tangent_item_gen<E, LPE, EPC, T, sizeof(T) == 4>(a, a.chunk0 + blockIdx.x, smem);
}

template <class T>
__global__ void __launch_bounds__(kTangentThreads, sizeof(T) == 8 ? 1 : 12)
    k_tangent_persistent(TangentArgs a, WorkQueue q) {
  extern __shared__ __align__(16) unsigned char smem[];
  for (;;) {
    int w0 = 0;
    if (threadIdx.x == 0) w0 = atomicAdd(q.counter, q.grain);
    w0 = __shfl_sync(0xffffffffu, w0, 0);
    if (w0 >= q.nitems) break;
    const int w1 = min(w0 + q.grain, q.nitems);
    for (int w = w0; w < w1; ++w) {
      const int cidx = q.items[w];
      switch (a.chunks[cidx].type) {
        case 0: hex8_item<T>(a, cidx, smem); break;
        case 1: tangent_item_gen<Hex20, 32, 1, T, sizeof(T) == 4>(a, cidx, smem); break;
        default: tangent_item_gen<Tet10, 8, 4, T, sizeof(T) == 4>(a, cidx, smem); break;
      }
      __syncwarp();   // the next item reuses the shared memory
    }
  }
}

template <class K>
cudaError_t prepare(K kern, size_t smem) {
  if (smem <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

int g_occ[2][2] = {{0, 0}, {0, 0}};   // persistent CTAs per SM: [FP32][b-bar layout]

template <class T>
cudaError_t init() {
  cudaError_t e;
  if ((e = prepare(k_tangent_hex8<T>, hex8_smem<T>(true))) != cudaSuccess) return e;
  if ((e = prepare(k_tangent_type<Hex20, 32, 1, T>, sizeof(TangentSmemGen<Hex20, 1, T>))) != cudaSuccess) return e;
  if ((e = prepare(k_tangent_type<Tet10, 8, 4, T>, sizeof(TangentSmemGen<Tet10, 4, T>))) != cudaSuccess) return e;
  if ((e = prepare(k_tangent_persistent<T>, tangent_smem<T>(true))) != cudaSuccess) return e;
  for (int bb = 0; bb < 2; ++bb) {
    int n = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_tangent_persistent<T>, kTangentThreads,
                                                      tangent_smem<T>(bb != 0));
    if (e != cudaSuccess) return e;
    g_occ[sizeof(T) == 4][bb] = std::max(1, n);
  }
  return cudaSuccess;
}

template <class T>
int occupancy(bool bbar) { return std::max(1, g_occ[sizeof(T) == 4][bbar ? 1 : 0]); }

template <class T>
cudaError_t launch(const DeviceModel& m, const TangentArgs& a, const Schedule& sc, int* counter, cudaStream_t s,
                   bool tc) {
  cudaError_t e = cudaSuccess;
  const bool bb = m.has_bbar != 0;
  if (sc.mode == W3G_SCHED_PERSISTENT && !tc) {
    const int occ = occupancy<T>(bb);
    const int per_sm = sc.tangent_ctas_per_sm > 0 ? std::min(sc.tangent_ctas_per_sm, occ) : occ;
    const int grain = std::max(1, sc.tangent_grain);
    const int need = (m.ntchunks + grain - 1) / grain;
    const int grid = std::max(1, std::min(m.nsm * per_sm, need));
    WorkQueue q{m.torder[sc.order == W3G_ORDER_HEAVY_FIRST ? 1 : 0], m.ntchunks, grain, counter};
    if ((e = cudaMemsetAsync(counter, 0, sizeof(int), s)) != cudaSuccess) return e;
    k_tangent_persistent<T><<<grid, kTangentThreads, tangent_smem<T>(bb), s>>>(a, q);
    return cudaGetLastError();
  }
  if (m.ttype_chunks[0] > 0 && !tc) {
    TangentArgs h = a;
    h.chunk0 = m.ttype_chunk0[0];
    k_tangent_hex8<T><<<m.ttype_chunks[0], kTangentThreads, hex8_smem<T>(bb), s>>>(h);
  }
  if (m.ttype_chunks[1] > 0 && !tc) {   // with the tensor-core forms, 20-node bricks have their kernel
    TangentArgs h = a;
    h.chunk0 = m.ttype_chunk0[1];
    k_tangent_type<Hex20, 32, 1, T><<<m.ttype_chunks[1], kTangentThreads, sizeof(TangentSmemGen<Hex20, 1, T>), s>>>(h);
  }
  if (m.ttype_chunks[2] > 0) {
    TangentArgs h = a;
    h.chunk0 = m.ttype_chunk0[2];
    k_tangent_type<Tet10, 8, 4, T><<<m.ttype_chunks[2], kTangentThreads, sizeof(TangentSmemGen<Tet10, 4, T>), s>>>(h);
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t init_tangent_kernels() {
  cudaError_t e = init<double>();
  return e == cudaSuccess ? init<float>() : e;
}

int persistent_tangent_occupancy(const DeviceModel& m, bool fp32) {
  return fp32 ? occupancy<float>(m.has_bbar != 0) : occupancy<double>(m.has_bbar != 0);
}

namespace {

template <class T>
cudaError_t launch_ranges(const DeviceModel& m, const TangentArgs& a, const int* first, const int* count,
                          cudaStream_t s, int* launches) {
  int n = 0;
  if (count[0] > 0) {
    TangentArgs h = a;
    h.chunk0 = first[0];
    k_tangent_hex8<T><<<count[0], kTangentThreads, hex8_smem<T>(m.has_bbar != 0), s>>>(h);
    ++n;
  }
  if (count[1] > 0) {
    TangentArgs h = a;
    h.chunk0 = first[1];
    k_tangent_type<Hex20, 32, 1, T><<<count[1], kTangentThreads, sizeof(TangentSmemGen<Hex20, 1, T>), s>>>(h);
    ++n;
  }
  if (count[2] > 0) {
    TangentArgs h = a;
    h.chunk0 = first[2];
    k_tangent_type<Tet10, 8, 4, T><<<count[2], kTangentThreads, sizeof(TangentSmemGen<Tet10, 4, T>), s>>>(h);
    ++n;
  }
  if (launches) *launches = n;
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_tangent_ranges(const DeviceModel& m, const TangentArgs& a, bool fp32, const int* first,
                                  const int* count, cudaStream_t s, int* launches) {
  return fp32 ? launch_ranges<float>(m, a, first, count, s, launches)
              : launch_ranges<double>(m, a, first, count, s, launches);
}

int tangent_kernel_launches(const DeviceModel& m, const Schedule& sc, bool tc) {
  if (sc.mode == W3G_SCHED_PERSISTENT && !tc) return m.ntchunks > 0 ? 1 : 0;
  if (tc)
    return (m.ntcchunks > 0 ? 1 : 0) + (m.ntcgtiles > 0 ? 1 : 0) + (m.ntc20tiles > 0 ? 1 : 0) +
           (m.ttype_chunks[2] > 0 ? 1 : 0);
  int n = 0;
  for (int t = 0; t < kNumTypes; ++t) n += m.ttype_chunks[t] > 0 ? 1 : 0;
  return n;
}

cudaError_t launch_tangent(const DeviceModel& m, const TangentArgs& a, bool fp32, const Schedule& sc, int* counter,
                           cudaStream_t s, bool tc) {
  if (m.ntchunks == 0) return cudaSuccess;
  return fp32 ? launch<float>(m, a, sc, counter, s, tc) : launch<double>(m, a, sc, counter, s, tc);
}

}  // namespace w3g
