// w3g_api.cu -- the C-ABI of include/w3g.h: model registration, resident
// device state, and the tanstf / drive_eps_sig_internal_forces / update
// replacements. No torch types cross this boundary.
#include <climits>
#include <cstdio>
#include <cstring>
#include <string>
#include <utility>
#include <vector>
#include <algorithm>
#include <thread>
#include "w3g_internal.cuh"
#include "w3g_elem.cuh"

using namespace w3g;

#include "w3g_context.cuh"
#include "w3g_umat.cuh"

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CK(call)                                                                           \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return fail(W3G_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_));         \
  } while (0)

// trailing elements allocated beyond the arrays that 1-D bulk copies read
// (cep, rot_n1, urcs_n1; edest, cdest): a copy of a tile's slab is rounded
// out to 16-byte boundaries and may read up to 12 bytes past the last
// element
constexpr size_t kBulkPad = 4;

template <class T>
cudaError_t dalloc(T** p, size_t n) {
  if (n == 0) n = 1;
  return cudaMalloc((void**)p, n * sizeof(T));
}

void free_all(w3g_context* c) {
  DeviceModel& m = c->m;
  DeviceState& s = c->s;
  if (c->graph.exec) cudaGraphExecDestroy(c->graph.exec);
  void* ptrs[] = {m.blocks, m.chunks, m.tchunks, m.tcchunks, m.tcgtiles, m.tc20tiles, s.tc_timeout, m.rorder[0], m.rorder[1], m.torder[0], m.torder[1], m.edest,
                  m.cdest, m.mat, m.umat_props, m.dn[0], m.dn[1], m.dn[2], m.dn32[0], m.dn32[1], m.dn32[2],
                  m.ifv_rowptr, m.ifv_src, s.params, s.counters, m.xtal, m.xtype, m.mm10_gp, s.mm10_scr,
                  s.mm10_iters, s.mm10_order, s.mm10_ident, s.mm10_bins,
                  s.geo, s.c_geo, s.geo_dirty,
                  s.hist, s.hist1, s.urcs_n, s.urcs_n1, s.eps_n, s.eps_n1, s.rot_n1, s.cep, s.estiff,
                  s.estiff32, s.einf, s.evol, s.partials, s.ifv_partials, s.status, s.d_info,
                  m.blocks_packed, s.estiff_packed, s.estiff_packed32,
                  s.d_c, s.d_u, s.d_du, s.d_ifv};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (c->h_stage) cudaFreeHost(c->h_stage);
  for (cudaEvent_t& ev : c->part_done)
    if (ev) cudaEventDestroy(ev);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  if (c->stream) cudaStreamDestroy(c->stream);
}

__global__ void k_init_rot(double* rot, long long ngp_total) {
  long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (k < ngp_total) {
    double* r = rot + k * 9;
    r[0] = 1.0; r[1] = 0.0; r[2] = 0.0; r[3] = 0.0; r[4] = 1.0; r[5] = 0.0; r[6] = 0.0; r[7] = 0.0; r[8] = 1.0;
  }
}

// copy n values between per-block host pointers and one device array
int blocks_h2d(w3g_context* c, double* dev, double* const* host, int per_elem_or_gp, bool per_gp) {
  for (int b = 0; b < c->m.nelblk; ++b) {
    const BlockDesc& bd = c->blocks[b];
    size_t n = (size_t)bd.span * (per_gp ? bd.ngp : 1) * per_elem_or_gp;
    size_t off = (size_t)(per_gp ? bd.gp_off : bd.felem) * per_elem_or_gp;
    if (!host[b]) continue;
    CK(cudaMemcpyAsync(dev + off, host[b], n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

int blocks_d2h(w3g_context* c, const double* dev, double* const* host, int per, bool per_gp) {
  for (int b = 0; b < c->m.nelblk; ++b) {
    const BlockDesc& bd = c->blocks[b];
    size_t n = (size_t)bd.span * (per_gp ? bd.ngp : 1) * per;
    size_t off = (size_t)(per_gp ? bd.gp_off : bd.felem) * per;
    if (!host[b]) continue;
    CK(cudaMemcpyAsync(host[b], dev + off, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

// history blocks: (hist, ngp, span) each, hist per block
int hist_h2d(w3g_context* c, double* dev, double* const* host) {
  for (int b = 0; b < c->m.nelblk; ++b) {
    const BlockDesc& bd = c->blocks[b];
    if (!host[b]) continue;
    CK(cudaMemcpyAsync(dev + bd.hist_off, host[b], (size_t)bd.hist * bd.ngp * bd.span * sizeof(double),
                       cudaMemcpyHostToDevice, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

int hist_d2h(w3g_context* c, const double* dev, double* const* host) {
  for (int b = 0; b < c->m.nelblk; ++b) {
    const BlockDesc& bd = c->blocks[b];
    if (!host[b]) continue;
    CK(cudaMemcpyAsync(host[b], dev + bd.hist_off, (size_t)bd.hist * bd.ngp * bd.span * sizeof(double),
                       cudaMemcpyDeviceToHost, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

TangentArgs tangent_args(w3g_context* c, const double* d_c, const double* d_u, const double* d_du) {
  TangentArgs a;
  for (int t = 0; t < kNumTypes; ++t) { a.dn[t] = c->m.dn[t]; a.dn32[t] = c->m.dn32[t]; }
  a.blocks = c->m.blocks;
  a.chunks = c->m.tchunks;
  a.chunk0 = 0;
  a.edest = c->m.edest;
  a.cdest = c->m.cdest;
  a.c = d_c; a.u = d_u; a.du = d_du;
  a.rot_n1 = c->s.rot_n1;
  a.urcs_n1 = c->s.urcs_n1;
  a.cep = c->s.cep;
  a.hist1 = c->s.hist1;
  a.estiff = c->precision != W3G_TANGENT_FP64 ? (void*)c->s.estiff32 : (void*)c->s.estiff;
  a.qbar = c->m.qbar;
  a.beta_fact = c->m.beta_fact;
  a.bbar_beta = c->m.bbar_beta;
  a.wait_limit = c->wait_limit;
  return a;
}

// enqueues the tangent kernels; returns the number of kernel launches or
// a negative status
int enqueue_tangent(w3g_context* c, const double* d_c, const double* d_u, const double* d_du, cudaStream_t st) {
  TangentArgs a = tangent_args(c, d_c, d_u, d_du);
  const int p = c->precision;
  if (c->m.asym) {   // asymmetric assembly: full matrices
    const bool f32 = p != W3G_TANGENT_FP64;
    cudaError_t e = launch_tangent_full(c->m, a, f32, st);   // 8-node bricks, any [D]
    int n = c->m.ttype_chunks[0] > 0 ? 1 : 0;
    if (e == cudaSuccess && c->m.packed_total > 0) {
      // 20-node bricks and tetrahedra (mm01, symmetric [D]): packed into
      // the scratch array, then expanded
      TangentArgs ap = a;
      ap.blocks = c->m.blocks_packed;
      ap.estiff = f32 ? (void*)c->s.estiff_packed32 : (void*)c->s.estiff_packed;
      int first[kNumTypes], count[kNumTypes], k = 0;
      for (int t = 0; t < kNumTypes; ++t) { first[t] = c->m.ttype_chunk0[t]; count[t] = t == 0 ? 0 : c->m.ttype_chunks[t]; }
      e = launch_tangent_ranges(c->m, ap, f32, first, count, st, &k);
      n += k;
      if (e == cudaSuccess) e = launch_expand_packed(c->m, a, ap.estiff, f32, st);
      ++n;
    }
    if (e != cudaSuccess) return fail(W3G_ECUDA, std::string("tangent launch: ") + cudaGetErrorString(e));
    return n;
  }
  const bool tc = p >= W3G_TANGENT_TF32;
  cudaError_t e = cudaSuccess;
  if (tc) {
    const bool bf16 = p == W3G_TANGENT_BF16 || p == W3G_TANGENT_BF16X3;
    const bool split = p == W3G_TANGENT_TF32X3 || p == W3G_TANGENT_BF16X3;
    e = launch_tangent_tcg_hex8(c->m, a, bf16, split, c->s.tc_timeout, st);
    if (e == cudaSuccess) e = launch_tangent_tc_hex8(c->m, a, bf16, split, c->s.tc_timeout, st);
    if (e == cudaSuccess) e = launch_tangent_tc_hex20(c->m, a, bf16, split, c->s.tc_timeout, st);
  }
  if (e == cudaSuccess)
    e = launch_tangent(c->m, a, c->precision != W3G_TANGENT_FP64, c->sched, c->s.counters + 1, st, tc);
  if (e != cudaSuccess) return fail(W3G_ECUDA, std::string("tangent launch: ") + cudaGetErrorString(e));
  return tangent_kernel_launches(c->m, c->sched, tc);
}

int run_tangent(w3g_context* c, const double* d_c, const double* d_u, const double* d_du, cudaStream_t st) {
  const int n = enqueue_tangent(c, d_c, d_u, d_du, st);
  if (n < 0) return n;
  c->last_launches = n;
  return 0;
}

// enqueues recovery after the iteration scalars are in place (everything
// but k_begin_recover, so that it can be captured); returns the number of
// kernel launches or a negative status
int enqueue_recover(w3g_context* c, const double* d_c, const double* d_u, const double* d_du, double* d_ifv,
                    cudaStream_t st) {
  RecoverArgs a;
  for (int t = 0; t < kNumTypes; ++t) a.dn[t] = c->m.dn[t];
  a.blocks = c->m.blocks;
  a.chunks = c->m.chunks;
  a.chunk0 = 0;
  a.edest = c->m.edest;
  a.cdest = c->m.cdest;
  a.mat = c->m.mat;
  a.c = d_c; a.u = d_u; a.du = d_du;
  a.hist = c->s.hist; a.hist1 = c->s.hist1;
  a.urcs_n = c->s.urcs_n; a.urcs_n1 = c->s.urcs_n1;
  a.eps_n = c->s.eps_n; a.eps_n1 = c->s.eps_n1;
  a.rot_n1 = c->s.rot_n1;
  a.cep = c->s.cep;
  a.einf = c->s.einf;
  a.umat_props = c->m.umat_props;
  a.evol = c->s.evol;
  a.partials = c->s.partials;
  a.status = c->s.status;
  a.geo = c->s.geo;
  a.geo_dirty = c->s.geo_dirty;
  a.params = c->s.params;
  a.beta_fact = c->m.beta_fact;
  a.bbar_beta = c->m.bbar_beta;
  a.asym = c->m.asym;
  a.xtal = c->m.xtal;
  a.xtype = c->m.xtype;
  a.mm10_scr = c->s.mm10_scr;
  a.mm10_gp = c->m.mm10_gp;
  a.mm10_iters = c->s.mm10_iters;
  a.mm10_order = c->s.mm10_order;
  a.mm10_ident = c->s.mm10_ident;
  a.mm10_sorted = c->sched.order == W3G_ORDER_HEAVY_FIRST ? 1 : 0;
  a.mm10_bins = c->s.mm10_bins;
  a.mm10_counter = c->s.counters + 2;
  a.dt = c->m.dt;
  cudaError_t e = launch_recover(c->m, a, c->s.c_geo, c->sched, c->s.counters, st);
  if (e == cudaSuccess) e = launch_assemble_ifv(c->m, c->s.einf, d_ifv, c->s.ifv_partials, c->ifv_parts, st);
  if (e == cudaSuccess)
    e = launch_finalize(c->m, c->s.partials, c->s.ifv_partials, c->ifv_parts, c->s.status, c->s.d_info, st);
  if (e != cudaSuccess) return fail(W3G_ECUDA, std::string("recover launch: ") + cudaGetErrorString(e));
  // coordinate check/commit/clear, element kernels, ifv assembly, finalize
  return 5 + recover_kernel_launches(c->m, c->sched);
}

int begin_recover(w3g_context* c, int step, int iter, int extrap, cudaStream_t st) {
  cudaError_t e = launch_begin_recover(c->s.params, c->s.status, step, iter, (iter >= 1 || extrap) ? 1 : 0, st);
  if (e != cudaSuccess) return fail(W3G_ECUDA, std::string("recover launch: ") + cudaGetErrorString(e));
  return 0;
}

int run_recover(w3g_context* c, int step, int iter, int extrap, const double* d_c, const double* d_u,
                const double* d_du, double* d_ifv, cudaStream_t st) {
  int r = begin_recover(c, step, iter, extrap, st);
  if (r) return r;
  const int n = enqueue_recover(c, d_c, d_u, d_du, d_ifv, st);
  if (n < 0) return n;
  c->last_launches = 1 + n;
  return 0;
}

}  // namespace

void w3g::set_last_error(const std::string& msg) { g_err = msg; }

namespace {

// number of non-finite values among n (device counter, order-free)
template <class T>
__global__ void k_count_nonfinite(const T* __restrict__ v, long long n, unsigned long long* bad) {
  unsigned long long local = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    local += isfinite(v[i]) ? 0ull : 1ull;
  if (local) atomicAdd(bad, local);
}

template <class T>
cudaError_t count_nonfinite(const T* v, long long n, unsigned long long* bad, cudaStream_t st) {
  if (n <= 0 || !v) return cudaSuccess;
  const long long blocks = std::min<long long>((n + 255) / 256, 4096);
  k_count_nonfinite<T><<<(int)blocks, 256, 0, st>>>(v, n, bad);
  return cudaGetLastError();
}

// copies Ke of blocks [b0, b1) to the host pointers, blocks whose host
// arrays follow each other in memory in one copy
int copy_estiff_range(w3g_context* c, double* const* estiff, int b0, int b1, cudaStream_t st) {
  for (int b = b0; b < b1; ++b) {
    const BlockDesc& bd = c->blocks[b];
    if (!estiff[b]) continue;
    int e = b;
    size_t run = (size_t)bd.ek_rows * bd.span;
    while (e + 1 < b1 && estiff[e + 1] && estiff[e + 1] == estiff[e] + (size_t)c->blocks[e].ek_rows * c->blocks[e].span) {
      ++e;
      run += (size_t)c->blocks[e].ek_rows * c->blocks[e].span;
    }
    CK(cudaMemcpyAsync(estiff[b], c->s.estiff + bd.estiff_off, run * sizeof(double), cudaMemcpyDeviceToHost, st));
    b = e;
  }
  return 0;
}

// FP64 tangent with host Ke: the blocks are cut into parts of similar Ke
// size; each part's kernels run on the compute stream and its Ke is copied
// to the host on a second stream while the next part computes, so that
// only the last part's copy is exposed
int tanstf_overlapped(w3g_context* c, double* const* estiff, cudaStream_t st) {
  constexpr int kParts = 8;
  if (!c->copy_stream) {
    CK(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    for (cudaEvent_t& ev : c->part_done) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  }
  const int nb = c->m.nelblk;
  const long long total = c->m.estiff_total;
  TangentArgs a = tangent_args(c, c->s.d_c, c->s.d_u, c->s.d_du);
  int launches = 0, b0 = 0;
  for (int k = 0; k < kParts && b0 < nb; ++k) {
    int b1 = b0 + 1;
    const long long target = total * (k + 1) / kParts;
    while (b1 < nb && (k == kParts - 1 || c->blocks[b1].estiff_off < target)) ++b1;
    // per type: the work items of blocks [b0, b1) (items are in block order within a type)
    int first[kNumTypes], count[kNumTypes];
    for (int t = 0; t < kNumTypes; ++t) {
      const Chunk* beg = c->h_tchunks.data() + c->m.ttype_chunk0[t];
      const Chunk* end = beg + c->m.ttype_chunks[t];
      const Chunk* lo = std::lower_bound(beg, end, b0, [](const Chunk& x, int v) { return x.blk < v; });
      const Chunk* hi = std::lower_bound(lo, end, b1, [](const Chunk& x, int v) { return x.blk < v; });
      first[t] = (int)(lo - c->h_tchunks.data());
      count[t] = (int)(hi - lo);
    }
    int n = 0;
    cudaError_t e = launch_tangent_ranges(c->m, a, false, first, count, st, &n);
    if (e != cudaSuccess) return fail(W3G_ECUDA, std::string("tangent launch: ") + cudaGetErrorString(e));
    launches += n;
    CK(cudaEventRecord(c->part_done[k], st));
    CK(cudaStreamWaitEvent(c->copy_stream, c->part_done[k], 0));
    int r = copy_estiff_range(c, estiff, b0, b1, c->copy_stream);
    if (r) return r;
    b0 = b1;
  }
  c->last_launches = launches;
  CK(cudaStreamSynchronize(c->copy_stream));
  CK(cudaStreamSynchronize(st));
  return 0;
}

// precision forms with host Ke: one copy of the FP32 matrices, widened to
// double by host threads
int download_estiff32(w3g_context* c, double* const* estiff, cudaStream_t st) {
  const size_t total = (size_t)c->m.estiff_total;
  if (c->h_stage_n < total) {
    if (c->h_stage) cudaFreeHost(c->h_stage);
    c->h_stage = nullptr;
    c->h_stage_n = 0;
    CK(cudaMallocHost((void**)&c->h_stage, total * sizeof(double)));
    c->h_stage_n = total;
  }
  float* f = reinterpret_cast<float*>(c->h_stage);
  CK(cudaMemcpyAsync(f, c->s.estiff32, total * sizeof(float), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  const int nb = c->m.nelblk;
  const int nth = (int)std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  auto work = [&](int t) {
    for (int b = t; b < nb; b += nth) {
      if (!estiff[b]) continue;
      const BlockDesc& bd = c->blocks[b];
      const float* src = f + bd.estiff_off;
      double* dst = estiff[b];
      const size_t n = (size_t)bd.ek_rows * bd.span;
      for (size_t k = 0; k < n; ++k) dst[k] = src[k];
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nth; ++t) th.emplace_back(work, t);
  work(0);
  for (auto& t : th) t.join();
  return 0;
}

}  // namespace

extern "C" {

const char* w3g_last_error(void) { return g_err.c_str(); }

int w3g_create(int device, const w3g_model_desc* md, w3g_context** out) {
  if (!md || !out) return fail(W3G_EARG, "null argument");
  *out = nullptr;
  if (md->nelblk <= 0 || md->noelem <= 0 || !md->elblks || !md->props || !md->iprops || !md->lprops ||
      !md->edest || !md->cdest)
    return fail(W3G_EARG, "incomplete model description");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
    return fail(W3G_ECUDA, "CUDA device " + std::to_string(device) + " not available");
  CK(cudaSetDevice(device));

  w3g_context* c = new w3g_context();
  c->device = device;
  DeviceModel& m = c->m;
  m.nelblk = md->nelblk; m.noelem = md->noelem; m.nodof = md->nodof; m.ncoord = md->ncoord;
  m.qbar = md->qbar_flag ? 1 : 0;
  m.beta_fact = md->beta_fact;
  m.bbar_beta = (1.0 - md->eps_bbar) * (1.0 / 3.0);   // bmod.f: beta = (one - eps_stab)*third
  m.asym = md->asymmetric_assembly ? 1 : 0;

  // ---- block table (elblks, iprops, lprops) ----
  std::vector<BlockDesc>& B = c->blocks;
  B.resize(md->nelblk);
  long long gp = 0, cep = 0, est = 0, einf = 0, geo = 0, hist = 0;
  int expect_felem = 1, n_mm10_gp = 0;
  bool any_umat = false;
  std::vector<Chunk> type_chunks[kNumTypes], ttype_chunks[kNumTypes], mm10_chunks;
  std::vector<int> mm10_gp;
  for (int b = 0; b < md->nelblk; ++b) {
    BlockDesc& d = B[b];
    d.span = md->elblks[3 * b];
    int felem1 = md->elblks[3 * b + 1];
    if (d.span < 1 || d.span > W3G_MXVL || felem1 < 1 || felem1 + d.span - 1 > md->noelem) {
      delete c;
      return fail(W3G_EARG, "block " + std::to_string(b + 1) + ": bad span/felem");
    }
    if (felem1 != expect_felem) {
      delete c;
      return fail(W3G_EARG, "blocks must cover elements 1..noelem in order");
    }
    expect_felem = felem1 + d.span;
    d.felem = felem1 - 1;
    const int* ip = md->iprops + (size_t)d.felem * W3G_MXELPR;
    const int* lp = md->lprops + (size_t)d.felem * W3G_MXELPR;
    d.etype = ip[0]; d.nnode = ip[1]; d.ngp = ip[5]; d.mat = ip[24];
    d.totdof = d.nnode * ip[3];
    d.utsz = (d.totdof * d.totdof - d.totdof) / 2 + d.totdof;
    d.ek_rows = md->asymmetric_assembly ? d.totdof * d.totdof : d.utsz;   // tanstf.f:223-225
    if (md->asymmetric_assembly && d.etype != W3G_ETYPE_L3DISOP && d.mat == W3G_MAT_CRYSTAL) {
      delete c;
      return fail(W3G_EUNSUPPORTED, "block " + std::to_string(b + 1) + ": mm10 needs 8-node bricks");
    }
    // b-bar is an option of the 8-node brick (elprp.f); other types ignore lprops(19)
    d.geonl = lp[17] != 0; d.bbar = lp[18] != 0 && d.etype == W3G_ETYPE_L3DISOP;
    // (etype, nnode, ngp, integration order) with a GPU path
    const bool ok_type = ip[3] == 3 &&
                         ((d.etype == W3G_ETYPE_L3DISOP && d.nnode == 8 && d.ngp == 8 && ip[4] == 1) ||
                          (d.etype == W3G_ETYPE_Q3DISOP && d.nnode == 20 && d.ngp == 27 && ip[4] == 1) ||
                          (d.etype == W3G_ETYPE_TET10 && d.nnode == 10 && d.ngp == 4 && ip[4] == 4));
    if (!ok_type) {
      delete c;
      return fail(W3G_EUNSUPPORTED, "block " + std::to_string(b + 1) + ": element type not supported");
    }
    if (d.mat != W3G_MAT_BILINEAR && d.mat != W3G_MAT_CRYSTAL && d.mat != W3G_MAT_UMAT) {
      delete c;
      return fail(W3G_EUNSUPPORTED, "block " + std::to_string(b + 1) + ": material model not supported");
    }
    if (d.mat == W3G_MAT_UMAT && !md->umat_props) {
      delete c;
      return fail(W3G_EARG, "block " + std::to_string(b + 1) + ": UMAT elements without umat_props");
    }
    // WARP3D hands a UMAT the F-bar gradients of b-bar bricks
    // (gtmat1_make_fbar), which are not formed here
    if (d.mat == W3G_MAT_UMAT && d.bbar) {
      delete c;
      return fail(W3G_EUNSUPPORTED, "block " + std::to_string(b + 1) + ": UMAT with b-bar");
    }
    if (d.mat == W3G_MAT_CRYSTAL) {
      if (d.etype != W3G_ETYPE_L3DISOP) {
        delete c;
        return fail(W3G_EUNSUPPORTED, "block " + std::to_string(b + 1) + ": mm10 needs 8-node bricks");
      }
      if (!md->crystals || md->ncrystals <= 0 || !md->elem_crystal || !md->elem_angles || !(md->dt > 0.0)) {
        delete c;
        return fail(W3G_EARG, "block " + std::to_string(b + 1) + ": mm10 without crystal data or dt");
      }
      for (int i = 0; i < d.span; ++i) {
        const int cn = md->elem_crystal[d.felem + i];
        if (cn < 0 || cn >= md->ncrystals) {
          delete c;
          return fail(W3G_EARG, "element " + std::to_string(d.felem + i + 1) + ": bad crystal index");
        }
        const w3g_crystal& cr = md->crystals[cn];
        if ((cr.slip_type != 1 && cr.slip_type != 2) || cr.elastic_type != 1 || cr.h_type != 1) {
          delete c;
          return fail(W3G_EUNSUPPORTED, "crystal " + std::to_string(cn) +
                                            ": only fcc or bcc (12-system) slip, isotropic elasticity, Voce hardening");
        }
      }
    }
    // mm10 blocks with b-bar: WARP3D also forms F-bar (gtmat1_make_fbar),
    // which only UMATs read (rstgp1.f:3786-3787); mm10 sees the b-bar
    // strain increment, internal forces and tangent, as built here
    if (d.bbar) m.has_bbar = 1;
    d.gp_off = gp; d.cep_off = cep; d.estiff_off = est; d.einf_off = einf; d.geo_off = geo;
    d.hist = d.mat == W3G_MAT_CRYSTAL ? kHistMM10 : d.mat == W3G_MAT_UMAT ? kUmatNstatv : kHistMM01;
    if (d.mat == W3G_MAT_UMAT) any_umat = true;
    d.hist_off = hist;
    d.mm10_off = d.mat == W3G_MAT_CRYSTAL ? n_mm10_gp : -1;
    hist += (long long)d.hist * d.span * d.ngp;
    if (d.mat == W3G_MAT_CRYSTAL) {
      for (int i = 0; i < d.span; ++i)
        for (int g = 0; g < d.ngp; ++g) mm10_gp.push_back((b << 12) | (i << 3) | g);
      n_mm10_gp += d.span * d.ngp;
    }
    gp += (long long)d.span * d.ngp;
    cep += 21LL * d.span * d.ngp;
    est += (long long)d.ek_rows * d.span;
    einf += (long long)d.totdof * d.span;
    geo += (long long)(3 * d.nnode + 1) * d.span * d.ngp;
    const int ts = type_slot(d.etype);
    if (d.mat == W3G_MAT_CRYSTAL) {   // recovered by the mm10 kernels
      for (int i0 = 0; i0 < d.span; i0 += kChunk) mm10_chunks.push_back(Chunk{b, i0, std::min(kChunk, d.span - i0), 3});
    } else {
      for (int i0 = 0, per = kRecoverChunk[ts]; i0 < d.span; i0 += per)
        type_chunks[ts].push_back(Chunk{b, i0, std::min(per, d.span - i0), ts});
    }
    for (int i0 = 0, per = kTangentChunk[ts]; i0 < d.span; i0 += per)
      ttype_chunks[ts].push_back(Chunk{b, i0, std::min(per, d.span - i0), ts});
  }
  std::vector<Chunk> chunks, tchunks;
  for (int t = 0; t < kNumTypes; ++t) {
    m.type_chunk0[t] = (int)chunks.size();
    m.type_chunks[t] = (int)type_chunks[t].size();
    chunks.insert(chunks.end(), type_chunks[t].begin(), type_chunks[t].end());
    m.ttype_chunk0[t] = (int)tchunks.size();
    m.ttype_chunks[t] = (int)ttype_chunks[t].size();
    tchunks.insert(tchunks.end(), ttype_chunks[t].begin(), ttype_chunks[t].end());
  }
  m.ntchunks = (int)tchunks.size();
  c->h_tchunks = tchunks;
  // tensor-core tiles of 8-node bricks: gradient-pair tiles of 16
  // elements, b-bar blocks in tiles of 5 (the B-bar operand kernel)
  std::vector<Chunk> tcchunks;
  std::vector<TcgTile> tcgtiles;
  for (int b = 0; b < md->nelblk; ++b) {
    const BlockDesc& d = B[b];
    if (d.etype != W3G_ETYPE_L3DISOP) continue;
    if (d.bbar)
      for (int i0 = 0; i0 < d.span; i0 += 5) tcchunks.push_back(Chunk{b, i0, std::min(5, d.span - i0), 0});
    else
      for (int i0 = 0; i0 < d.span; i0 += 16)
        tcgtiles.push_back(TcgTile{i0, std::min(16, d.span - i0), d.span,
                                   (d.geonl ? 1 : 0) | (d.mat == W3G_MAT_CRYSTAL ? 2 : 0), d.cep_off, d.gp_off,
                                   d.estiff_off, d.einf_off, d.hist_off, 0});
  }
  // tensor-core records of 20-node bricks: up to 8 consecutive elements
  std::vector<TcgTile> tc20tiles;
  for (int b = 0; b < md->nelblk; ++b) {
    const BlockDesc& d = B[b];
    if (d.etype != W3G_ETYPE_Q3DISOP) continue;
    for (int i0 = 0; i0 < d.span; i0 += 8)
      tc20tiles.push_back(TcgTile{i0, std::min(8, d.span - i0), d.span, d.geonl ? 1 : 0, d.cep_off, d.gp_off,
                                  d.estiff_off, d.einf_off, d.hist_off, 0});
  }
  m.ntcchunks = (int)tcchunks.size();
  m.ntcgtiles = (int)tcgtiles.size();
  m.ntc20tiles = (int)tc20tiles.size();
  m.nrchunks = (int)chunks.size();
  m.mm10_chunk0 = (int)chunks.size();
  m.mm10_chunks = (int)mm10_chunks.size();
  m.n_mm10_gp = n_mm10_gp;
  // schedule orders: block order, and heaviest item type first (estimated
  // work per item: recovery ~ elements x Gauss points x (30 + nodes),
  // tangent ~ elements x Gauss points x node pairs)
  auto orders = [&](const std::vector<Chunk>& ch, const int* per, bool tangent, std::vector<int>* out) {
    out[0].resize(ch.size());
    for (size_t k = 0; k < ch.size(); ++k) out[0][k] = (int)k;
    const int nn[kNumTypes] = {8, 20, 10}, ng[kNumTypes] = {8, 27, 4};
    double cost[kNumTypes];
    for (int t = 0; t < kNumTypes; ++t)
      cost[t] = (double)per[t] * ng[t] * (tangent ? nn[t] * (nn[t] + 1) / 2 : 30 + nn[t]);
    out[1] = out[0];
    std::stable_sort(out[1].begin(), out[1].end(), [&](int x, int y) { return cost[ch[x].type] > cost[ch[y].type]; });
  };
  std::vector<int> rord[2], tord[2];
  orders(chunks, kRecoverChunk, false, rord);   // the three element types only
  orders(tchunks, kTangentChunk, true, tord);
  chunks.insert(chunks.end(), mm10_chunks.begin(), mm10_chunks.end());
  if (expect_felem != md->noelem + 1) {
    delete c;
    return fail(W3G_EARG, "blocks do not cover all elements");
  }
  m.ngp_total = gp; m.cep_total = cep; m.estiff_total = est; m.einf_total = einf; m.geo_total = geo;
  // asymmetric assembly: packed offsets of the 20-node brick / tetrahedron
  // blocks in the scratch array their matrices are expanded from
  std::vector<BlockDesc> Bp(B);
  if (m.asym)
    for (int b = 0; b < md->nelblk; ++b)
      if (B[b].etype != W3G_ETYPE_L3DISOP) {
        Bp[b].estiff_off = m.packed_total;
        m.packed_total += (long long)B[b].utsz * B[b].span;
      }
  m.hist_total = hist;
  m.nchunks = (int)chunks.size();

  // ---- edest / cdest, ifv CSR ----
  std::vector<int> ed(einf), cd(einf);
  for (int b = 0; b < md->nelblk; ++b) {
    size_t n = (size_t)B[b].totdof * B[b].span;
    std::memcpy(&ed[B[b].einf_off], md->edest[b], n * sizeof(int));
    std::memcpy(&cd[B[b].einf_off], md->cdest[b], n * sizeof(int));
  }
  std::vector<int> rowptr(md->nodof + 1, 0);
  for (int b = 0; b < md->nelblk; ++b) {
    const BlockDesc& d = B[b];
    for (int i = 0; i < d.span; ++i)
      for (int j = 0; j < d.totdof; ++j) {
        int gd = ed[d.einf_off + (size_t)i * d.totdof + j];
        int gc = cd[d.einf_off + (size_t)i * d.totdof + j];
        if (gd < 1 || gd > md->nodof || gc < 1 || gc > md->ncoord) {
          delete c;
          return fail(W3G_EARG, "edest/cdest index out of range in block " + std::to_string(b + 1));
        }
        rowptr[gd]++;
      }
  }
  for (int k = 0; k < md->nodof; ++k) rowptr[k + 1] += rowptr[k];
  std::vector<long long> src(einf);
  {
    std::vector<int> fill(rowptr.begin(), rowptr.end() - 1);
    // ascending einfvec index: block, then dof j, then element i
    for (int b = 0; b < md->nelblk; ++b) {
      const BlockDesc& d = B[b];
      for (int j = 0; j < d.totdof; ++j)
        for (int i = 0; i < d.span; ++i) {
          int gd = ed[d.einf_off + (size_t)i * d.totdof + j] - 1;
          src[fill[gd]++] = d.einf_off + (long long)j * d.span + i;
        }
    }
  }
  // ---- material properties (setup_mm01_rknstr) ----
  std::vector<MatProps> mat(md->noelem);
  for (int e = 0; e < md->noelem; ++e) {
    const float* p = md->props + (size_t)e * W3G_MXELPR;
    const int* lp = md->lprops + (size_t)e * W3G_MXELPR;
    mat[e].e = p[6]; mat[e].nu = p[7]; mat[e].beta = p[13]; mat[e].h = p[14]; mat[e].yld = p[22];
    mat[e].lnelas = lp[16] ? 1.0 : 0.0;
    fill_mat_constants(mat[e]);
  }
  // mm10: per-element crystal data (setup_mm10_rknstr) and definitions
  std::vector<CrystalElem> xtal;
  std::vector<CrystalType> xtype;
  if (n_mm10_gp > 0) {
    xtal.resize(md->noelem);
    std::memset(xtal.data(), 0, xtal.size() * sizeof(CrystalElem));
    for (int b = 0; b < md->nelblk; ++b) {
      const BlockDesc& d = B[b];
      if (d.mat != W3G_MAT_CRYSTAL) continue;
      for (int i = 0; i < d.span; ++i) {
        const int e = d.felem + i;
        const int cn = md->elem_crystal[e];
        build_crystal_elem(md->crystals[cn], cn, md->elem_angles + 3 * (size_t)e, xtal[e]);
      }
    }
    xtype.resize(md->ncrystals);
    for (int k = 0; k < md->ncrystals; ++k) {
      const w3g_crystal& cr = md->crystals[k];
      CrystalType& t = xtype[k];
      t.rate_n = cr.harden_n; t.tau_y = cr.tau_y; t.tau_v = cr.tau_v; t.theta_0 = cr.theta_o;
      t.voche_m = cr.voche_m; t.iD_v = cr.iD_v; t.k_0 = cr.k_o; t.burgers = cr.b;
      t.atol = cr.atol; t.atol1 = cr.atol1; t.rtol = cr.rtol; t.rtol1 = cr.rtol1;
      t.miter = cr.miter; t.pad = 0;
    }
    m.dt = md->dt;
  }
  std::vector<double> dnt[kNumTypes] = {std::vector<double>(dn_table_size<Hex8>()),
                                        std::vector<double>(dn_table_size<Hex20>()),
                                        std::vector<double>(dn_table_size<Tet10>())};
  fill_dn_table<Hex8>(dnt[0].data());
  fill_dn_table<Hex20>(dnt[1].data());
  fill_dn_table<Tet10>(dnt[2].data());
  std::vector<float> dnt32[kNumTypes];
  for (int t = 0; t < kNumTypes; ++t) dnt32[t].assign(dnt[t].begin(), dnt[t].end());
  {
    int dev_sms = 0;
    CK(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, device));
    m.nsm = dev_sms;
  }

  DeviceState& s = c->s;
  cudaError_t e = cudaSuccess;
#define AL(p, n) if (e == cudaSuccess) e = dalloc(&(p), (size_t)(n))
  AL(m.blocks, md->nelblk);
  AL(m.chunks, m.nchunks);
  AL(m.tchunks, m.ntchunks);
  AL(m.tcchunks, m.ntcchunks);
  AL(m.tcgtiles, m.ntcgtiles);
  AL(m.tc20tiles, m.ntc20tiles);
  AL(s.tc_timeout, 1);
  for (int k = 0; k < 2; ++k) {
    AL(m.rorder[k], m.nrchunks);
    AL(m.torder[k], m.ntchunks);
  }
  AL(s.params, 1);
  AL(s.counters, 3);
  if (n_mm10_gp > 0) {
    AL(m.xtal, md->noelem);
    AL(m.xtype, md->ncrystals);
    AL(m.mm10_gp, n_mm10_gp);
    AL(s.mm10_scr, (long long)kMm10Scratch * n_mm10_gp);
    AL(s.mm10_iters, n_mm10_gp);
    AL(s.mm10_order, n_mm10_gp);
    AL(s.mm10_ident, n_mm10_gp);
    AL(s.mm10_bins, 128);
  }
  AL(m.edest, einf + kBulkPad);   // int arrays: 16 bytes of slack for the tiles' index-slab copies
  AL(m.cdest, einf + kBulkPad);
  AL(m.mat, md->noelem);
  if (any_umat) AL(m.umat_props, (long long)W3G_UMAT_NPROPS * md->noelem);
  for (int t = 0; t < kNumTypes; ++t) {
    AL(m.dn[t], dnt[t].size());
    AL(m.dn32[t], dnt32[t].size());
  }
  AL(m.ifv_rowptr, md->nodof + 1);
  AL(m.ifv_src, einf);
  AL(s.hist, hist);
  AL(s.hist1, hist);
  AL(s.urcs_n, 9 * gp);
  AL(s.urcs_n1, 9 * gp + kBulkPad);
  AL(s.eps_n, 6 * gp);
  AL(s.eps_n1, 6 * gp);
  AL(s.rot_n1, 9 * gp + kBulkPad);
  AL(s.cep, cep + kBulkPad);
  AL(s.estiff, est);
  if (m.packed_total > 0) {
    AL(m.blocks_packed, md->nelblk);
    AL(s.estiff_packed, m.packed_total);
  }
  AL(s.einf, einf);
  AL(s.evol, md->noelem);
  AL(s.geo, geo);
  AL(s.c_geo, md->ncoord);
  AL(s.geo_dirty, 1);
  AL(s.partials, 2 * m.nchunks);
  c->ifv_parts = assemble_ifv_parts(md->nodof);
  AL(s.ifv_partials, c->ifv_parts);
  AL(s.status, 2);   // [0] step-cut key, [1] scratch counter of w3g_check_finite
  AL(s.d_info, 1);
  AL(s.d_c, md->ncoord);
  AL(s.d_u, md->nodof);
  AL(s.d_du, md->nodof);
  AL(s.d_ifv, md->nodof);
#undef AL
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    free_all(c);
    delete c;
    return fail(W3G_ENOMEM, std::string("device allocation: ") + cudaGetErrorString(e));
  }
  cudaStream_t st = c->stream;
#define UP(d, h, n) if (e == cudaSuccess) e = cudaMemcpyAsync(d, h, (size_t)(n) * sizeof(*(h)), cudaMemcpyHostToDevice, st)
  UP(m.blocks, B.data(), md->nelblk);
  if (m.packed_total > 0) UP(m.blocks_packed, Bp.data(), md->nelblk);
  UP(m.chunks, chunks.data(), m.nchunks);
  UP(m.tchunks, tchunks.data(), m.ntchunks);
  UP(m.tcchunks, tcchunks.data(), m.ntcchunks);
  UP(m.tcgtiles, tcgtiles.data(), m.ntcgtiles);
  UP(m.tc20tiles, tc20tiles.data(), m.ntc20tiles);
  for (int k = 0; k < 2; ++k) {
    UP(m.rorder[k], rord[k].data(), m.nrchunks);
    UP(m.torder[k], tord[k].data(), m.ntchunks);
  }
  UP(m.edest, ed.data(), einf);
  UP(m.cdest, cd.data(), einf);
  UP(m.mat, mat.data(), md->noelem);
  if (any_umat) UP(m.umat_props, md->umat_props, (long long)W3G_UMAT_NPROPS * md->noelem);
  if (n_mm10_gp > 0) {
    UP(m.xtal, xtal.data(), md->noelem);
    UP(m.xtype, xtype.data(), md->ncrystals);
    UP(m.mm10_gp, mm10_gp.data(), n_mm10_gp);
    for (int k = 0; k < n_mm10_gp; ++k) mm10_gp[k] = k;   // reused as the natural order
    UP(s.mm10_ident, mm10_gp.data(), n_mm10_gp);
  }
  for (int t = 0; t < kNumTypes; ++t) {
    UP(m.dn[t], dnt[t].data(), dnt[t].size());
    UP(m.dn32[t], dnt32[t].data(), dnt32[t].size());
  }
  UP(m.ifv_rowptr, rowptr.data(), md->nodof + 1);
  UP(m.ifv_src, src.data(), einf);
#undef UP
  // WARP3D's initial state: zeros, rotations = identity (src/reopen.f:1912-1915)
  double* zs[] = {s.hist, s.hist1, s.urcs_n, s.urcs_n1, s.eps_n, s.eps_n1, s.cep, s.estiff, s.einf, s.evol};
  long long zn[] = {hist, hist, 9 * gp, 9 * gp, 6 * gp, 6 * gp, cep, est, einf, md->noelem};
  for (int k = 0; k < 10 && e == cudaSuccess; ++k) e = cudaMemsetAsync(zs[k], 0, (size_t)zn[k] * sizeof(double), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(s.geo_dirty, 0xff, sizeof(int), st);   // nonzero: not built
  if (e == cudaSuccess) e = cudaMemsetAsync(s.counters, 0, 3 * sizeof(int), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(s.tc_timeout, 0, sizeof(int), st);
  if (e == cudaSuccess && n_mm10_gp > 0) e = cudaMemsetAsync(s.mm10_iters, 0, (size_t)n_mm10_gp * sizeof(int), st);
  if (e == cudaSuccess) e = init_kernels();
  if (e == cudaSuccess) {
    k_init_rot<<<(unsigned)((gp + 255) / 256), 256, 0, st>>>(s.rot_n1, gp);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    free_all(c);
    delete c;
    return fail(W3G_ECUDA, std::string("model upload: ") + cudaGetErrorString(e));
  }
  *out = c;
  return 0;
}

int w3g_destroy(w3g_context* c) {
  if (!c) return 0;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  free_all(c);
  delete c;
  return 0;
}

int w3g_set_tangent_precision(w3g_context* c, int precision) {
  if (!c) return fail(W3G_EARG, "null context");
  if (precision < W3G_TANGENT_FP64 || precision > W3G_TANGENT_BF16X3) return fail(W3G_EARG, "bad precision");
  if (c->m.asym && precision >= W3G_TANGENT_TF32)
    return fail(W3G_EUNSUPPORTED, "asymmetric assembly: FP64 and FP32 tangents only");
  CK(cudaSetDevice(c->device));
  if (precision != W3G_TANGENT_FP64 && !c->s.estiff32) {
    CK(dalloc(&c->s.estiff32, (size_t)c->m.estiff_total));
    CK(cudaMemsetAsync(c->s.estiff32, 0, (size_t)c->m.estiff_total * sizeof(float), c->stream));
  }
  if (precision != W3G_TANGENT_FP64 && c->m.packed_total > 0 && !c->s.estiff_packed32)
    CK(dalloc(&c->s.estiff_packed32, (size_t)c->m.packed_total));
  c->precision = precision;
  return 0;
}

int w3g_umat_features(int* info) {
  if (!info) return fail(W3G_EARG, "null argument");
  for (int k = 0; k < 4; ++k) info[k] = kUmatInfo[k];
  return 0;
}

int w3g_set_update_mode(w3g_context* c, int mode) {
  if (!c) return fail(W3G_EARG, "null context");
  if (mode != W3G_UPDATE_COPY && mode != W3G_UPDATE_SWAP) return fail(W3G_EARG, "unknown update mode");
  c->update_mode = mode;
  return 0;
}

int w3g_set_wait_limit(w3g_context* c, long long polls) {
  if (!c) return fail(W3G_EARG, "null context");
  c->wait_limit = polls < 0 ? W3G_WAIT_LIMIT_DEFAULT : polls;
  return 0;
}

int w3g_state_upload(w3g_context* c, const w3g_block_state* h) {
  if (!c || !h) return fail(W3G_EARG, "null argument");
  CK(cudaSetDevice(c->device));
  int r = 0;
  if (h->history && (r = hist_h2d(c, c->s.hist, h->history))) return r;
  if (h->history1 && (r = hist_h2d(c, c->s.hist1, h->history1))) return r;
  if (h->urcs_n && (r = blocks_h2d(c, c->s.urcs_n, h->urcs_n, 9, true))) return r;
  if (h->urcs_n1 && (r = blocks_h2d(c, c->s.urcs_n1, h->urcs_n1, 9, true))) return r;
  if (h->eps_n && (r = blocks_h2d(c, c->s.eps_n, h->eps_n, 6, true))) return r;
  if (h->eps_n1 && (r = blocks_h2d(c, c->s.eps_n1, h->eps_n1, 6, true))) return r;
  if (h->rot_n1 && (r = blocks_h2d(c, c->s.rot_n1, h->rot_n1, 9, true))) return r;
  if (h->cep && (r = blocks_h2d(c, c->s.cep, h->cep, 21, true))) return r;
  if (h->element_vol && (r = blocks_h2d(c, c->s.evol, h->element_vol, 1, false))) return r;
  if (h->einfvec) {
    for (int b = 0; b < c->m.nelblk; ++b) {
      const BlockDesc& bd = c->blocks[b];
      if (!h->einfvec[b]) continue;
      CK(cudaMemcpyAsync(c->s.einf + bd.einf_off, h->einfvec[b], (size_t)bd.totdof * bd.span * sizeof(double),
                         cudaMemcpyHostToDevice, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
  }
  return 0;
}

int w3g_state_download(w3g_context* c, const w3g_block_state* h) {
  if (!c || !h) return fail(W3G_EARG, "null argument");
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  int r = 0;
  if (h->history && (r = hist_d2h(c, c->s.hist, h->history))) return r;
  if (h->history1 && (r = hist_d2h(c, c->s.hist1, h->history1))) return r;
  if (h->urcs_n && (r = blocks_d2h(c, c->s.urcs_n, h->urcs_n, 9, true))) return r;
  if (h->urcs_n1 && (r = blocks_d2h(c, c->s.urcs_n1, h->urcs_n1, 9, true))) return r;
  if (h->eps_n && (r = blocks_d2h(c, c->s.eps_n, h->eps_n, 6, true))) return r;
  if (h->eps_n1 && (r = blocks_d2h(c, c->s.eps_n1, h->eps_n1, 6, true))) return r;
  if (h->rot_n1 && (r = blocks_d2h(c, c->s.rot_n1, h->rot_n1, 9, true))) return r;
  if (h->cep && (r = blocks_d2h(c, c->s.cep, h->cep, 21, true))) return r;
  if (h->element_vol && (r = blocks_d2h(c, c->s.evol, h->element_vol, 1, false))) return r;
  if (h->einfvec) {
    for (int b = 0; b < c->m.nelblk; ++b) {
      const BlockDesc& bd = c->blocks[b];
      if (!h->einfvec[b]) continue;
      CK(cudaMemcpyAsync(h->einfvec[b], c->s.einf + bd.einf_off, (size_t)bd.totdof * bd.span * sizeof(double),
                         cudaMemcpyDeviceToHost, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
  }
  return 0;
}

int w3g_tanstf(w3g_context* c, int step, int iter, const double* hc, const double* hu, const double* hdu,
               double* const* estiff) {
  CallScope scope_("w3g_tanstf", c ? &c->t_tangent : nullptr, c ? &c->n_tangent : nullptr);
  (void)step; (void)iter;
  if (!c || !hc || !hu || !hdu) return fail(W3G_EARG, "null argument");
  CK(cudaSetDevice(c->device));
  cudaStream_t st = c->stream;
  CK(cudaMemcpyAsync(c->s.d_c, hc, (size_t)c->m.ncoord * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->s.d_u, hu, (size_t)c->m.nodof * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->s.d_du, hdu, (size_t)c->m.nodof * sizeof(double), cudaMemcpyHostToDevice, st));
  if (estiff && c->precision == W3G_TANGENT_FP64 && c->sched.mode == W3G_SCHED_PER_TYPE && !c->m.asym)
    return tanstf_overlapped(c, estiff, st);
  int r = run_tangent(c, c->s.d_c, c->s.d_u, c->s.d_du, st);
  if (r) return r;
  if (estiff && c->precision == W3G_TANGENT_FP64) {
    r = copy_estiff_range(c, estiff, 0, c->m.nelblk, st);
    if (r) return r;
  } else if (estiff) {
    r = download_estiff32(c, estiff, st);   // FP32 forms: widened on the host
    if (r) return r;
  }
  CK(cudaStreamSynchronize(st));
  if (c->precision >= W3G_TANGENT_TF32) {
    int timeout = 0;
    CK(cudaMemcpy(&timeout, c->s.tc_timeout, sizeof(int), cudaMemcpyDeviceToHost));
    if (timeout) {   // reported once: the flag starts clear for the next call
      CK(cudaMemset(c->s.tc_timeout, 0, sizeof(int)));
      return fail(W3G_EFATAL, "tensor-core tangent: a bounded wait gave up (Ke of the unfinished tiles set to NaN)");
    }
  }
  return 0;
}

int w3g_recover(w3g_context* c, int step, int iter, int extrapolated_du, const double* hc, const double* hu,
                const double* hdu, double* hifv, w3g_recover_info* info) {
  CallScope scope_("w3g_recover", c ? &c->t_recover : nullptr, c ? &c->n_recover : nullptr);
  if (!c || !hc || !hu || !hdu) return fail(W3G_EARG, "null argument");
  CK(cudaSetDevice(c->device));
  cudaStream_t st = c->stream;
  CK(cudaMemcpyAsync(c->s.d_c, hc, (size_t)c->m.ncoord * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->s.d_u, hu, (size_t)c->m.nodof * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->s.d_du, hdu, (size_t)c->m.nodof * sizeof(double), cudaMemcpyHostToDevice, st));
  int r = run_recover(c, step, iter, extrapolated_du, c->s.d_c, c->s.d_u, c->s.d_du, c->s.d_ifv, st);
  if (r) return r;
  w3g_recover_info hi;
  CK(cudaMemcpyAsync(&hi, c->s.d_info, sizeof(hi), cudaMemcpyDeviceToHost, st));
  if (hifv) CK(cudaMemcpyAsync(hifv, c->s.d_ifv, (size_t)c->m.nodof * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (info) *info = hi;
  if (hi.material_cut_step) {
    if (hifv) std::memset(hifv, 0, (size_t)c->m.nodof * sizeof(double));
    return hi.material_cut_step;   // W3G_STEP_CUT or W3G_LOCAL_FAIL
  }
  return 0;
}

int w3g_update(w3g_context* c) {
  CallScope scope_("w3g_update", c ? &c->t_update : nullptr, c ? &c->n_update : nullptr);
  if (!c) return fail(W3G_EARG, "null context");
  CK(cudaSetDevice(c->device));
  const long long gp = c->m.ngp_total;
  cudaStream_t st = c->stream;
  if (c->update_mode == W3G_UPDATE_SWAP) {
    CK(cudaStreamSynchronize(st));   // no kernel of this context may still use the arrays
    std::swap(c->s.hist, c->s.hist1);
    std::swap(c->s.eps_n, c->s.eps_n1);
    std::swap(c->s.urcs_n, c->s.urcs_n1);
    // the mm10 local solve starts from history1: its blocks keep n+1 = n
    // (runs of consecutive mm10 blocks copied together)
    const auto& B = c->blocks;
    for (size_t b = 0; b < B.size();) {
      if (B[b].mat != W3G_MAT_CRYSTAL) { ++b; continue; }
      const long long off = B[b].hist_off;
      long long n = 0;
      for (; b < B.size() && B[b].mat == W3G_MAT_CRYSTAL; ++b) n += (long long)B[b].hist * B[b].span * B[b].ngp;
      CK(cudaMemcpyAsync(c->s.hist1 + off, c->s.hist + off, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice,
                         st));
    }
    // the cached iteration graph holds the exchanged pointers
    if (c->graph.exec) {
      CK(cudaGraphExecDestroy(c->graph.exec));
      c->graph.exec = nullptr;
    }
    CK(cudaStreamSynchronize(st));
    return 0;
  }
  CK(cudaMemcpyAsync(c->s.hist, c->s.hist1, (size_t)c->m.hist_total * sizeof(double), cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(c->s.eps_n, c->s.eps_n1, (size_t)6 * gp * sizeof(double), cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(c->s.urcs_n, c->s.urcs_n1, (size_t)9 * gp * sizeof(double), cudaMemcpyDeviceToDevice, st));
  CK(cudaStreamSynchronize(st));
  return 0;
}

int w3g_tanstf_dev(w3g_context* c, int step, int iter, const void* d_c, const void* d_u, const void* d_du,
                   void* stream) {
  CallScope scope_("w3g_tanstf_dev", c ? &c->t_tangent : nullptr, c ? &c->n_tangent : nullptr);
  (void)step; (void)iter;
  if (!c || !d_c || !d_u || !d_du) return fail(W3G_EARG, "null argument");
  CK(cudaSetDevice(c->device));
  return run_tangent(c, (const double*)d_c, (const double*)d_u, (const double*)d_du, (cudaStream_t)stream);
}

int w3g_recover_dev(w3g_context* c, int step, int iter, int extrapolated_du, const void* d_c, const void* d_u,
                    const void* d_du, void* d_ifv, void* stream) {
  CallScope scope_("w3g_recover_dev", c ? &c->t_recover : nullptr, c ? &c->n_recover : nullptr);
  if (!c || !d_c || !d_u || !d_du || !d_ifv) return fail(W3G_EARG, "null argument");
  CK(cudaSetDevice(c->device));
  return run_recover(c, step, iter, extrapolated_du, (const double*)d_c, (const double*)d_u, (const double*)d_du,
                     (double*)d_ifv, (cudaStream_t)stream);
}

namespace {

bool valid_schedule(const Schedule& sc) {
  return (sc.mode == W3G_SCHED_PER_TYPE || sc.mode == W3G_SCHED_PERSISTENT) && sc.recover_ctas_per_sm >= 0 &&
         sc.tangent_ctas_per_sm >= 0 && sc.recover_grain >= 1 && sc.tangent_grain >= 1 &&
         (sc.order == W3G_ORDER_BLOCKS || sc.order == W3G_ORDER_HEAVY_FIRST);
}

bool same_schedule(const Schedule& x, const Schedule& y) {
  return x.mode == y.mode && x.recover_ctas_per_sm == y.recover_ctas_per_sm &&
         x.tangent_ctas_per_sm == y.tangent_ctas_per_sm && x.recover_grain == y.recover_grain &&
         x.tangent_grain == y.tangent_grain && x.order == y.order;
}

Schedule from_abi(const w3g_schedule& s) {
  return Schedule{s.mode, s.recover_ctas_per_sm, s.tangent_ctas_per_sm, s.recover_grain, s.tangent_grain, s.order};
}

w3g_schedule to_abi(const Schedule& s) {
  return w3g_schedule{s.mode, s.recover_ctas_per_sm, s.tangent_ctas_per_sm, s.recover_grain, s.tangent_grain, s.order};
}

// enqueues the capturable part of one iteration (after k_begin_recover);
// returns the number of kernel launches or a negative status
int enqueue_iteration(w3g_context* c, int what, const double* d_c, const double* d_u, const double* d_du,
                      double* d_ifv, cudaStream_t st) {
  int n = 0;
  if (what & W3G_ITER_RECOVER) {
    const int r = enqueue_recover(c, d_c, d_u, d_du, d_ifv, st);
    if (r < 0) return r;
    n += r;
  }
  if (what & W3G_ITER_TANGENT) {
    const int r = enqueue_tangent(c, d_c, d_u, d_du, st);
    if (r < 0) return r;
    n += r;
  }
  return n;
}

// (re)captures the iteration graph when what, pointers, precision or the
// schedule differ from the cached one
int ensure_graph(w3g_context* c, int what, const void* d_c, const void* d_u, const void* d_du, void* d_ifv) {
  IterationGraph& g = c->graph;
  if (g.exec && g.what == what && g.precision == c->precision && g.c == d_c && g.u == d_u && g.du == d_du &&
      g.ifv == d_ifv && same_schedule(g.sched, c->sched) && g.wait_limit == c->wait_limit)
    return 0;
  if (g.exec) {
    CK(cudaGraphExecDestroy(g.exec));
    g.exec = nullptr;
  }
  cudaStream_t cs = c->stream;
  CK(cudaStreamSynchronize(cs));
  CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
  const int n = enqueue_iteration(c, what, (const double*)d_c, (const double*)d_u, (const double*)d_du,
                                  (double*)d_ifv, cs);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(cs, &graph);
  if (n < 0) {
    if (graph) cudaGraphDestroy(graph);
    return n;
  }
  if (e != cudaSuccess) return fail(W3G_ECUDA, std::string("iteration capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&g.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    g.exec = nullptr;
    return fail(W3G_ECUDA, std::string("iteration graph: ") + cudaGetErrorString(e));
  }
  g.what = what;
  g.precision = c->precision;
  g.c = d_c; g.u = d_u; g.du = d_du; g.ifv = d_ifv;
  g.sched = c->sched;
  g.wait_limit = c->wait_limit;
  g.launches = n;
  return 0;
}

// runs `what` once under schedule sc (directly, not as a graph) and
// returns its device time in ms, or a negative value on error
double time_once(w3g_context* c, const Schedule& sc, int what, int step, int iter, int extrap, const double* d_c,
                 const double* d_u, const double* d_du, double* d_ifv, cudaStream_t st, cudaEvent_t e0,
                 cudaEvent_t e1) {
  const Schedule keep = c->sched;
  c->sched = sc;
  float ms = -1.f;
  int r = 0;
  if (what & W3G_ITER_RECOVER) r = begin_recover(c, step, iter, extrap, st);
  if (!r && cudaEventRecord(e0, st) == cudaSuccess) {
    const int n = enqueue_iteration(c, what, d_c, d_u, d_du, d_ifv, st);
    if (n >= 0 && cudaEventRecord(e1, st) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess)
      cudaEventElapsedTime(&ms, e0, e1);
  }
  c->sched = keep;
  return ms;
}

}  // namespace

int w3g_set_schedule(w3g_context* c, const w3g_schedule* sched) {
  if (!c || !sched) return fail(W3G_EARG, "null argument");
  const Schedule sc = from_abi(*sched);
  if (!valid_schedule(sc)) return fail(W3G_EARG, "bad schedule");
  c->sched = sc;
  return 0;
}

int w3g_get_schedule(w3g_context* c, w3g_schedule* sched) {
  if (!c || !sched) return fail(W3G_EARG, "null argument");
  *sched = to_abi(c->sched);
  return 0;
}

}  // extern "C"

namespace w3g {
int enqueue_element_iteration(w3g_context* c, int what, const double* d_c, const double* d_u, const double* d_du,
                              double* d_ifv, cudaStream_t st) {
  return enqueue_iteration(c, what, d_c, d_u, d_du, d_ifv, st);
}
int enqueue_begin_recover(w3g_context* c, int step, int iter, int extrapolated_du, cudaStream_t st) {
  return begin_recover(c, step, iter, extrapolated_du, st);
}
const w3g_recover_info* device_recover_info(const w3g_context* c) { return c->s.d_info; }
}  // namespace w3g

extern "C" {

int w3g_iteration_dev(w3g_context* c, int step, int iter, int extrapolated_du, int what, const void* d_c,
                      const void* d_u, const void* d_du, void* d_ifv, void* stream) {
  if (!c || !d_c || !d_u || !d_du) return fail(W3G_EARG, "null argument");
  if (what <= 0 || what > (W3G_ITER_RECOVER | W3G_ITER_TANGENT)) return fail(W3G_EARG, "bad what");
  if ((what & W3G_ITER_RECOVER) && !d_ifv) return fail(W3G_EARG, "null ifv");
  CK(cudaSetDevice(c->device));
  int r = ensure_graph(c, what, d_c, d_u, d_du, d_ifv);
  if (r) return r;
  cudaStream_t st = (cudaStream_t)stream;
  int n = 0;
  if (what & W3G_ITER_RECOVER) {
    if ((r = begin_recover(c, step, iter, extrapolated_du, st))) return r;
    n = 1;
  }
  CK(cudaGraphLaunch(c->graph.exec, st));
  c->last_launches = n + c->graph.launches;
  return 0;
}

int w3g_autotune(w3g_context* c, int step, int iter, int extrapolated_du, const void* d_c, const void* d_u,
                 const void* d_du, void* d_ifv, void* stream, int reps, w3g_schedule* best, double* best_ms) {
  if (!c || !d_c || !d_u || !d_du || !d_ifv) return fail(W3G_EARG, "null argument");
  CK(cudaSetDevice(c->device));
  reps = std::max(1, reps);
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const double* pc = (const double*)d_c;
  const double* pu = (const double*)d_u;
  const double* pdu = (const double*)d_du;
  double* pifv = (double*)d_ifv;
  auto measure = [&](const Schedule& sc, int what) {
    double t = time_once(c, sc, what, step, iter, extrapolated_du, pc, pu, pdu, pifv, st, e0, e1);   // warm-up
    if (t < 0) return -1.0;
    double best_t = 1e300;
    for (int k = 0; k < reps; ++k) {
      t = time_once(c, sc, what, step, iter, extrapolated_du, pc, pu, pdu, pifv, st, e0, e1);
      if (t < 0) return -1.0;
      best_t = std::min(best_t, t);
    }
    return best_t;
  };
  // candidates: per-type launches, or the persistent kernels with each
  // CTAs-per-SM count up to occupancy, queue grain 1 or 4, either order
  const int occ_r = persistent_recover_occupancy();
  const int occ_t = persistent_tangent_occupancy(c->m, c->precision != W3G_TANGENT_FP64);
  double total_best = 1e300;
  Schedule chosen = c->sched;
  int status = 0;
  for (int order = 0; order < 2 && !status; ++order) {
    for (int mode = 0; mode < 2 && !status; ++mode) {
      if (mode == W3G_SCHED_PER_TYPE && order == W3G_ORDER_BLOCKS) continue;   // order unused per type
      Schedule base{mode, 0, 0, 1, 1, order};
      double tr = 1e300, tt = 1e300;
      Schedule br = base, bt = base;
      std::vector<int> rc = {0}, tc = {0}, grains = {1};
      if (mode == W3G_SCHED_PERSISTENT) {
        rc.clear(); tc.clear();
        for (int k = 1; k <= occ_r; ++k) rc.push_back(k);
        for (int k = std::max(1, occ_t / 4); k <= occ_t; k += std::max(1, occ_t / 4)) tc.push_back(k);
        grains = {1, 4};
      }
      for (int g : grains)
        for (int k : rc) {
          Schedule sc = base;
          sc.recover_ctas_per_sm = k;
          sc.recover_grain = g;
          const double t = measure(sc, W3G_ITER_RECOVER);
          if (t < 0) { status = fail(W3G_ECUDA, "autotune: recovery run failed"); break; }
          if (t < tr) { tr = t; br = sc; }
        }
      for (int g : grains)
        for (int k : tc) {
          if (status) break;
          Schedule sc = base;
          sc.tangent_ctas_per_sm = k;
          sc.tangent_grain = g;
          const double t = measure(sc, W3G_ITER_TANGENT);
          if (t < 0) { status = fail(W3G_ECUDA, "autotune: tangent run failed"); break; }
          if (t < tt) { tt = t; bt = sc; }
        }
      if (!status && tr + tt < total_best) {
        total_best = tr + tt;
        chosen = base;
        chosen.recover_ctas_per_sm = br.recover_ctas_per_sm;
        chosen.recover_grain = br.recover_grain;
        chosen.tangent_ctas_per_sm = bt.tangent_ctas_per_sm;
        chosen.tangent_grain = bt.tangent_grain;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (status) return status;
  c->sched = chosen;
  // leave the state of one iteration with these arguments
  int r = begin_recover(c, step, iter, extrapolated_du, st);
  if (!r) {
    const int n = enqueue_iteration(c, W3G_ITER_RECOVER | W3G_ITER_TANGENT, pc, pu, pdu, pifv, st);
    if (n < 0) r = n;
  }
  if (r) return r;
  CK(cudaStreamSynchronize(st));
  if (best) *best = to_abi(chosen);
  if (best_ms) *best_ms = total_best;
  return 0;
}

int w3g_local_iterations(w3g_context* c, int* counts, int n) {
  if (!c || (!counts && n > 0)) return fail(W3G_EARG, "null argument");
  CK(cudaSetDevice(c->device));
  if (n != c->m.n_mm10_gp) return fail(W3G_EARG, "count array length must equal the mm10 Gauss points");
  if (n == 0) return 0;
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaMemcpy(counts, c->s.mm10_iters, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost));
  return 0;
}

int w3g_recover_info_get(w3g_context* c, w3g_recover_info* info) {
  if (!c || !info) return fail(W3G_EARG, "null argument");
  CK(cudaSetDevice(c->device));
  CK(cudaMemcpy(info, c->s.d_info, sizeof(*info), cudaMemcpyDeviceToHost));
  return info->material_cut_step;
}

int w3g_estiff_device(w3g_context* c, void** d_estiff, long long* count) {
  if (!c || !d_estiff || !count) return fail(W3G_EARG, "null argument");
  *d_estiff = c->precision != W3G_TANGENT_FP64 ? (void*)c->s.estiff32 : (void*)c->s.estiff;
  *count = c->m.estiff_total;
  return 0;
}

int w3g_last_launch_count(w3g_context* c) { return c ? c->last_launches : 0; }


int w3g_timers_get(w3g_context* c, w3g_timers* t) {
  if (!c || !t) return fail(W3G_EARG, "null argument");
  t->tangent_s = c->t_tangent;
  t->recover_s = c->t_recover;
  t->update_s = c->t_update;
  t->tangent_calls = c->n_tangent;
  t->recover_calls = c->n_recover;
  t->update_calls = c->n_update;
  return 0;
}

int w3g_timers_reset(w3g_context* c) {
  if (!c) return fail(W3G_EARG, "null context");
  c->t_tangent = c->t_recover = c->t_update = 0.0;
  c->n_tangent = c->n_recover = c->n_update = 0;
  return 0;
}

int w3g_check_finite(w3g_context* c, long long* bad) {
  if (!c || !bad) return fail(W3G_EARG, "null argument");
  CK(cudaSetDevice(c->device));
  cudaStream_t st = c->stream;
  unsigned long long* d_bad = reinterpret_cast<unsigned long long*>(c->s.status) + 1;   // scratch word
  CK(cudaMemsetAsync(d_bad, 0, sizeof(unsigned long long), st));
  const long long gp = c->m.ngp_total;
  cudaError_t e = count_nonfinite(c->s.urcs_n1, 9 * gp, d_bad, st);
  if (e == cudaSuccess) e = count_nonfinite(c->s.eps_n1, 6 * gp, d_bad, st);
  if (e == cudaSuccess) e = count_nonfinite(c->s.hist1, c->m.hist_total, d_bad, st);
  if (e == cudaSuccess) e = count_nonfinite(c->s.einf, c->m.einf_total, d_bad, st);
  if (e == cudaSuccess) {
    if (c->precision == W3G_TANGENT_FP64) e = count_nonfinite(c->s.estiff, c->m.estiff_total, d_bad, st);
    else e = count_nonfinite(c->s.estiff32, c->m.estiff_total, d_bad, st);
  }
  if (e != cudaSuccess) return fail(W3G_ECUDA, std::string("w3g_check_finite: ") + cudaGetErrorString(e));
  unsigned long long h = 0;
  CK(cudaMemcpyAsync(&h, d_bad, sizeof(h), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  *bad = (long long)h;
  return 0;
}

int w3g_device_name(int device, char* name, int len) {
  if (!name || len <= 0) return fail(W3G_EARG, "null argument");
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, device));
  std::strncpy(name, prop.name, (size_t)len - 1);
  name[len - 1] = '\0';
  return 0;
}

}  // extern "C"

int w3g_fail(int code, const std::string& msg) { return fail(code, msg); }
