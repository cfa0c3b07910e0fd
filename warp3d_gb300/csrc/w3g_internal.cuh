// w3g_internal.cuh -- device-resident element-block state and the
// launch-argument structs shared by the kernels and the C-ABI layer.
//
// Layout in HBM: every blocked array of WARP3D's elem_block_data is kept
// as ONE device allocation holding all blocks back to back, block b at
// the offset in its BlockDesc. Inside a block the reference's layout is
// kept unchanged, so a block's slice can be copied to or from the
// Fortran block pointer with one memcpy:
//   (k, ngp, span) arrays (history, urcs, eps, rot): element-major, the
//       element's ngp*k values contiguous -> global element index e,
//       GP g: (gp_off + i*ngp + g)*k
//   cep (21, span, ngp): GP-major inside the block
//   estiff (utsz, span), einfvec (span, totdof)
#pragma once
#include <cstdint>
#include <string>
#include <cuda_runtime.h>
#include "../../include/w3g.h"

namespace w3g {

constexpr int kMxvl = W3G_MXVL;
constexpr int kHistMM01 = 11;      // mm01_set_sizes, src/mm01.f:976-979
constexpr int kChunk = 8;          // elements per work item (largest of the types)
// element types with a GPU path; work items are grouped by type in this
// order: 0 = 8-node brick (l3disop), 1 = 20-node brick (q3disop),
// 2 = 10-node tetrahedron (tet10)
constexpr int kNumTypes = 3;
__host__ __device__ constexpr int type_slot(int etype) {
  return etype == W3G_ETYPE_L3DISOP ? 0 : etype == W3G_ETYPE_Q3DISOP ? 1 : etype == W3G_ETYPE_TET10 ? 2 : -1;
}
// elements per work item: recovery items run on 64 threads (one per
// Gauss point, 32 lanes for the 27-point brick, 4 per tetrahedron),
// tangent items on one warp (4 lanes per 8-node brick, 32 per 20-node
// brick, 8 per tetrahedron)
constexpr int kRecoverChunk[kNumTypes] = {8, 2, 16};
constexpr int kTangentChunk[kNumTypes] = {8, 1, 4};
constexpr int kRecoverThreads = 64;
constexpr int kTangentThreads = 32;

struct BlockDesc {
  int span;
  int felem;          // 0-based first element
  int etype, nnode, ngp, totdof, utsz, mat;
  int ek_rows;        // rows of estiff per element: utsz, or totdof^2 (asymmetric assembly)
  int geonl, bbar;
  long long gp_off;     // sum of span*ngp over previous blocks
  long long cep_off;    // sum of 21*span*ngp
  long long estiff_off; // sum of ek_rows*span
  long long einf_off;   // sum of totdof*span (also edest/cdest offset)
  long long geo_off;    // sum of (3*nnode+1)*span*ngp (undeformed-geometry cache)
  long long hist_off;   // sum of hist*span*ngp (material history)
  int hist;             // history words per Gauss point (11 mm01, 158 mm10)
  int mm10_off;         // first mm10 Gauss point of the block (-1: not mm10)
};

// one work item = up to kRecoverChunk / kTangentChunk [type] consecutive
// elements of one block
struct Chunk {
  int blk;
  int i0;     // first relative element
  int n;      // number of elements
  int type;   // type_slot of the block's element type
};

// one tile (up to 16 consecutive elements of a block) of the gradient-pair
// tensor-core tangent, with the block fields the kernel reads resolved on
// the host, so that a tile costs one 64-byte load
struct TcgTile {
  int i0, n, span, flags;     // flags: 1 = finite strain (geonl), 2 = mm10 ([D] from history1)
  long long cep_off, gp_off, estiff_off, einf_off, hist_off, pad;
};
static_assert(sizeof(TcgTile) == 64, "TcgTile is one 64-byte record");

// ---- mm10 crystal plasticity (w3g_mm10.cu) -----------------------------
constexpr int kHistMM10 = 158;     // one 12-system crystal, one hardening variable
constexpr int kSlip = 12;          // slip systems (fcc or bcc)
constexpr int kMm10Scratch = 25;   // per GP: uddt 6, R(n+1) 9, F(n+1) 9, det F(n+1)
// per-element crystal data, built on the host at model creation exactly as
// setup_mm10_rknstr does (src/rknstr.f:1568-2027)
struct CrystalElem {
  double C[36];           // elastic stiffness rotated to the reference frame, column-major
  double ms[kSlip][6];    // sym(b x n) of each slip system, Voigt
  double qs[kSlip][3];    // skew(b x n) as (w23, w13, w12)
  double g[9];            // lattice -> reference rotation (rotation_g)
  double angles[3];       // initial Euler angles, degrees (Kocks)
  int type;               // crystal definition
  int pad;
};
struct CrystalType {      // scalars of a crystal definition
  double rate_n, tau_y, tau_v, theta_0, voche_m, iD_v, k_0, burgers;
  double atol, atol1, rtol, rtol1;
  int miter, pad;
};
void build_crystal_elem(const w3g_crystal& c, int type, const double* angles, CrystalElem& x);

// per-call scalars of recovery, read by the kernels from device memory so
// that a captured launch sequence can be replayed with new values
struct IterParams {
  int step, iter, nonlinear, pad;
};

// device work queue of a persistent launch: CTAs take `grain` consecutive
// entries of `items` (work-item indices, in schedule order) at a time
// from `counter`, which is zero when the launch starts
struct WorkQueue {
  const int* items;
  int nitems;
  int grain;
  int* counter;
};

// how the element work of a call is launched
struct Schedule {
  int mode;                 // W3G_SCHED_PER_TYPE or W3G_SCHED_PERSISTENT
  int recover_ctas_per_sm;  // persistent grid = SMs x this (0: occupancy limit)
  int tangent_ctas_per_sm;
  int recover_grain;
  int tangent_grain;
  int order;                // W3G_ORDER_BLOCKS or W3G_ORDER_HEAVY_FIRST
};

// per-element mm01 properties as doubles (promoted from the float32
// props table exactly as setup_mm01_rknstr does, src/rknstr.f:1036-1054),
// plus the constants of mm01/cnst1 that depend only on them, evaluated on
// the host with the reference's expressions (fill_mat_constants).
struct MatProps {
  double e, nu, beta, h, yld;
  double lnelas;      // 1.0 = always linear elastic (lprops(17))
  double inv_e;       // 1/e
  double inv_gn;      // 1/(e/two/(one+nu))         mm01_init g_n
  double shear;       // e/(two*(one+nu))           mm01_init, cnst1 g
  double hbari;       // beta*h
  double hbark;       // (one-beta)*h
  double yld_root3;   // yld/sqrt(3)                mm01_set_history kn
  double k3;          // three*e*nu/((one+nu)*(one-two*nu)) + two*shear
  double c2, c3, c4;  // elastic [D] of cnst1
  double kbulk;       // (three*l + two*g)/three   cnst1 k
  double gamma;       // one/(one + h/(three*g))   cnst1
};

inline void fill_mat_constants(MatProps& m) {
  const double one = 1.0, two = 2.0, three = 3.0;
  m.inv_e = one / m.e;
  m.inv_gn = one / (m.e / two / (one + m.nu));
  m.shear = m.e / (two * (one + m.nu));
  m.hbari = m.beta * m.h;
  m.hbark = (one - m.beta) * m.h;
  m.yld_root3 = m.yld / 1.7320508075688772;
  m.k3 = three * m.e * m.nu / ((one + m.nu) * (one - two * m.nu)) + two * m.shear;
  const double c1 = (m.e / ((one + m.nu) * (one - two * m.nu)));
  m.c2 = (one - m.nu) * c1;
  m.c3 = ((one - two * m.nu) / two) * c1;
  m.c4 = m.nu * c1;
  const double l = (m.e * m.nu) / ((one + m.nu) * (one - two * m.nu));
  m.kbulk = (three * l + two * m.shear) / three;
  m.gamma = one / (one + m.h / (three * m.shear));
}

struct DeviceModel {
  int nelblk = 0, noelem = 0, nodof = 0, ncoord = 0;
  int qbar = 1;
  double beta_fact = 1.0;
  double bbar_beta = 1.0 / 3.0;    // bmod's beta = (1 - eps_bbar) / 3
  int has_bbar = 0;                // any 8-node brick block with b-bar
  int asym = 0;                    // asymmetric assembly: full element matrices
  // asymmetric assembly with 20-node bricks or tetrahedra (mm01, symmetric
  // [D]): their packed matrices go to a scratch array first (block table
  // with packed offsets), then are expanded to the full layout
  BlockDesc* blocks_packed = nullptr;
  long long packed_total = 0;
  int nsm = 0;
  int nchunks = 0;                          // recovery work items (partials)
  int nrchunks = 0;                         // of these, items of the three element types
  int type_chunk0[kNumTypes] = {0, 0, 0};   // first recovery item of each type
  int type_chunks[kNumTypes] = {0, 0, 0};   // recovery items of each type
  int ntchunks = 0;                         // tangent work items
  int ttype_chunk0[kNumTypes] = {0, 0, 0};
  int ttype_chunks[kNumTypes] = {0, 0, 0};
  long long ngp_total = 0, cep_total = 0, estiff_total = 0, einf_total = 0, geo_total = 0, hist_total = 0;
  // mm10: recovery items of 8-node bricks with crystal plasticity
  // (type slot 3 in the recovery chunk list), Gauss points, crystal data
  int mm10_chunk0 = 0, mm10_chunks = 0;
  int n_mm10_gp = 0;
  CrystalElem* xtal = nullptr;
  CrystalType* xtype = nullptr;
  int* mm10_gp = nullptr;
  double dt = 1.0;
  BlockDesc* blocks = nullptr;     // device
  Chunk* chunks = nullptr;         // device, recovery items grouped by type
  Chunk* tchunks = nullptr;        // device, tangent items grouped by type
  Chunk* tcchunks = nullptr;       // device, tensor-core tangent tiles of b-bar 8-node bricks (<= 5 elements)
  int ntcchunks = 0;
  TcgTile* tcgtiles = nullptr;     // device, gradient-pair tensor-core tiles of the other 8-node bricks (<= 16)
  int ntcgtiles = 0;
  TcgTile* tc20tiles = nullptr;    // device, tensor-core records of 20-node bricks (<= 8 elements)
  int ntc20tiles = 0;
  // schedule orders of the work items (W3G_ORDER_BLOCKS, _HEAVY_FIRST)
  int* rorder[2] = {nullptr, nullptr};
  int* torder[2] = {nullptr, nullptr};
  int* edest = nullptr;            // device, concatenated (totdof, span)
  int* cdest = nullptr;
  MatProps* mat = nullptr;         // device, noelem
  double* umat_props = nullptr;    // device, W3G_UMAT_NPROPS * noelem when the model has UMAT elements
  double* dn[kNumTypes] = {nullptr, nullptr, nullptr};   // device, fill_dn_table per type
  float* dn32[kNumTypes] = {nullptr, nullptr, nullptr};  // device, the same in float
  // deterministic ifv assembly: CSR over global dofs of einfvec indices
  int* ifv_rowptr = nullptr;       // nodof+1
  long long* ifv_src = nullptr;    // einf_total
};

struct DeviceState {
  double* hist = nullptr;    // 11 * ngp_total
  double* hist1 = nullptr;
  double* urcs_n = nullptr;  // 9 * ngp_total
  double* urcs_n1 = nullptr;
  double* eps_n = nullptr;   // 6 * ngp_total
  double* eps_n1 = nullptr;
  double* rot_n1 = nullptr;  // 9 * ngp_total
  double* cep = nullptr;     // cep_total
  double* estiff = nullptr;  // estiff_total (FP64 form)
  float* estiff32 = nullptr; // estiff_total (FP32 form), lazily allocated
  double* estiff_packed = nullptr;   // packed_total (asymmetric assembly scratch)
  float* estiff_packed32 = nullptr;  // the same for the FP32 form, lazily allocated
  double* einf = nullptr;    // einf_total
  double* evol = nullptr;    // noelem
  // undeformed geometry per GP (dN/dX, det[J0]) and the coordinates it
  // was built from; geo_dirty = 1 until built
  double* geo = nullptr;     // geo_total: (3*nnode+1) per GP, block b at geo_off
  double* c_geo = nullptr;   // ncoord
  int* geo_dirty = nullptr;
  // per-launch scratch
  double* partials = nullptr;      // 2 * nchunks: energy, plastic work
  double* ifv_partials = nullptr;  // per CTA of the ifv assembly
  unsigned long long* status = nullptr;  // first det[F] <= 0 point, w3g::bad_point_key order
  IterParams* params = nullptr;
  int* counters = nullptr;         // work-queue heads: recovery, tangent, mm10
  int* tc_timeout = nullptr;       // set when a tensor-core tile's MMA wait gave up
  // mm10 per-GP scratch and scheduling
  double* mm10_scr = nullptr;      // kMm10Scratch * n_mm10_gp
  int* mm10_iters = nullptr;       // n_mm10_gp
  int* mm10_order = nullptr;       // n_mm10_gp, GPs sorted by last iteration count
  int* mm10_ident = nullptr;       // n_mm10_gp, natural order
  int* mm10_bins = nullptr;        // counting-sort bins
  w3g_recover_info* d_info = nullptr;
  // host-call staging
  double* d_c = nullptr;
  double* d_u = nullptr;
  double* d_du = nullptr;
  double* d_ifv = nullptr;
};

// ---- launch arguments --------------------------------------------------
struct TangentArgs {
  const double* dn[kNumTypes];   // fill_dn_table per element type
  const float* dn32[kNumTypes];  // the same tables rounded to float
  const double* hist1;           // mm10 blocks take [D] from history1(1:36)
  const BlockDesc* blocks;
  const Chunk* chunks;
  int chunk0;            // work item of blockIdx.x == 0
  const int* edest;
  const int* cdest;
  const double* c;
  const double* u;
  const double* du;
  const double* rot_n1;
  const double* urcs_n1;
  const double* cep;
  void* estiff;          // double* or float*
  int qbar;
  double beta_fact;
  double bbar_beta;      // (1 - eps_bbar) / 3
  long long wait_limit;  // polls of every bounded wait in the tensor-core kernels (0: give up at once)
};

struct RecoverArgs {
  const double* dn[kNumTypes];
  const BlockDesc* blocks;
  const Chunk* chunks;
  int chunk0;
  const int* edest;
  const int* cdest;
  const MatProps* mat;
  const double* c;
  const double* u;
  const double* du;
  const double* hist;
  double* hist1;
  const double* urcs_n;
  double* urcs_n1;
  const double* eps_n;
  double* eps_n1;
  double* rot_n1;
  double* cep;
  double* einf;
  double* evol;
  double* partials;
  unsigned long long* status;
  double* geo;
  int* geo_dirty;
  const IterParams* params;
  double beta_fact;
  double bbar_beta;          // (1 - eps_bbar) / 3
  int asym;                  // asymmetric assembly: mm10 tangents not symmetrized
  const double* umat_props;  // UMAT elements: kUmatNprops per element (noelem entries), else null
  // mm10 blocks
  const CrystalElem* xtal;   // noelem entries (mm10 elements)
  const CrystalType* xtype;
  double* mm10_scr;          // kMm10Scratch per mm10 GP
  const int* mm10_gp;        // mm10 GP -> (block << 12) | (element << 3) | gp
  int* mm10_iters;           // local Newton iterations of the last update, per mm10 GP
  int* mm10_order;           // work-queue order (device counting sort)
  const int* mm10_ident;     // natural order (W3G_ORDER_BLOCKS)
  int mm10_sorted;           // 1: sort by last iteration count
  int* mm10_bins;
  int* mm10_counter;
  double dt;
};

// ---- kernel launchers (defined in the .cu files) -----------------------
// element kernels of one call: per-type launches or one persistent launch
// (queue counters are reset inside)
// (tc: the tensor-core kernels take the 8- and 20-node bricks, per-type
// launches of the tetrahedra only)
cudaError_t launch_tangent(const DeviceModel& m, const TangentArgs& a, bool fp32, const Schedule& sc,
                           int* counter, cudaStream_t s, bool tc = false);
// 8-node brick tangents as full matrices (asymmetric assembly), per-type
// work items of type slot 0
cudaError_t launch_tangent_full(const DeviceModel& m, const TangentArgs& a, bool fp32, cudaStream_t s);
// asymmetric assembly of 20-node bricks and tetrahedra: the packed
// matrices (written through m.blocks_packed into `packed`) expanded to the
// full column-major layout of a.estiff
cudaError_t launch_expand_packed(const DeviceModel& m, const TangentArgs& a, const void* packed, bool fp32,
                                 cudaStream_t s);
// per-type launches over explicit work-item ranges (first item, count per
// type); returns the number of kernels launched through *launches
cudaError_t launch_tangent_ranges(const DeviceModel& m, const TangentArgs& a, bool fp32, const int* first,
                                  const int* count, cudaStream_t s, int* launches);
// precision forms on the tensor cores: b-bar 8-node bricks
// (w3g_tangent_tc.cu) and the other 8-node bricks, gradient-pair form
// (w3g_tangent_tcg.cu)
cudaError_t launch_tangent_tc_hex8(const DeviceModel& m, const TangentArgs& a, bool bf16, bool split,
                                   int* tc_timeout, cudaStream_t s);
cudaError_t init_tangent_tc_kernels();
cudaError_t launch_tangent_tcg_hex8(const DeviceModel& m, const TangentArgs& a, bool bf16, bool split,
                                    int* tc_timeout, cudaStream_t s);
cudaError_t init_tangent_tcg_kernels();
// the 20-node bricks on the tensor cores (w3g_tangent_tc20.cu)
cudaError_t launch_tangent_tc_hex20(const DeviceModel& m, const TangentArgs& a, bool bf16, bool split,
                                    int* tc_timeout, cudaStream_t s);
cudaError_t init_tangent_tc20_kernels();
cudaError_t launch_recover(const DeviceModel& m, const RecoverArgs& a, double* c_geo, const Schedule& sc,
                           int* counter, cudaStream_t s);
// launches of the element kernels under a schedule
int tangent_kernel_launches(const DeviceModel& m, const Schedule& sc, bool tc = false);
int recover_kernel_launches(const DeviceModel& m, const Schedule& sc);
// mm10 recovery of the crystal-plasticity items (kinematics, local
// solves from a work queue sorted by the last iteration counts, forces)
cudaError_t launch_mm10(const DeviceModel& m, const RecoverArgs& a, cudaStream_t s);
int mm10_kernel_launches(const DeviceModel& m, bool sorted);
// one-time kernel attributes (shared-memory opt-in) and occupancies;
// called at context creation, before any capture
cudaError_t init_tangent_kernels();
cudaError_t init_recover_kernels();
cudaError_t init_mm10_kernels();
inline cudaError_t init_kernels() {
  cudaError_t e = init_tangent_kernels();
  if (e == cudaSuccess) e = init_tangent_tc_kernels();
  if (e == cudaSuccess) e = init_tangent_tcg_kernels();
  if (e == cudaSuccess) e = init_tangent_tc20_kernels();
  if (e == cudaSuccess) e = init_recover_kernels();
  return e == cudaSuccess ? init_mm10_kernels() : e;
}
// one Newton iteration's element work (recovery and/or tangent, the
// W3G_ITER_* bits) enqueued on a stream, capturable; the iteration scalars
// are set by enqueue_begin_recover (not capturable: its arguments change)
int enqueue_element_iteration(w3g_context* c, int what, const double* d_c, const double* d_u, const double* d_du,
                              double* d_ifv, cudaStream_t st);
int enqueue_begin_recover(w3g_context* c, int step, int iter, int extrapolated_du, cudaStream_t st);
const w3g_recover_info* device_recover_info(const w3g_context* c);
// resident CTAs per SM of the persistent kernels
int persistent_tangent_occupancy(const DeviceModel& m, bool fp32);
int persistent_recover_occupancy();
// writes the iteration scalars and resets the step-cut status
cudaError_t launch_begin_recover(IterParams* params, unsigned long long* status, int step, int iter, int nonlinear,
                                 cudaStream_t s);
cudaError_t launch_assemble_ifv(const DeviceModel& m, const double* einf, double* ifv, double* ifv_partials,
                                int nparts, cudaStream_t s);
cudaError_t launch_finalize(const DeviceModel& m, const double* partials, const double* ifv_partials,
                            int nparts, const unsigned long long* status, w3g_recover_info* d_info, cudaStream_t s);

// Order in which WARP3D reports the element of a det[F] <= 0 point: the
// block loop returns at the first Gauss point (gpn) where any element of
// the block fails, checking F at n+1 for all elements before F at n+1/2
// (rstgp1.f:135-145, fcomp1 in gtmat1.f:649-664), and names the first
// failing element of that check. The smallest key is that point.
// kind (half_step): 0 det F(n+1) <= 0, 1 det F(n+1/2) <= 0, 2 mm10 local
// solve failed
__host__ __device__ inline unsigned long long bad_point_key(int blk, int gp, int half_step, int i) {
  return ((unsigned long long)blk << 40) | ((unsigned long long)gp << 24) | ((unsigned long long)half_step << 20) |
         (unsigned long long)i;
}
int assemble_ifv_parts(int nodof);

// message returned by w3g_last_error() (defined in w3g_api.cu)
void set_last_error(const std::string& msg);

}  // namespace w3g
