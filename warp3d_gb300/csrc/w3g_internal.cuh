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
constexpr int kTypeChunk[kNumTypes] = {8, 2, 8};   // elements per work item

struct BlockDesc {
  int span;
  int felem;          // 0-based first element
  int etype, nnode, ngp, totdof, utsz, mat;
  int geonl, bbar;
  long long gp_off;     // sum of span*ngp over previous blocks
  long long cep_off;    // sum of 21*span*ngp
  long long estiff_off; // sum of utsz*span
  long long einf_off;   // sum of totdof*span (also edest/cdest offset)
  long long geo_off;    // sum of (3*nnode+1)*span*ngp (undeformed-geometry cache)
};

// one work item = up to kTypeChunk[type] consecutive elements of one block
struct Chunk {
  int blk;
  int i0;     // first relative element
  int n;      // number of elements (<= kChunk)
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
  int nchunks = 0;
  int type_chunk0[kNumTypes] = {0, 0, 0};   // first work item of each type
  int type_chunks[kNumTypes] = {0, 0, 0};   // work items of each type
  long long ngp_total = 0, cep_total = 0, estiff_total = 0, einf_total = 0, geo_total = 0;
  BlockDesc* blocks = nullptr;     // device
  Chunk* chunks = nullptr;         // device
  int* edest = nullptr;            // device, concatenated (totdof, span)
  int* cdest = nullptr;
  MatProps* mat = nullptr;         // device, noelem
  double* dn_hex8 = nullptr;       // device, fill_dn_table<Hex8>
  double* dn_hex20 = nullptr;      // device, fill_dn_table<Hex20>
  double* dn_tet10 = nullptr;      // device, fill_dn_table<Tet10>
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
  w3g_recover_info* d_info = nullptr;
  // host-call staging
  double* d_c = nullptr;
  double* d_u = nullptr;
  double* d_du = nullptr;
  double* d_ifv = nullptr;
};

// ---- launch arguments --------------------------------------------------
struct TangentArgs {
  const double* dn;      // element table, fill_dn_table layout
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
};

struct RecoverArgs {
  const double* dn;
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
  int step, iter, nonlinear;
  double beta_fact;
};

// ---- kernel launchers (defined in the .cu files) -----------------------
cudaError_t launch_tangent_fp64(const DeviceModel& m, const TangentArgs& a, cudaStream_t s);
cudaError_t launch_tangent_fp32(const DeviceModel& m, const TangentArgs& a, cudaStream_t s);
cudaError_t launch_recover(const DeviceModel& m, const RecoverArgs& a, double* c_geo, cudaStream_t s);
// the 20-node brick and 10-node tetrahedron work items (w3g_generic.cu)
cudaError_t launch_tangent_other(const DeviceModel& m, TangentArgs a, bool fp32, cudaStream_t s);
cudaError_t launch_recover_other(const DeviceModel& m, RecoverArgs a, cudaStream_t s);
cudaError_t launch_assemble_ifv(const DeviceModel& m, const double* einf, double* ifv, double* ifv_partials,
                                int nparts, cudaStream_t s);
cudaError_t launch_finalize(const DeviceModel& m, const double* partials, const double* ifv_partials,
                            int nparts, const unsigned long long* status, w3g_recover_info* d_info, cudaStream_t s);

// Order in which WARP3D reports the element of a det[F] <= 0 point: the
// block loop returns at the first Gauss point (gpn) where any element of
// the block fails, checking F at n+1 for all elements before F at n+1/2
// (rstgp1.f:135-145, fcomp1 in gtmat1.f:649-664), and names the first
// failing element of that check. The smallest key is that point.
__host__ __device__ inline unsigned long long bad_point_key(int blk, int gp, int half_step, int i) {
  return ((unsigned long long)blk << 40) | ((unsigned long long)gp << 24) | ((unsigned long long)half_step << 20) |
         (unsigned long long)i;
}
int assemble_ifv_parts(int nodof);

// message returned by w3g_last_error() (defined in w3g_api.cu)
void set_last_error(const std::string& msg);

}  // namespace w3g
