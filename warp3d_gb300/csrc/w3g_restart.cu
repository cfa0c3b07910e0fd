// w3g_restart.cu -- the element-block section of a WARP3D restart file.
//
// WARP3D's `save` command (store, src/store.f:329-341) writes the blocked
// element state with store_blocks (src/store.f:915-1010) as Fortran
// sequential unformatted records, and `reopen` reads it back
// (history_cep_init, stresses_init, rotation_init, strains_init in
// src/reopen.f). The records, in order:
//
//   per block: history (state n, hist x ngp x span), check record,
//              cep (21 x span x ngp), check record          [proc_type 1]
//   per block: urcs_n (9 x ngp x span), check record;  check record  [5]
//   per geonl block: rot_n1 (9 x ngp x span), check record;  check  [2]
//   per block: eps_n (6 x ngp x span), check record;  check record  [4]
//   per block: element volumes (span), check record;  check record  [6]
//
// A record is a 4-byte length, the bytes, the same 4-byte length (the
// sequential-unformatted layout of ifort and gfortran, little endian); a
// check record holds the 4-byte integer 2147483647. On reopen the n+1
// arrays start equal to the n arrays (history1, urcs_n1, eps_n1), as
// reopen.f does with vec_ops(..., 5).
//
// w3g_store_blocks writes this section for the resident state (to a new
// file, or appended to one whose earlier sections the caller has
// written); w3g_reopen_blocks reads it from a byte offset, checks every
// length and check record, and uploads it.
#include <cstdio>
#include <cstring>
#include <vector>
#include "w3g_context.cuh"

namespace {

constexpr int32_t kCheckKey = 2147483647;   // store.f: check_data_key

void put_u32le(unsigned char* p, uint32_t v) {
  p[0] = (unsigned char)(v & 0xFFu); p[1] = (unsigned char)((v >> 8) & 0xFFu);
  p[2] = (unsigned char)((v >> 16) & 0xFFu); p[3] = (unsigned char)((v >> 24) & 0xFFu);
}
uint32_t get_u32le(const unsigned char* p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

bool put_record(FILE* f, const void* data, size_t n) {
  if (n > 0x7FFFFFF0u) return false;   // larger records need Fortran subrecords
  unsigned char m[4];
  put_u32le(m, (uint32_t)n);
  return fwrite(m, 1, 4, f) == 4 && (n == 0 || fwrite(data, 1, n, f) == n) && fwrite(m, 1, 4, f) == 4;
}

bool put_key(FILE* f) {
  unsigned char k[4];
  put_u32le(k, (uint32_t)kCheckKey);
  return put_record(f, k, 4);
}

// reads one record of exactly n bytes into data
bool get_record(FILE* f, void* data, size_t n) {
  unsigned char m[4];
  if (fread(m, 1, 4, f) != 4 || get_u32le(m) != (uint32_t)n) return false;
  if (n && fread(data, 1, n, f) != n) return false;
  unsigned char t[4];
  return fread(t, 1, 4, f) == 4 && get_u32le(t) == (uint32_t)n;
}

bool get_key(FILE* f) {
  unsigned char k[4];
  return get_record(f, k, 4) && get_u32le(k) == (uint32_t)kCheckKey;
}

// host arrays of one state transfer, laid out per block
struct HostBlocks {
  std::vector<std::vector<double>> hist, cep, urcs, rot, eps, vol;
  std::vector<double*> p_hist, p_cep, p_urcs, p_rot, p_eps, p_vol;
  explicit HostBlocks(const w3g_context* c) {
    const int nb = c->m.nelblk;
    hist.resize(nb); cep.resize(nb); urcs.resize(nb); rot.resize(nb); eps.resize(nb); vol.resize(nb);
    for (int b = 0; b < nb; ++b) {
      const w3g::BlockDesc& d = c->blocks[b];
      const size_t gp = (size_t)d.span * d.ngp;
      hist[b].assign((size_t)d.hist * gp, 0.0);
      cep[b].assign(21 * gp, 0.0);
      urcs[b].assign(9 * gp, 0.0);
      rot[b].assign(9 * gp, 0.0);
      eps[b].assign(6 * gp, 0.0);
      vol[b].assign((size_t)d.span, 0.0);
      p_hist.push_back(hist[b].data()); p_cep.push_back(cep[b].data()); p_urcs.push_back(urcs[b].data());
      p_rot.push_back(rot[b].data()); p_eps.push_back(eps[b].data()); p_vol.push_back(vol[b].data());
    }
  }
  static size_t bytes(const std::vector<double>& v) { return v.size() * sizeof(double); }
};

struct File {
  FILE* f;
  explicit File(FILE* p) : f(p) {}
  ~File() { if (f) fclose(f); }
};

}  // namespace

extern "C" {

int w3g_store_blocks(w3g_context* c, const char* path, int append) {
  if (!c || !path) return w3g_fail(W3G_EARG, "null argument");
  HostBlocks h(c);
  w3g_block_state s{};
  s.history = h.p_hist.data(); s.cep = h.p_cep.data(); s.urcs_n = h.p_urcs.data();
  s.rot_n1 = h.p_rot.data(); s.eps_n = h.p_eps.data(); s.element_vol = h.p_vol.data();
  int r = w3g_state_download(c, &s);
  if (r) return r;
  File f(fopen(path, append ? "ab" : "wb"));
  if (!f.f) return w3g_fail(W3G_EARG, std::string("cannot open ") + path);
  const int nb = c->m.nelblk;
  bool ok = true;
  for (int b = 0; b < nb && ok; ++b)   // proc_type 1: history and [D]
    ok = put_record(f.f, h.hist[b].data(), HostBlocks::bytes(h.hist[b])) && put_key(f.f) &&
         put_record(f.f, h.cep[b].data(), HostBlocks::bytes(h.cep[b])) && put_key(f.f);
  for (int b = 0; b < nb && ok; ++b)   // 5: stresses at n
    ok = put_record(f.f, h.urcs[b].data(), HostBlocks::bytes(h.urcs[b])) && put_key(f.f);
  ok = ok && put_key(f.f);
  for (int b = 0; b < nb && ok; ++b)   // 2: rotations, geonl blocks
    if (c->blocks[b].geonl) ok = put_record(f.f, h.rot[b].data(), HostBlocks::bytes(h.rot[b])) && put_key(f.f);
  ok = ok && put_key(f.f);
  for (int b = 0; b < nb && ok; ++b)   // 4: strains at n
    ok = put_record(f.f, h.eps[b].data(), HostBlocks::bytes(h.eps[b])) && put_key(f.f);
  ok = ok && put_key(f.f);
  for (int b = 0; b < nb && ok; ++b)   // 6: element volumes
    ok = put_record(f.f, h.vol[b].data(), HostBlocks::bytes(h.vol[b])) && put_key(f.f);
  ok = ok && put_key(f.f);
  if (!ok || fflush(f.f) != 0) return w3g_fail(W3G_EARG, std::string("write failed: ") + path);
  return 0;
}

int w3g_reopen_blocks(w3g_context* c, const char* path, long long offset, long long* end_offset) {
  if (!c || !path || offset < 0) return w3g_fail(W3G_EARG, "null argument or negative offset");
  File f(fopen(path, "rb"));
  if (!f.f) return w3g_fail(W3G_EARG, std::string("cannot open ") + path);
  if (fseek(f.f, (long)offset, SEEK_SET) != 0) return w3g_fail(W3G_EARG, "seek failed");
  HostBlocks h(c);
  const int nb = c->m.nelblk;
  auto bad = [&](const char* what, int b) {
    return w3g_fail(W3G_EARG, std::string("restart blocks: bad ") + what + " record of block " +
                                  std::to_string(b + 1) + " (length or check record)");
  };
  for (int b = 0; b < nb; ++b) {
    if (!get_record(f.f, h.hist[b].data(), HostBlocks::bytes(h.hist[b])) || !get_key(f.f)) return bad("history", b);
    if (!get_record(f.f, h.cep[b].data(), HostBlocks::bytes(h.cep[b])) || !get_key(f.f)) return bad("cep", b);
  }
  for (int b = 0; b < nb; ++b)
    if (!get_record(f.f, h.urcs[b].data(), HostBlocks::bytes(h.urcs[b])) || !get_key(f.f)) return bad("stress", b);
  if (!get_key(f.f)) return bad("stress section end", nb - 1);
  for (int b = 0; b < nb; ++b)
    if (c->blocks[b].geonl &&
        (!get_record(f.f, h.rot[b].data(), HostBlocks::bytes(h.rot[b])) || !get_key(f.f)))
      return bad("rotation", b);
  if (!get_key(f.f)) return bad("rotation section end", nb - 1);
  for (int b = 0; b < nb; ++b)
    if (!get_record(f.f, h.eps[b].data(), HostBlocks::bytes(h.eps[b])) || !get_key(f.f)) return bad("strain", b);
  if (!get_key(f.f)) return bad("strain section end", nb - 1);
  for (int b = 0; b < nb; ++b)
    if (!get_record(f.f, h.vol[b].data(), HostBlocks::bytes(h.vol[b])) || !get_key(f.f)) return bad("volume", b);
  if (!get_key(f.f)) return bad("volume section end", nb - 1);
  if (end_offset) *end_offset = (long long)ftell(f.f);
  // n and n+1 from the same records (reopen.f: vec_ops(..., 5) copies);
  // rotations only for geonl blocks (the others keep theirs)
  std::vector<double*> p_rot(h.p_rot);
  bool any_small = false;
  for (int b = 0; b < nb; ++b)
    if (!c->blocks[b].geonl) any_small = true;
  w3g_block_state s{};
  s.history = h.p_hist.data(); s.history1 = h.p_hist.data();
  s.urcs_n = h.p_urcs.data(); s.urcs_n1 = h.p_urcs.data();
  s.eps_n = h.p_eps.data(); s.eps_n1 = h.p_eps.data();
  s.cep = h.p_cep.data(); s.element_vol = h.p_vol.data();
  if (!any_small) s.rot_n1 = p_rot.data();
  int r = w3g_state_upload(c, &s);
  if (r || !any_small) return r;
  // mixed geonl / small-displacement models: the geonl blocks' rotations
  // over the resident ones
  HostBlocks cur(c);
  w3g_block_state g{};
  g.rot_n1 = cur.p_rot.data();
  if ((r = w3g_state_download(c, &g))) return r;
  for (int b = 0; b < nb; ++b)
    if (c->blocks[b].geonl) std::memcpy(cur.rot[b].data(), h.rot[b].data(), HostBlocks::bytes(h.rot[b]));
  return w3g_state_upload(c, &g);
}

}  // extern "C"
