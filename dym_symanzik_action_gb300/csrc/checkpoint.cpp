// Chain checkpoint files: a chain's links and the state that, with its group
// table, fixes the rest of its run (shape, proposal pool, seed, sweep counter,
// couplings).  Hits draw from a Philox stream keyed by (seed, sweep, link,
// hit), so a chain loaded from a checkpoint continues exactly as the chain
// that wrote it.  The reference has no checkpoint for dym-mod-metro; its only
// configuration files are llr2d.cpp's raw int32 save_cfg/load_cfg
// (llr2d.cpp:262-271) and the SU(3) dumps of dym-mod-metro-savecfg.cpp:55-86.
//
// Layout (little-endian; 80-byte header):
//    0  char[8]  "DYMCKPT1"
//    8  u32      version (1)
//   12  i32      D, Nt, Nx
//   24  u32      P, the group order
//   28  i32      proposal pool (DYM_POOL_*)
//   32  u64      FNV-1a 64 of the Cayley table (row-major uint16, little-endian)
//   40  u64      seed
//   48  u32      sweeps done (the next sweep's key component)
//   52  u32      reserved (0)
//   56  f64      beta0, beta1, beta2
//   80  u16      links[D*V], direction-major: links[d*V + site]
//  end  u64      FNV-1a 64 of the link bytes
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "engine.h"

namespace dym {

namespace {

constexpr char kMagic[8] = {'D', 'Y', 'M', 'C', 'K', 'P', 'T', '1'};
constexpr uint32_t kVersion = 1;
constexpr size_t kHeader = 80;

void put_u32(uint8_t* p, uint32_t v) {
  for (int k = 0; k < 4; ++k) p[k] = (uint8_t)(v >> (8 * k));
}
void put_u64(uint8_t* p, uint64_t v) {
  for (int k = 0; k < 8; ++k) p[k] = (uint8_t)(v >> (8 * k));
}
void put_f64(uint8_t* p, double v) {
  uint64_t u;
  std::memcpy(&u, &v, 8);
  put_u64(p, u);
}
uint32_t get_u32(const uint8_t* p) {
  uint32_t v = 0;
  for (int k = 0; k < 4; ++k) v |= (uint32_t)p[k] << (8 * k);
  return v;
}
uint64_t get_u64(const uint8_t* p) {
  uint64_t v = 0;
  for (int k = 0; k < 8; ++k) v |= (uint64_t)p[k] << (8 * k);
  return v;
}
double get_f64(const uint8_t* p) {
  const uint64_t u = get_u64(p);
  double v;
  std::memcpy(&v, &u, 8);
  return v;
}

constexpr uint64_t kFnvOffset = 0xcbf29ce484222325ull, kFnvPrime = 0x100000001b3ull;

uint64_t fnv_u16(const uint16_t* v, size_t n, uint64_t h = kFnvOffset) {
  for (size_t i = 0; i < n; ++i) {
    h = (h ^ (uint8_t)(v[i] & 0xFFu)) * kFnvPrime;
    h = (h ^ (uint8_t)(v[i] >> 8)) * kFnvPrime;
  }
  return h;
}

// V = Nt * Nx^(D-1) for a plausible shape, else 0.
uint64_t volume(int32_t D, int32_t Nt, int32_t Nx) {
  if (D < 2 || D > 8 || Nt < 1 || Nx < 1) return 0;
  uint64_t V = (uint64_t)Nt;
  for (int b = 1; b < D; ++b) {
    V *= (uint64_t)Nx;
    if (V > 0xFFFFFFFFull) return 0;
  }
  return V;
}

}  // namespace

uint64_t table_hash(const Group& g) { return fnv_u16(g.mult.data(), g.mult.size()); }

int checkpoint_write(const char* path, const dym_checkpoint_info& h, const uint16_t* links) {
  const uint64_t V = volume(h.D, h.Nt, h.Nx);
  if (!path || !links || !V) return fail(DYM_EINVAL, "checkpoint: bad shape or null argument");
  const size_t n = (size_t)V * (size_t)h.D;
  std::vector<uint8_t> head(kHeader, 0);
  std::memcpy(head.data(), kMagic, 8);
  put_u32(&head[8], kVersion);
  put_u32(&head[12], (uint32_t)h.D);
  put_u32(&head[16], (uint32_t)h.Nt);
  put_u32(&head[20], (uint32_t)h.Nx);
  put_u32(&head[24], h.order);
  put_u32(&head[28], (uint32_t)h.pool);
  put_u64(&head[32], h.table_hash);
  put_u64(&head[40], h.seed);
  put_u32(&head[48], h.sweep);
  put_f64(&head[56], h.beta0);
  put_f64(&head[64], h.beta1);
  put_f64(&head[72], h.beta2);
  std::vector<uint8_t> body(2 * n + 8);
  for (size_t i = 0; i < n; ++i) {
    body[2 * i] = (uint8_t)(links[i] & 0xFFu);
    body[2 * i + 1] = (uint8_t)(links[i] >> 8);
  }
  put_u64(&body[2 * n], fnv_u16(links, n));
  // Written beside the target and renamed over it, so an interrupted save
  // leaves the previous checkpoint in place.
  const std::string tmp = std::string(path) + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) return fail(DYM_EIO, std::string("checkpoint: cannot create ") + tmp);
  const bool ok = std::fwrite(head.data(), 1, head.size(), f) == head.size() &&
                  std::fwrite(body.data(), 1, body.size(), f) == body.size();
  if (std::fclose(f) != 0 || !ok) {
    std::remove(tmp.c_str());
    return fail(DYM_EIO, std::string("checkpoint: cannot write ") + tmp);
  }
  if (std::rename(tmp.c_str(), path) != 0) {
    std::remove(tmp.c_str());
    return fail(DYM_EIO, std::string("checkpoint: cannot rename onto ") + path);
  }
  return DYM_OK;
}

int checkpoint_read(const char* path, dym_checkpoint_info* h, std::vector<uint16_t>* links) {
  if (!path || !h) return fail(DYM_EINVAL, "checkpoint: null argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(DYM_EIO, std::string("checkpoint: cannot open ") + path);
  long size = -1;
  if (std::fseek(f, 0, SEEK_END) == 0) size = std::ftell(f);
  if (size < 0 || std::fseek(f, 0, SEEK_SET) != 0) {
    std::fclose(f);
    return fail(DYM_EIO, std::string("checkpoint: cannot read ") + path);
  }
  std::vector<uint8_t> buf((size_t)size);
  const bool rd_ok = std::fread(buf.data(), 1, buf.size(), f) == buf.size();
  std::fclose(f);
  if (!rd_ok) return fail(DYM_EIO, std::string("checkpoint: cannot read ") + path);
  if (buf.size() < kHeader || std::memcmp(buf.data(), kMagic, 8) != 0)
    return fail(DYM_EFORMAT, "checkpoint: not a chain checkpoint (bad magic or short header)");
  if (get_u32(&buf[8]) != kVersion) return fail(DYM_EFORMAT, "checkpoint: unknown version");
  dym_checkpoint_info r{};
  r.D = (int32_t)get_u32(&buf[12]);
  r.Nt = (int32_t)get_u32(&buf[16]);
  r.Nx = (int32_t)get_u32(&buf[20]);
  r.order = get_u32(&buf[24]);
  r.pool = (int32_t)get_u32(&buf[28]);
  r.table_hash = get_u64(&buf[32]);
  r.seed = get_u64(&buf[40]);
  r.sweep = get_u32(&buf[48]);
  r.beta0 = get_f64(&buf[56]);
  r.beta1 = get_f64(&buf[64]);
  r.beta2 = get_f64(&buf[72]);
  const uint64_t V = volume(r.D, r.Nt, r.Nx);
  if (!V || r.order == 0 || r.order > DYM_PMAX) return fail(DYM_EFORMAT, "checkpoint: bad shape or group order");
  const size_t n = (size_t)V * (size_t)r.D;
  if (buf.size() != kHeader + 2 * n + 8)
    return fail(DYM_EFORMAT, "checkpoint: size " + std::to_string(buf.size()) + " does not match the lattice (" +
                                 std::to_string(kHeader + 2 * n + 8) + " bytes)");
  std::vector<uint16_t> l(n);
  for (size_t i = 0; i < n; ++i) l[i] = (uint16_t)(buf[kHeader + 2 * i] | (buf[kHeader + 2 * i + 1] << 8));
  if (get_u64(&buf[kHeader + 2 * n]) != fnv_u16(l.data(), n))
    return fail(DYM_EFORMAT, "checkpoint: link checksum mismatch");
  *h = r;
  if (links) links->swap(l);
  return DYM_OK;
}

}  // namespace dym
