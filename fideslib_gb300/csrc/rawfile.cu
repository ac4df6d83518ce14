// Raw residue files (declarations and layout: include/fideslib_gb300.h, "Raw residue files").
//
// The reference moves keys and ciphertexts between OpenFHE and the GPU as raw residue arrays (RawCipherText,
// RawPlainText and RawKeySwitchKey, src/CKKS/openfhe-interface/RawCiphertext.cuh:19-93): per tower its modulus and
// N residues in evaluation form, bit-reversed, plus the scaling metadata.  OpenFHE's own serialisation (cereal)
// is not in this tree, so this file format is this library's: the same content, stored little-endian with a
// self-check, so that keys and ciphertexts can be kept on disk and reloaded into a context with the same moduli
// and roots.  It is not OpenFHE's cereal format.
//
// Layout: a 96-byte header, then rows u64 moduli, rows u64 roots (0 = not recorded), then polys x rows x N u64
// residues, then an 8-byte FNV-1a 64 hash of everything before it.
//   bytes  0..7   magic "FGBRAW01"
//          8..11  kind (fides_raw_info.kind)      12..15 log_n
//         16..19  rows                            20..23 polys
//         24..27  noise_deg                       28..31 slots
//         32..35  id (Galois element / switch-key id)
//         36..39  reserved (0)                    40..47 scale (IEEE-754 double)
//         48..95  zero
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fideslib_gb300.h"
#include "engine.hpp"

struct fides_ctx {
  fgb::Context* c;
};

namespace fgb {
int set_last_error(int code, const char* msg);
}

namespace {

constexpr char kMagic[8] = {'F', 'G', 'B', 'R', 'A', 'W', '0', '1'};
constexpr size_t kHeader = 96;

int err(int code, const std::string& m) { return fgb::set_last_error(code, m.c_str()); }

struct Fnv {
  uint64_t h = 1469598103934665603ull;
  void add(const void* p, size_t n) {
    const unsigned char* b = (const unsigned char*)p;
    for (size_t i = 0; i < n; i++) {
      h ^= b[i];
      h *= 1099511628211ull;
    }
  }
};

void put32(unsigned char* b, uint32_t v) {
  for (int i = 0; i < 4; i++) b[i] = (unsigned char)(v >> (8 * i));
}
void put64(unsigned char* b, uint64_t v) {
  for (int i = 0; i < 8; i++) b[i] = (unsigned char)(v >> (8 * i));
}
uint32_t get32(const unsigned char* b) {
  uint32_t v = 0;
  for (int i = 0; i < 4; i++) v |= (uint32_t)b[i] << (8 * i);
  return v;
}
uint64_t get64(const unsigned char* b) {
  uint64_t v = 0;
  for (int i = 0; i < 8; i++) v |= (uint64_t)b[i] << (8 * i);
  return v;
}

// Little-endian u64 arrays: on a little-endian host the bytes are the values' own.
bool host_is_le() {
  const uint32_t x = 1;
  unsigned char c;
  std::memcpy(&c, &x, 1);
  return c == 1;
}

int check_info(const fides_raw_info& in) {
  if (in.kind < FIDES_RAW_CIPHERTEXT || in.kind > FIDES_RAW_SWITCH_KEY) return err(FIDES_EINVAL, "unknown raw kind");
  if (in.log_n < 1 || in.log_n > 17 || in.rows < 1 || in.rows > 64 || in.polys < 1 || in.polys > 16)
    return err(FIDES_EINVAL, "raw header sizes out of range");
  return FIDES_OK;
}

void encode_header(const fides_raw_info& in, unsigned char* h) {
  std::memset(h, 0, kHeader);
  std::memcpy(h, kMagic, 8);
  put32(h + 8, in.kind);
  put32(h + 12, in.log_n);
  put32(h + 16, in.rows);
  put32(h + 20, in.polys);
  put32(h + 24, in.noise_deg);
  put32(h + 28, in.slots);
  put32(h + 32, in.id);
  put32(h + 36, 0);
  uint64_t sb;
  std::memcpy(&sb, &in.scale, 8);
  put64(h + 40, sb);
}

int decode_header(const unsigned char* h, fides_raw_info* out) {
  if (std::memcmp(h, kMagic, 8) != 0) return err(FIDES_EINVAL, "not a raw residue file (bad magic)");
  fides_raw_info in{};
  in.kind = get32(h + 8);
  in.log_n = get32(h + 12);
  in.rows = get32(h + 16);
  in.polys = get32(h + 20);
  in.noise_deg = get32(h + 24);
  in.slots = get32(h + 28);
  in.id = get32(h + 32);
  in.reserved = get32(h + 36);
  const uint64_t sb = get64(h + 40);
  std::memcpy(&in.scale, &sb, 8);
  if (int rc = check_info(in)) return rc;
  *out = in;
  return FIDES_OK;
}

size_t residues_of(const fides_raw_info& in) { return (size_t)in.polys * in.rows << in.log_n; }

int write_u64s(FILE* f, Fnv& h, const uint64_t* v, size_t n) {
  std::vector<unsigned char> buf;
  const size_t chunk = 1 << 16;
  for (size_t i = 0; i < n; i += chunk) {
    const size_t m = n - i < chunk ? n - i : chunk;
    buf.resize(m * 8);
    if (host_is_le()) {
      std::memcpy(buf.data(), v + i, m * 8);
    } else {
      for (size_t k = 0; k < m; k++) put64(buf.data() + 8 * k, v[i + k]);
    }
    h.add(buf.data(), buf.size());
    if (std::fwrite(buf.data(), 1, buf.size(), f) != buf.size()) return err(FIDES_EINVAL, "short write");
  }
  return FIDES_OK;
}

int read_u64s(FILE* f, Fnv& h, uint64_t* v, size_t n) {
  std::vector<unsigned char> buf;
  const size_t chunk = 1 << 16;
  for (size_t i = 0; i < n; i += chunk) {
    const size_t m = n - i < chunk ? n - i : chunk;
    buf.resize(m * 8);
    if (std::fread(buf.data(), 1, buf.size(), f) != buf.size()) return err(FIDES_EINVAL, "raw file is truncated");
    h.add(buf.data(), buf.size());
    if (host_is_le()) {
      std::memcpy(v + i, buf.data(), m * 8);
    } else {
      for (size_t k = 0; k < m; k++) v[i + k] = get64(buf.data() + 8 * k);
    }
  }
  return FIDES_OK;
}

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) std::fclose(f);
  }
};

// Reads a whole file: header, moduli, roots and residues, and checks the trailing hash.
int read_all(const char* path, fides_raw_info* info, std::vector<uint64_t>* mods, std::vector<uint64_t>* roots,
             std::vector<uint64_t>* data) {
  if (!path || !info) return err(FIDES_EINVAL, "null argument");
  File fl;
  fl.f = std::fopen(path, "rb");
  if (!fl.f) return err(FIDES_EINVAL, std::string("cannot open ") + path);
  unsigned char h[kHeader];
  if (std::fread(h, 1, kHeader, fl.f) != kHeader) return err(FIDES_EINVAL, "raw file is truncated");
  if (int rc = decode_header(h, info)) return rc;
  Fnv fnv;
  fnv.add(h, kHeader);
  mods->resize(info->rows);
  roots->resize(info->rows);
  data->resize(residues_of(*info));
  if (int rc = read_u64s(fl.f, fnv, mods->data(), mods->size())) return rc;
  if (int rc = read_u64s(fl.f, fnv, roots->data(), roots->size())) return rc;
  if (int rc = read_u64s(fl.f, fnv, data->data(), data->size())) return rc;
  unsigned char t[8];
  if (std::fread(t, 1, 8, fl.f) != 8) return err(FIDES_EINVAL, "raw file is truncated");
  if (get64(t) != fnv.h) return err(FIDES_EINVAL, "raw file is corrupt (hash mismatch)");
  for (size_t r = 0; r < data->size(); r++) {
    const uint64_t q = (*mods)[(r >> info->log_n) % info->rows];
    if (q == 0 || (*data)[r] >= q) return err(FIDES_EINVAL, "raw file holds a residue not below its modulus");
  }
  return FIDES_OK;
}

// Tower i of a file row: Q tower i for i < nq rows of a ciphertext or plaintext; keys carry all nq + np towers.
int match_context(const fgb::Context* c, const fides_raw_info& in, const std::vector<uint64_t>& mods,
                  const std::vector<uint64_t>& roots) {
  if ((int)in.log_n != c->logN) return err(FIDES_EINVAL, "raw file is for another ring dimension");
  for (uint32_t i = 0; i < in.rows; i++) {
    if (mods[i] != c->mod[i])
      return err(FIDES_EINVAL, "raw file tower " + std::to_string(i) + " has another modulus than the context");
    if (roots[i] != 0 && roots[i] != c->psi[i])
      return err(FIDES_EINVAL, "raw file tower " + std::to_string(i) + " was transformed with another root");
  }
  return FIDES_OK;
}

}  // namespace

extern "C" {

int fides_raw_write(const char* path, const fides_raw_info* info, const uint64_t* moduli, const uint64_t* roots,
                    const uint64_t* data) {
  if (!path || !info || !moduli || !data) return err(FIDES_EINVAL, "null argument");
  if (int rc = check_info(*info)) return rc;
  File fl;
  const std::string tmp = std::string(path) + ".tmp";
  fl.f = std::fopen(tmp.c_str(), "wb");
  if (!fl.f) return err(FIDES_EINVAL, std::string("cannot create ") + tmp);
  unsigned char h[kHeader];
  encode_header(*info, h);
  Fnv fnv;
  fnv.add(h, kHeader);
  if (std::fwrite(h, 1, kHeader, fl.f) != kHeader) return err(FIDES_EINVAL, "short write");
  std::vector<uint64_t> r(info->rows, 0);
  if (roots) r.assign(roots, roots + info->rows);
  if (int rc = write_u64s(fl.f, fnv, moduli, info->rows)) return rc;
  if (int rc = write_u64s(fl.f, fnv, r.data(), info->rows)) return rc;
  if (int rc = write_u64s(fl.f, fnv, data, residues_of(*info))) return rc;
  unsigned char t[8];
  put64(t, fnv.h);
  if (std::fwrite(t, 1, 8, fl.f) != 8) return err(FIDES_EINVAL, "short write");
  if (std::fclose(fl.f) != 0) {
    fl.f = nullptr;
    return err(FIDES_EINVAL, "cannot close the file");
  }
  fl.f = nullptr;
  if (std::rename(tmp.c_str(), path) != 0) return err(FIDES_EINVAL, std::string("cannot rename to ") + path);
  return FIDES_OK;
}

int fides_raw_read_info(const char* path, fides_raw_info* info) {
  if (!path || !info) return err(FIDES_EINVAL, "null argument");
  File fl;
  fl.f = std::fopen(path, "rb");
  if (!fl.f) return err(FIDES_EINVAL, std::string("cannot open ") + path);
  unsigned char h[kHeader];
  if (std::fread(h, 1, kHeader, fl.f) != kHeader) return err(FIDES_EINVAL, "raw file is truncated");
  return decode_header(h, info);
}

int fides_raw_read(const char* path, fides_raw_info* info, uint64_t* moduli, uint64_t* roots, uint64_t* data) {
  std::vector<uint64_t> m, r, d;
  fides_raw_info in{};
  if (int rc = read_all(path, &in, &m, &r, &d)) return rc;
  if (info) *info = in;
  if (moduli) std::memcpy(moduli, m.data(), m.size() * 8);
  if (roots) std::memcpy(roots, r.data(), r.size() * 8);
  if (data) std::memcpy(data, d.data(), d.size() * 8);
  return FIDES_OK;
}

int fides_ct_save(fides_ctx* ctx, uint32_t handle, const char* path) {
  if (!ctx || !ctx->c || !path) return err(FIDES_EINVAL, "null argument");
  fides_ct_meta m{};
  if (int rc = fides_ct_meta_get(ctx, handle, &m)) return rc;
  if (m.reserved) return err(FIDES_EINVAL, "extended-basis ciphertexts are not saved; KeySwitchDown first");
  const fgb::Context* c = ctx->c;
  std::vector<uint64_t> data((size_t)2 * m.towers * c->N);
  if (int rc = fides_ct_store(ctx, handle, data.data(), nullptr)) return rc;
  fides_raw_info in{FIDES_RAW_CIPHERTEXT, (uint32_t)c->logN, m.towers, 2, m.noise_deg, m.slots, 0, 0, m.scale};
  return fides_raw_write(path, &in, (const uint64_t*)c->mod.data(), (const uint64_t*)c->psi.data(), data.data());
}

int fides_ct_load_file(fides_ctx* ctx, const char* path, uint32_t* handle) {
  if (!ctx || !ctx->c || !handle) return err(FIDES_EINVAL, "null argument");
  std::vector<uint64_t> m, r, d;
  fides_raw_info in{};
  if (int rc = read_all(path, &in, &m, &r, &d)) return rc;
  if (in.kind != FIDES_RAW_CIPHERTEXT || in.polys != 2) return err(FIDES_EINVAL, "the file holds no ciphertext");
  if ((int)in.rows > ctx->c->nq) return err(FIDES_EINVAL, "more towers than the context's Q basis");
  if (int rc = match_context(ctx->c, in, m, r)) return rc;
  const fides_ct_meta meta{in.rows, in.noise_deg, in.slots, 0, in.scale};
  return fides_ct_load(ctx, d.data(), &meta, handle);
}

int fides_key_load_file(fides_ctx* ctx, const char* path) {
  if (!ctx || !ctx->c) return err(FIDES_EINVAL, "null argument");
  std::vector<uint64_t> m, r, d;
  fides_raw_info in{};
  if (int rc = read_all(path, &in, &m, &r, &d)) return rc;
  const fgb::Context* c = ctx->c;
  if (in.kind < FIDES_RAW_RELIN_KEY) return err(FIDES_EINVAL, "the file holds no key");
  if ((int)in.rows != c->ntow || (int)in.polys != 2 * c->dnum)
    return err(FIDES_EINVAL, "key shape differs from the context's [2][dnum][nq + np]");
  if (int rc = match_context(c, in, m, r)) return rc;
  switch (in.kind) {
    case FIDES_RAW_RELIN_KEY: return fides_load_eval_mult_key(ctx, d.data());
    case FIDES_RAW_ROTATION_KEY: return fides_load_rotation_key(ctx, in.id, d.data());
    default: return fides_load_switch_key(ctx, in.id, d.data());
  }
}

}  // extern "C"
