// snapshot.cu — the Canvaz painting file (src/session.rs:6-99, 248-310).
//
// Layout (little-endian):
//   "PSIM", u32 version 1, u32 w, u32 h,
//   f32 tilt_deg, f32 tilt_dir_deg, f32 cure_rate, f32 h_max, f32 s_max,
//   f64 total_deposited                                   (44 bytes)
//   u32 part count (8: the planes of Film::read_state, src/film/mod.rs:1277-1301)
//   per part: u64 length, u32 chunk count, per chunk: u64 size + chunk
// A part is cut into 32 MiB pieces; each chunk is the piece's uncompressed
// size (u32) followed by an LZ4 block (the format of lz4_flex 0.11's
// compress_prepend_size).  The LZ4 block coder below is written from the
// published LZ4 block format: sequences of a token (literal length, match
// length - 4), literals, a 16-bit match offset; the last 5 bytes of a block
// are literals and no match starts in its last 12.
//
// Host code only; chunks are (de)compressed on all host threads.
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <new>
#include <vector>

#include "film_handle.h"

namespace {

constexpr size_t CHUNK = 32u << 20;
constexpr uint32_t VERSION = 1;
constexpr size_t HEADER = 44;
constexpr int MINMATCH = 4, LASTLITERALS = 5, MFLIMIT = 12, HASH_BITS = 16;

uint32_t read32(const uint8_t* p) {
  uint32_t v;
  std::memcpy(&v, p, 4);
  return v;
}
uint32_t hash4(uint32_t v) { return (v * 2654435761u) >> (32 - HASH_BITS); }

size_t lz4_bound(size_t n) { return n + n / 255 + 16; }

// Writes a length continuation (the part above 15) as 255s and a remainder.
bool put_len(uint8_t*& op, const uint8_t* end, size_t len) {
  for (; len >= 255; len -= 255) {
    if (op >= end) return false;
    *op++ = 255;
  }
  if (op >= end) return false;
  *op++ = (uint8_t)len;
  return true;
}

// LZ4 block of src[0, n) into dst (capacity cap); returns its size, 0 when
// it does not fit.  Greedy: one 4-byte hash table, matches extended forward.
size_t lz4_compress(const uint8_t* src, size_t n, uint8_t* dst, size_t cap) {
  std::vector<int64_t> table((size_t)1 << HASH_BITS, -1);
  uint8_t* op = dst;
  const uint8_t* oend = dst + cap;
  size_t ip = 0, anchor = 0;
  auto emit = [&](size_t lit_end, size_t offset, size_t mlen, bool last) -> bool {
    const size_t lit = lit_end - anchor;
    if (op >= oend) return false;
    uint8_t* token = op++;
    *token = (uint8_t)((lit >= 15 ? 15 : lit) << 4);
    if (lit >= 15 && !put_len(op, oend, lit - 15)) return false;
    if ((size_t)(oend - op) < lit) return false;
    std::memcpy(op, src + anchor, lit);
    op += lit;
    if (last) return true;
    if (oend - op < 2) return false;
    *op++ = (uint8_t)(offset & 0xff);
    *op++ = (uint8_t)(offset >> 8);
    const size_t ml = mlen - MINMATCH;
    *token |= (uint8_t)(ml >= 15 ? 15 : ml);
    if (ml >= 15 && !put_len(op, oend, ml - 15)) return false;
    return true;
  };
  if (n >= (size_t)MFLIMIT + 1) {
    const size_t match_limit = n - LASTLITERALS;  // a match ends at or before this
    while (ip + MFLIMIT <= n) {
      const uint32_t seq = read32(src + ip);
      const uint32_t h = hash4(seq);
      const int64_t ref = table[h];
      table[h] = (int64_t)ip;
      if (ref >= 0 && ip - (size_t)ref <= 65535 && read32(src + ref) == seq) {
        size_t len = MINMATCH;
        while (ip + len < match_limit && src[ref + len] == src[ip + len]) ++len;
        if (!emit(ip, ip - (size_t)ref, len, false)) return 0;
        ip += len;
        anchor = ip;
      } else {
        ++ip;
      }
    }
  }
  if (!emit(n, 0, 0, true)) return 0;
  return (size_t)(op - dst);
}

// Decodes an LZ4 block of n bytes into exactly out_n bytes; false when the
// block is malformed or does not decode to out_n bytes.
bool lz4_decompress(const uint8_t* src, size_t n, uint8_t* dst, size_t out_n) {
  size_t ip = 0, op = 0;
  while (ip < n) {
    const uint8_t token = src[ip++];
    size_t lit = token >> 4;
    if (lit == 15) {
      uint8_t b;
      do {
        if (ip >= n) return false;
        b = src[ip++];
        lit += b;
      } while (b == 255);
    }
    if (lit > n - ip || lit > out_n - op) return false;
    std::memcpy(dst + op, src + ip, lit);
    ip += lit;
    op += lit;
    if (ip == n) break;  // the last sequence has no match
    if (n - ip < 2) return false;
    const size_t offset = (size_t)src[ip] | ((size_t)src[ip + 1] << 8);
    ip += 2;
    if (offset == 0 || offset > op) return false;
    size_t mlen = token & 15u;
    if (mlen == 15) {
      uint8_t b;
      do {
        if (ip >= n) return false;
        b = src[ip++];
        mlen += b;
      } while (b == 255);
    }
    mlen += MINMATCH;
    if (mlen > out_n - op) return false;
    for (size_t k = 0; k < mlen; ++k) dst[op + k] = dst[op - offset + k];  // may overlap
    op += mlen;
  }
  return op == out_n;
}

void put_u32(std::vector<uint8_t>& out, uint32_t v) {
  uint8_t b[4];
  std::memcpy(b, &v, 4);
  out.insert(out.end(), b, b + 4);
}
void put_u64(std::vector<uint8_t>& out, uint64_t v) {
  uint8_t b[8];
  std::memcpy(b, &v, 8);
  out.insert(out.end(), b, b + 8);
}

// Runs fn(i) for i in [0, n) on the host's threads.
template <class Fn>
void parallel_for(size_t n, Fn fn) {
  const size_t nt = std::min<size_t>(n, std::max(1u, std::thread::hardware_concurrency()));
  std::vector<std::thread> pool;
  for (size_t t = 0; t < nt; ++t)
    pool.emplace_back([&, t] {
      for (size_t i = t; i < n; i += nt) fn(i);
    });
  for (auto& th : pool) th.join();
}

// session.rs pack(): every part in 32 MiB chunks, each size-prepended LZ4
bool pack_parts(const std::vector<std::vector<uint8_t>>& parts, std::vector<uint8_t>& out) {
  put_u32(out, (uint32_t)parts.size());
  for (const auto& p : parts) {
    const size_t nchunks = (p.size() + CHUNK - 1) / CHUNK;
    std::vector<std::vector<uint8_t>> chunks(nchunks);
    bool ok = true;
    parallel_for(nchunks, [&](size_t k) {
      const size_t off = k * CHUNK, len = std::min(CHUNK, p.size() - off);
      std::vector<uint8_t>& c = chunks[k];
      c.resize(4 + lz4_bound(len));
      const uint32_t l32 = (uint32_t)len;
      std::memcpy(c.data(), &l32, 4);
      const size_t z = lz4_compress(p.data() + off, len, c.data() + 4, c.size() - 4);
      if (!z) ok = false;
      c.resize(4 + z);
    });
    if (!ok) return false;
    put_u64(out, p.size());
    put_u32(out, (uint32_t)nchunks);
    for (const auto& c : chunks) {
      put_u64(out, c.size());
      out.insert(out.end(), c.begin(), c.end());
    }
  }
  return true;
}

// session.rs unpack()
bool unpack_parts(const uint8_t* data, size_t n, std::vector<std::vector<uint8_t>>& parts) {
  size_t off = 0;
  auto take = [&](size_t k, const uint8_t*& p) -> bool {
    if (k > n - off) return false;
    p = data + off;
    off += k;
    return true;
  };
  const uint8_t* p;
  if (!take(4, p)) return false;
  const uint32_t count = read32(p);
  if (count > 64) return false;  // a painting file holds 8 parts
  parts.resize(count);
  for (uint32_t i = 0; i < count; ++i) {
    uint64_t len;
    uint32_t nchunks;
    if (!take(8, p)) return false;
    std::memcpy(&len, p, 8);
    if (!take(4, p)) return false;
    nchunks = read32(p);
    // every chunk takes at least its 8-byte length and a 4-byte raw size, and
    // holds at most CHUNK raw bytes: sizes the file cannot back are rejected
    // before anything is allocated for them
    if (nchunks > (n - off) / 12 || len > (uint64_t)nchunks * CHUNK) return false;
    std::vector<const uint8_t*> cp(nchunks);
    std::vector<uint64_t> cl(nchunks);
    for (uint32_t k = 0; k < nchunks; ++k) {
      if (!take(8, p)) return false;
      std::memcpy(&cl[k], p, 8);
      if (!take(cl[k], cp[k]) || cl[k] < 4) return false;
      if (read32(cp[k]) > CHUNK) return false;
    }
    std::vector<std::vector<uint8_t>> dec(nchunks);
    bool ok = true;
    parallel_for(nchunks, [&](size_t k) {
      const uint32_t raw = read32(cp[k]);
      dec[k].resize(raw);
      if (!lz4_decompress(cp[k] + 4, cl[k] - 4, dec[k].data(), raw)) ok = false;
    });
    if (!ok) return false;
    std::vector<uint8_t>& joined = parts[i];
    for (const auto& d : dec) joined.insert(joined.end(), d.begin(), d.end());
    if (joined.size() != len) return false;
  }
  return true;
}

// Byte sizes of the 8 state planes (reference layout, f16 pigments).
void part_sizes(size_t n, size_t out[8]) {
  const size_t s[8] = {4 * n, 4 * n, 8 * n, 16 * n, 128 * n, 16 * n, 32 * n, 4 * n};
  for (int k = 0; k < 8; ++k) out[k] = s[k];
}

}  // namespace

extern "C" {

cf_status cf_lz4_compress(const uint8_t* src, uint64_t n, uint8_t* dst, uint64_t cap, uint64_t* out_len) {
  if ((!src && n) || !dst || !out_len || n > 0xffffffffull || cap < 4) return CF_ERR_INVALID_ARG;
  const uint32_t l32 = (uint32_t)n;
  std::memcpy(dst, &l32, 4);
  const size_t z = lz4_compress(src, (size_t)n, dst + 4, (size_t)cap - 4);
  if (!z) return CF_ERR_INVALID_ARG;
  *out_len = 4 + z;
  return CF_OK;
}

cf_status cf_lz4_decompress(const uint8_t* src, uint64_t n, uint8_t* dst, uint64_t cap, uint64_t* out_len) {
  if (!src || n < 4 || !out_len) return CF_ERR_INVALID_ARG;
  const uint32_t raw = read32(src);
  *out_len = raw;
  if (!dst) return CF_OK;  // size query
  if (raw > cap || !lz4_decompress(src + 4, (size_t)n - 4, dst, raw)) return CF_ERR_INVALID_ARG;
  return CF_OK;
}

}  // extern "C"

namespace {

cf_status snapshot_save(cf_film* f, const cf_snapshot_info* info, uint8_t** out, uint64_t* out_len) {
  if (!f || !info || !out || !out_len) return fail(f, CF_ERR_INVALID_ARG, "cf_snapshot_save: null");
  size_t sz[8];
  part_sizes(f->n, sz);
  std::vector<std::vector<uint8_t>> parts(8);
  for (int k = 0; k < 8; ++k) parts[k].resize(sz[k]);
  cf_state_view v{};
  v.h = parts[0].data();
  v.m = parts[1].data();
  v.rheo = parts[2].data();
  v.strata_h = parts[3].data();
  v.strata_pig = parts[4].data();
  v.strata_cure = parts[5].data();
  v.sub_refl = parts[6].data();
  v.lay = parts[7].data();
  v.pig_format = CF_PIG_F16;
  v.device = 0;
  cf_status s = cf_read_state(f, &v);
  if (s != CF_OK) return s;
  std::vector<uint8_t> buf;
  buf.reserve(HEADER + f->n * 64);
  buf.insert(buf.end(), {'P', 'S', 'I', 'M'});
  put_u32(buf, VERSION);
  put_u32(buf, f->w);
  put_u32(buf, f->h);
  for (float x : {info->tilt_deg, info->tilt_dir_deg, info->cure_rate, info->h_max, info->s_max}) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    put_u32(buf, u);
  }
  uint64_t td;
  std::memcpy(&td, &info->total_deposited, 8);
  put_u64(buf, td);
  if (!pack_parts(parts, buf)) return fail(f, CF_ERR_INVALID_ARG, "cf_snapshot_save: compression");
  uint8_t* mem = (uint8_t*)std::malloc(buf.size());
  if (!mem) return fail(f, CF_ERR_OUT_OF_MEMORY, "cf_snapshot_save: host memory");
  std::memcpy(mem, buf.data(), buf.size());
  *out = mem;
  *out_len = buf.size();
  return CF_OK;
}

cf_status snapshot_load(cf_film* f, const uint8_t* data, uint64_t len, cf_snapshot_info* info) {
  if (!f || !data) return fail(f, CF_ERR_INVALID_ARG, "cf_snapshot_load: null");
  if (len < HEADER || std::memcmp(data, "PSIM", 4) != 0) return fail(f, CF_ERR_INVALID_ARG, "not a painting file");
  if (read32(data + 4) != VERSION) return fail(f, CF_ERR_INVALID_ARG, "painting file of another version");
  if (read32(data + 8) != f->w || read32(data + 12) != f->h)
    return fail(f, CF_ERR_INVALID_ARG, "painting file of another canvas size");
  if (info) {
    info->w = read32(data + 8);
    info->h = read32(data + 12);
    float* fl[5] = {&info->tilt_deg, &info->tilt_dir_deg, &info->cure_rate, &info->h_max, &info->s_max};
    for (int k = 0; k < 5; ++k) std::memcpy(fl[k], data + 16 + 4 * k, 4);
    std::memcpy(&info->total_deposited, data + 36, 8);
  }
  std::vector<std::vector<uint8_t>> parts;
  if (!unpack_parts(data + HEADER, (size_t)len - HEADER, parts)) return fail(f, CF_ERR_INVALID_ARG, "damaged painting file");
  size_t sz[8];
  part_sizes(f->n, sz);
  if (parts.size() != 8) return fail(f, CF_ERR_INVALID_ARG, "painting file: part count");
  for (int k = 0; k < 8; ++k)
    if (parts[k].size() != sz[k]) return fail(f, CF_ERR_INVALID_ARG, "painting file: part size");
  cf_state_view v{};
  v.h = parts[0].data();
  v.m = parts[1].data();
  v.rheo = parts[2].data();
  v.strata_h = parts[3].data();
  v.strata_pig = parts[4].data();
  v.strata_cure = parts[5].data();
  v.sub_refl = parts[6].data();
  v.lay = parts[7].data();
  v.pig_format = CF_PIG_F16;
  v.device = 0;
  return cf_write_state(f, &v);
}

}  // namespace

extern "C" {

// No exception crosses the C ABI: host memory that runs out while a file is
// packed or unpacked becomes CF_ERR_OUT_OF_MEMORY, anything else thrown
// CF_ERR_INVALID_ARG.
cf_status cf_snapshot_save(cf_film* f, const cf_snapshot_info* info, uint8_t** out, uint64_t* out_len) {
  try {
    return snapshot_save(f, info, out, out_len);
  } catch (const std::bad_alloc&) {
    return fail(f, CF_ERR_OUT_OF_MEMORY, "cf_snapshot_save: host memory");
  } catch (...) {
    return fail(f, CF_ERR_INVALID_ARG, "cf_snapshot_save");
  }
}

cf_status cf_snapshot_free(uint8_t* buf) {
  std::free(buf);
  return CF_OK;
}

cf_status cf_snapshot_load(cf_film* f, const uint8_t* data, uint64_t len, cf_snapshot_info* info) {
  try {
    return snapshot_load(f, data, len, info);
  } catch (const std::bad_alloc&) {
    return fail(f, CF_ERR_OUT_OF_MEMORY, "cf_snapshot_load: host memory");
  } catch (...) {
    return fail(f, CF_ERR_INVALID_ARG, "cf_snapshot_load");
  }
}

}  // extern "C"
