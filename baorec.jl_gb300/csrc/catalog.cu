// Catalog I/O around the reconstruction: whitespace-delimited ASCII
// catalogs (read with CSV.jl in examples/lightcone.jl:22-23 and
// examples/simulation.jl:13) and .npy output of the shifted positions
// (npzwrite of hcat(x, y, z), examples/simulation.jl:38-40).
//
// Reader: the file is mapped, split at line boundaries into one chunk per
// host thread, and each field is converted by strtof in the C locale, which
// rounds correctly to FP32; rows are concatenated in file order.  Writer: an
// (n, ncols) little-endian float32 array with fortran_order True (the
// columns one after the other, as NPZ.jl writes a Julia matrix); device
// columns stream to the file through two pinned staging buffers so the
// copy of one block overlaps the write of the previous one.
#include <fcntl.h>
#include <locale.h>
#include <stdlib.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"

namespace baorec {
namespace {

#define CAT_FAIL(code, ...) (ctx ? set_error(ctx, code, __VA_ARGS__) : set_error_noctx(code, __VA_ARGS__))

struct Mapped {
  const char* p = nullptr;
  size_t n = 0;
  int fd = -1;
  ~Mapped() {
    if (p && n) munmap(const_cast<char*>(p), n);
    if (fd >= 0) close(fd);
  }
};

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

// Start of the line after `pos` (pos itself when it already starts a line).
size_t line_start_from(const char* p, size_t n, size_t pos) {
  if (pos == 0) return 0;
  const void* nl = memchr(p + pos - 1, '\n', n - (pos - 1));
  return nl ? (size_t)((const char*)nl - p) + 1 : n;
}

struct Chunk {
  size_t begin, end;
  std::vector<std::vector<float>> cols;
  int64_t rows = 0;
  int64_t bad_line = 0;                   // first malformed line, 1-based within the chunk (0: none)
  int bad_kind = 0;                       // 1 short row, 2 unparsable field
};

// Parse the lines of [c.begin, c.end): skip blank lines and lines whose first
// non-blank character is `comment`; keep fields `cols` (0-based).
void parse_chunk(const char* p, Chunk& c, const std::vector<int>& cols, int maxcol, int comment, locale_t loc,
                 bool store) {
  std::vector<const char*> fb(maxcol + 1), fe(maxcol + 1);
  char buf[128];
  size_t i = c.begin;
  int64_t line = 1;
  while (i < c.end) {
    const char* nl = (const char*)memchr(p + i, '\n', c.end - i);
    const size_t le = nl ? (size_t)(nl - p) : c.end;
    size_t j = i;
    while (j < le && is_space(p[j])) ++j;
    if (j < le && !(comment && p[j] == (char)comment)) {
      int nf = 0;
      while (j < le && nf <= maxcol) {
        const size_t s = j;
        while (j < le && !is_space(p[j])) ++j;
        fb[nf] = p + s;
        fe[nf] = p + j;
        ++nf;
        while (j < le && is_space(p[j])) ++j;
      }
      if (nf <= maxcol) {
        if (!c.bad_line) { c.bad_line = line; c.bad_kind = 1; }
      } else if (store) {
        for (size_t q = 0; q < cols.size(); ++q) {
          const int f = cols[q];
          const size_t len = (size_t)(fe[f] - fb[f]);
          if (len == 0 || len >= sizeof(buf)) {
            if (!c.bad_line) { c.bad_line = line; c.bad_kind = 2; }
            c.cols[q].push_back(0.0f);
            continue;
          }
          memcpy(buf, fb[f], len);
          buf[len] = 0;
          char* endp = nullptr;
          const float v = strtof_l(buf, &endp, loc);
          if (endp != buf + len && !c.bad_line) { c.bad_line = line; c.bad_kind = 2; }
          c.cols[q].push_back(v);
        }
        ++c.rows;
      } else {
        ++c.rows;
      }
    }
    i = le + 1;
    ++line;
  }
}

int map_file(baorec_ctx* ctx, const char* path, Mapped& m) {
  m.fd = open(path, O_RDONLY);
  if (m.fd < 0) return CAT_FAIL(BAOREC_ERR_ARG, "read_ascii: cannot open %s", path);
  struct stat st;
  if (fstat(m.fd, &st) != 0) return CAT_FAIL(BAOREC_ERR_ARG, "read_ascii: cannot stat %s", path);
  m.n = (size_t)st.st_size;
  if (m.n == 0) return BAOREC_OK;
  void* q = mmap(nullptr, m.n, PROT_READ, MAP_PRIVATE, m.fd, 0);
  if (q == MAP_FAILED) {
    m.n = 0;
    return CAT_FAIL(BAOREC_ERR_ARG, "read_ascii: cannot map %s", path);
  }
  m.p = (const char*)q;
  return BAOREC_OK;
}

}  // namespace
}  // namespace baorec

using namespace baorec;

extern "C" int baorec_read_ascii(baorec_ctx* ctx, const char* path, const int32_t* cols, int32_t ncols, int32_t skip,
                                 int32_t comment, float** out, int64_t n_max, int64_t* n_rows, uint32_t flags) {
  if (!path || !cols || ncols < 1 || ncols > 64 || skip < 0 || !n_rows || n_max < 0)
    return CAT_FAIL(BAOREC_ERR_ARG, "read_ascii: bad arguments");
  if (out && !(flags & BAOREC_HOST) && !ctx)
    return CAT_FAIL(BAOREC_ERR_ARG, "read_ascii: device outputs need a context");
  std::vector<int> cv(cols, cols + ncols);
  int maxcol = 0;
  for (int c : cv) {
    if (c < 0) return CAT_FAIL(BAOREC_ERR_ARG, "read_ascii: negative column index");
    maxcol = std::max(maxcol, c);
  }
  Mapped m;
  int st = map_file(ctx, path, m);
  if (st != BAOREC_OK) return st;
  // the first `skip` lines are dropped whatever they hold
  size_t pos = 0;
  int64_t line0 = 1;
  for (int s = 0; s < skip && pos < m.n; ++s, ++line0) {
    const void* nl = memchr(m.p + pos, '\n', m.n - pos);
    pos = nl ? (size_t)((const char*)nl - m.p) + 1 : m.n;
  }
  const size_t body = m.n - pos;
  unsigned nt = std::thread::hardware_concurrency();
  nt = std::max(1u, std::min(nt, 64u));
  if (body < ((size_t)1 << 20)) nt = 1;
  std::vector<Chunk> ch(nt);
  for (unsigned t = 0; t < nt; ++t) {
    ch[t].begin = line_start_from(m.p, m.n, pos + body * t / nt);
    ch[t].end = t + 1 < nt ? line_start_from(m.p, m.n, pos + body * (t + 1) / nt) : m.n;
    if (t == 0) ch[t].begin = pos;
    ch[t].cols.resize(ncols);
  }
  locale_t loc = newlocale(LC_NUMERIC_MASK, "C", (locale_t)0);
  if (!loc) return CAT_FAIL(BAOREC_ERR_ARG, "read_ascii: no C locale");
  const bool store = out != nullptr;
  std::vector<std::thread> th;
  for (unsigned t = 1; t < nt; ++t)
    th.emplace_back(parse_chunk, m.p, std::ref(ch[t]), std::cref(cv), maxcol, comment, loc, store);
  parse_chunk(m.p, ch[0], cv, maxcol, comment, loc, store);
  for (auto& x : th) x.join();
  freelocale(loc);
  int64_t total = 0;
  for (auto& c : ch) {
    if (c.bad_line) {
      // file line number: the skipped lines, the lines before the chunk, the line in the chunk
      int64_t before = 0;
      for (size_t q = pos; q < c.begin; ++q) before += m.p[q] == '\n';
      return CAT_FAIL(BAOREC_ERR_ARG, "read_ascii: %s line %lld: %s", path, (long long)(line0 - 1 + before + c.bad_line),
                      c.bad_kind == 1 ? "fewer fields than the highest requested column" : "field is not a number");
    }
    total += c.rows;
  }
  *n_rows = total;
  if (!out) return BAOREC_OK;
  if (total > n_max)
    return CAT_FAIL(BAOREC_ERR_TOO_LARGE, "read_ascii: %lld rows, room for %lld", (long long)total, (long long)n_max);
  for (int q = 0; q < ncols; ++q) {
    if (!out[q]) return CAT_FAIL(BAOREC_ERR_ARG, "read_ascii: missing output column %d", q);
    int64_t off = 0;
    for (auto& c : ch) {
      const size_t bytes = c.cols[q].size() * sizeof(float);
      if (bytes) {
        if (flags & BAOREC_HOST) {
          memcpy(out[q] + off, c.cols[q].data(), bytes);
        } else {
          CK(cudaMemcpyAsync(out[q] + off, c.cols[q].data(), bytes, cudaMemcpyHostToDevice, ctx->stream));
        }
      }
      off += (int64_t)c.cols[q].size();
    }
  }
  if (!(flags & BAOREC_HOST)) CK(cudaStreamSynchronize(ctx->stream));   // the host vectors die here
  return BAOREC_OK;
}

extern "C" int baorec_write_npy(baorec_ctx* ctx, const char* path, const float* const* cols, int32_t ncols, int64_t n,
                                uint32_t flags) {
  if (!path || !cols || ncols < 1 || n < 0) return CAT_FAIL(BAOREC_ERR_ARG, "write_npy: bad arguments");
  if (!(flags & BAOREC_HOST) && !ctx) return CAT_FAIL(BAOREC_ERR_ARG, "write_npy: device columns need a context");
  for (int q = 0; q < ncols; ++q)
    if (!cols[q] && n > 0) return CAT_FAIL(BAOREC_ERR_ARG, "write_npy: missing column %d", q);
  // format 1.0: magic, version, little-endian header length, the header
  // dict padded with spaces and ended by a newline to a multiple of 64 bytes
  char dict[160];
  int dl = snprintf(dict, sizeof(dict), "{'descr': '<f4', 'fortran_order': True, 'shape': (%lld, %d), }",
                    (long long)n, (int)ncols);
  std::string hdr(dict, (size_t)dl);
  const size_t pre = 10;
  size_t total = pre + hdr.size() + 1;
  const size_t pad = (64 - total % 64) % 64;
  hdr.append(pad, ' ');
  hdr.push_back('\n');
  const size_t hl = hdr.size();
  FILE* fp = fopen(path, "wb");
  if (!fp) return CAT_FAIL(BAOREC_ERR_ARG, "write_npy: cannot create %s", path);
  unsigned char head[10] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0, (unsigned char)(hl & 0xff), (unsigned char)(hl >> 8)};
  bool ok = fwrite(head, 1, 10, fp) == 10 && fwrite(hdr.data(), 1, hl, fp) == hl;
  if (flags & BAOREC_HOST) {
    for (int q = 0; ok && q < ncols; ++q) ok = fwrite(cols[q], sizeof(float), (size_t)n, fp) == (size_t)n;
  } else if (ok && n > 0) {
    // two pinned blocks: block b+1 is copied while block b is written
    const size_t blk = (size_t)1 << 22;   // floats per block (16 MB)
    float* pin[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaError_t e = cudaMallocHost(&pin[0], blk * sizeof(float));
    if (e == cudaSuccess) e = cudaMallocHost(&pin[1], blk * sizeof(float));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
    std::vector<std::pair<const float*, size_t>> blocks;
    for (int q = 0; q < ncols; ++q)
      for (size_t o = 0; o < (size_t)n; o += blk) blocks.push_back({cols[q] + o, std::min(blk, (size_t)n - o)});
    auto issue = [&](size_t b) {
      const int s = (int)(b & 1);
      cudaError_t r = cudaMemcpyAsync(pin[s], blocks[b].first, blocks[b].second * sizeof(float),
                                      cudaMemcpyDeviceToHost, ctx->stream);
      if (r == cudaSuccess) r = cudaEventRecord(ev[s], ctx->stream);
      return r;
    };
    if (e == cudaSuccess && !blocks.empty()) e = issue(0);
    for (size_t b = 0; e == cudaSuccess && ok && b < blocks.size(); ++b) {
      if (b + 1 < blocks.size()) e = issue(b + 1);
      if (e == cudaSuccess) e = cudaEventSynchronize(ev[b & 1]);
      if (e == cudaSuccess) ok = fwrite(pin[b & 1], sizeof(float), blocks[b].second, fp) == blocks[b].second;
    }
    cudaStreamSynchronize(ctx->stream);
    for (int s = 0; s < 2; ++s) {
      if (ev[s]) cudaEventDestroy(ev[s]);
      if (pin[s]) cudaFreeHost(pin[s]);
    }
    if (e != cudaSuccess) {
      fclose(fp);
      return set_error(ctx, BAOREC_ERR_CUDA, "write_npy: %s", cudaGetErrorString(e));
    }
  }
  if (fclose(fp) != 0) ok = false;
  if (!ok) return CAT_FAIL(BAOREC_ERR_ARG, "write_npy: short write to %s", path);
  return BAOREC_OK;
}
