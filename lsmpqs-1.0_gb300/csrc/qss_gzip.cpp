// qss_gzip.cpp -- parallel gzip writer for the data-array files.
//
// The reference compresses every saved array by running the gzip program on
// the raw file (src/utilities/qss_file.c:13-64): one core, ~40 MB/s, i.e.
// ~25 s for one 512^3 level set, which is longer than a curvature step on the
// GPU.  Here the payload is cut into chunks that are deflated on all host
// cores, each chunk as its own gzip member; a gzip file may hold several
// members back to back and every gzip reader (gunzip, zlib, Python's gzip)
// returns their concatenation, so the decompressed bytes are exactly those
// of the reference's file.  zlib is loaded at run time (no build-time
// dependency); without it the caller falls back to the gzip program.
#include <dlfcn.h>

#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

namespace {

// zlib's z_stream (zlib.h); its layout is part of zlib's stable ABI
struct ZStream {
  const unsigned char* next_in;
  unsigned avail_in;
  unsigned long total_in;
  unsigned char* next_out;
  unsigned avail_out;
  unsigned long total_out;
  const char* msg;
  void* state;
  void* zalloc;
  void* zfree;
  void* opaque;
  int data_type;
  unsigned long adler;
  unsigned long reserved;
};

constexpr int kZOk = 0, kZStreamEnd = 1, kZFinish = 4, kZDeflated = 8, kZDefaultStrategy = 0;
constexpr int kGzipWindow = 15 + 16;  // 32 KiB window, gzip wrapper
constexpr int kLevel = 1;             // fastest deflate; the payload is FP64 data
constexpr size_t kChunk = (size_t)16 << 20;

using InitFn = int (*)(ZStream*, int, int, int, int, int, const char*, int);
using DeflateFn = int (*)(ZStream*, int);
using EndFn = int (*)(ZStream*);
using BoundFn = unsigned long (*)(ZStream*, unsigned long);

struct ZLib {
  InitFn init = nullptr;
  DeflateFn deflate = nullptr;
  EndFn end = nullptr;
  BoundFn bound = nullptr;
  bool ok = false;
};

const ZLib& zlib() {
  static const ZLib lib = [] {
    ZLib z;
    void* h = dlopen("libz.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!h) return z;
    z.init = (InitFn)dlsym(h, "deflateInit2_");
    z.deflate = (DeflateFn)dlsym(h, "deflate");
    z.end = (EndFn)dlsym(h, "deflateEnd");
    z.bound = (BoundFn)dlsym(h, "deflateBound");
    z.ok = z.init && z.deflate && z.end && z.bound;
    return z;
  }();
  return lib;
}

// one gzip member holding [p, p + n)
bool member(const ZLib& z, const unsigned char* p, size_t n, std::vector<unsigned char>& out) {
  ZStream s;
  memset(&s, 0, sizeof s);
  if (z.init(&s, kLevel, kZDeflated, kGzipWindow, 8, kZDefaultStrategy, "1.2.11", (int)sizeof(ZStream)) != kZOk)
    return false;
  out.resize(z.bound(&s, (unsigned long)n) + 64);
  s.next_in = p;
  s.avail_in = (unsigned)n;
  s.next_out = out.data();
  s.avail_out = (unsigned)out.size();
  const int rc = z.deflate(&s, kZFinish);
  const size_t used = s.total_out;
  z.end(&s);
  if (rc != kZStreamEnd) return false;
  out.resize(used);
  return true;
}

bool gzip_write(const char* path, const void* head, size_t head_len, const void* data, size_t len) {
  const ZLib& z = zlib();
  if (!z.ok) return false;
  const unsigned char* d = (const unsigned char*)data;
  const size_t nchunks = (len + kChunk - 1) / kChunk;
  std::vector<std::vector<unsigned char>> parts(nchunks + 1);
  if (!member(z, (const unsigned char*)head, head_len, parts[0])) return false;
  unsigned hw = std::thread::hardware_concurrency();
  size_t nthreads = hw ? hw : 4;
  if (nthreads > nchunks) nthreads = nchunks;
  std::vector<char> ok(nchunks, 0);
  auto work = [&](size_t t) {
    for (size_t c = t; c < nchunks; c += nthreads) {
      const size_t off = c * kChunk, n = (len - off < kChunk) ? len - off : kChunk;
      ok[c] = member(z, d + off, n, parts[c + 1]) ? 1 : 0;
    }
  };
  std::vector<std::thread> pool;
  for (size_t t = 1; t < nthreads; t++) pool.emplace_back(work, t);
  if (nthreads) work(0);
  for (auto& th : pool) th.join();
  for (char o : ok)
    if (!o) return false;
  FILE* fp = fopen(path, "wb");
  if (!fp) return false;
  bool good = true;
  for (const auto& p : parts)
    if (!p.empty() && fwrite(p.data(), 1, p.size(), fp) != p.size()) good = false;
  if (fclose(fp) != 0) good = false;
  if (!good) remove(path);
  return good;
}

}  // namespace

// Writes path as gzip of head (head_len bytes) followed by data (len bytes).
// Returns false, writing nothing, when zlib is unavailable or fails (the
// caller then writes the file and runs the gzip program, as the reference).
bool qss_gzip_write(const char* path, const void* head, size_t head_len, const void* data, size_t len) {
  try {
    return gzip_write(path, head, head_len, data, len);
  } catch (...) {  // out of host memory for the compressed chunks, or no threads
    remove(path);
    return false;
  }
}
