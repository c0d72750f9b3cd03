// Matrix Market (.mtx) -> host CSR with the reference's ingest semantics:
// readMtx<float>(..., directed = 0, ...) followed by coo2csr
// (test_spmm_full.cu:99-113, backend/readMtx.hpp:351-422, :246-304,
// backend/mmio.hpp:128-228):
//   * banner "%%MatrixMarket matrix coordinate <real|integer|pattern>
//     <general|symmetric|hermitian|skew-symmetric>", fields
//     case-insensitive;
//   * comment lines start with '%'; the size line is the first other line
//     (if it does not hold three integers, integers are read on until three
//     are found, as mm_read_mtx_crd_size does);
//   * entries are 1-based "row col [value]"; pattern entries get 1.0,
//     integer values are read as integers, real values as float;
//   * no symmetrisation and no removal of duplicates or self-loops (the
//     reference's removeSelfloop call is commented out, readMtx.hpp:413): a
//     symmetric file yields only the listed triangle;
//   * entries sorted by (row, col); entries with equal (row, col) keep file
//     order (the reference's std::sort leaves their order unspecified).
// Unlike the reference, a truncated file, an index outside the stated size,
// a complex or dense ("array") file is an error instead of undefined state.
//
// Large files are parsed by several host threads: the entry section is cut
// at line starts into one piece per thread, each piece is parsed on its own,
// and the pieces are joined in file order (the first NZ entries count, the
// first error among them is reported, as a front-to-back read would).  A
// file whose entries span lines across a cut is parsed front to back.  The
// per-row column sorts and the final gather run on the same threads.
#include <algorithm>
#include <charconv>
#include <cctype>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include <unistd.h>

#include "common.cuh"

namespace {

int host_threads();
template <typename Fn>
void run_threads(int T, Fn f);

// An array that is not value-initialised when allocated (the reader fills
// every element before reading it).
template <typename T>
struct RawArray {
  std::unique_ptr<T[]> p;
  explicit RawArray(size_t n) : p(new T[n > 0 ? n : 1]) {}
  T *data() { return p.get(); }
  T &operator[](size_t i) { return p[i]; }
  const T &operator[](size_t i) const { return p[i]; }
};

// A byte buffer that is not zero-filled when allocated.
struct CharBuf {
  std::unique_ptr<char[]> p;
  size_t n = 0;
  char *data() { return p.get(); }
  const char *data() const { return p.get(); }
  size_t size() const { return n; }
  char operator[](size_t i) const { return p[i]; }
};

struct Reader {
  CharBuf buf;
  size_t pos = 0;

  // The whole file plus a terminating NUL; files over 64 MB are read by
  // several threads (pread of disjoint ranges).
  bool load(const char *path) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (n < 0) {
      std::fclose(f);
      return false;
    }
    buf.p.reset(new char[(size_t)n + 1]);
    size_t got = 0;
    const int T = host_threads();
    if (T > 1 && n > (64l << 20)) {
      const int fd = fileno(f);
      std::vector<size_t> part(T, 0);
      run_threads(T, [&](int t) {
        const size_t b = (size_t)n * t / T, e = (size_t)n * (t + 1) / T;
        size_t done = 0;
        while (b + done < e) {
          const ssize_t r = pread(fd, buf.p.get() + b + done, e - b - done, (off_t)(b + done));
          if (r <= 0) break;
          done += (size_t)r;
        }
        part[t] = done;
      });
      // the file as far as it could be read from the start
      for (int t = 0; t < T; ++t) {
        const size_t b = (size_t)n * t / T, e = (size_t)n * (t + 1) / T;
        got += part[t];
        if (b + part[t] < e) break;
      }
    } else if (n > 0) {
      got = std::fread(buf.p.get(), 1, (size_t)n, f);
    }
    std::fclose(f);
    buf.p[got] = '\0';
    buf.n = got + 1;
    return true;
  }
  bool eof() const { return pos + 1 >= buf.size(); }
  // next line without the newline; false at end of file
  bool line(std::string *out) {
    if (eof()) return false;
    size_t s = pos;
    while (pos + 1 < buf.size() && buf[pos] != '\n') ++pos;
    out->assign(buf.data() + s, pos - s);
    if (pos + 1 < buf.size()) ++pos;
    if (!out->empty() && out->back() == '\r') out->pop_back();
    return true;
  }
  void skip_ws() {
    while (pos + 1 < buf.size() && std::isspace((unsigned char)buf[pos])) ++pos;
  }
  bool read_long(long *v) {
    skip_ws();
    if (eof()) return false;
    char *end = nullptr;
    errno = 0;
    long x = std::strtol(buf.data() + pos, &end, 10);
    if (end == buf.data() + pos) return false;
    pos = (size_t)(end - buf.data());
    *v = x;
    return true;
  }
  bool read_float(float *v) {
    skip_ws();
    if (eof()) return false;
    char *end = nullptr;
    float x = std::strtof(buf.data() + pos, &end);
    if (end == buf.data() + pos) return false;
    pos = (size_t)(end - buf.data());
    *v = x;
    return true;
  }
};

// Entries parsed from one piece of the entry section [b, e): stops at the
// end of the piece, after `limit` entries, or at the first bad entry.
struct Piece {
  std::vector<int> ri, ci;
  std::vector<float> v;
  int err = 0;         // 0 none, 1 row/col missing, 2 value missing, 3 outside the matrix
  bool split = false;  // an entry continues past the end of the piece
};

// Next token start in [p, e) after whitespace, or e.
inline const char *skip(const char *p, const char *e) {
  while (p < e && std::isspace((unsigned char)*p)) ++p;
  return p;
}

// strtol / strtof on the token at p (not whitespace), through from_chars
// where that gives the same result: a decimal integer, or a float token
// starting with a digit, '-' or '.' that from_chars reads up to whitespace
// or the end of the piece.  Anything else ('+' signs, hex floats, inf / nan
// spellings, out-of-range values) goes to strtol / strtof.  Returns the end
// of the token, p when there is none.
inline const char *scan_long(const char *p, const char *e, long *out) {
  const auto r = std::from_chars(p, e, *out);
  if (r.ec == std::errc()) return r.ptr;
  char *end = nullptr;
  *out = std::strtol(p, &end, 10);
  return end;
}

inline bool ends_token(const char *q, const char *e) {
  return q == e || *q == '\0' || std::isspace((unsigned char)*q);
}

inline const char *scan_float(const char *p, const char *e, float *out) {
  const char c0 = *p, c1 = p + 1 < e ? p[1] : '\0';
  const bool numeric = (c0 >= '0' && c0 <= '9') || c0 == '.' ||
                       (c0 == '-' && ((c1 >= '0' && c1 <= '9') || c1 == '.'));
  if (numeric) {
    const auto r = std::from_chars(p, e, *out);
    if (r.ec == std::errc() && ends_token(r.ptr, e)) return r.ptr;
  }
  char *end = nullptr;
  *out = std::strtof(p, &end);
  return end;
}

void parse_piece(const char *b, const char *e, bool last, int kind, long M, long N, long limit, Piece *out) {
  const char *p = b;
  out->ri.reserve((size_t)((e - b) / 8));
  out->ci.reserve((size_t)((e - b) / 8));
  out->v.reserve((size_t)((e - b) / 8));
  long got = 0;
  while (got < limit) {
    const char *end = nullptr;
    p = skip(p, e);
    if (p == e) {  // piece exhausted between entries
      if (last) out->err = 1;
      return;
    }
    long r = 0, c = 0;
    end = scan_long(p, e, &r);
    if (end == p) {
      out->err = 1;
      return;
    }
    p = skip(end, e);
    if (p == e) {
      if (last) out->err = 1;
      else out->split = true;
      return;
    }
    end = scan_long(p, e, &c);
    if (end == p) {
      out->err = 1;
      return;
    }
    p = end;
    float val = 1.0f;
    if (kind != 2) {
      p = skip(p, e);
      if (p == e) {
        if (last) out->err = 2;
        else out->split = true;
        return;
      }
      if (kind == 0) {
        end = scan_float(p, e, &val);
      } else {
        long iv = 0;
        end = scan_long(p, e, &iv);
        val = (float)(int)iv;
      }
      if (end == p) {
        out->err = 2;
        return;
      }
      p = end;
    }
    if (r < 1 || r > M || c < 1 || c > N) {
      out->err = 3;
      return;
    }
    out->ri.push_back((int)(r - 1));
    out->ci.push_back((int)(c - 1));
    out->v.push_back(val);
    ++got;
  }
}

int host_threads() {
  const unsigned hc = std::thread::hardware_concurrency();
  return (int)std::max(1u, std::min(hc, 16u));
}

// Run f(t) for t in [0, T) on T threads (t = 0 on the calling thread).
template <typename Fn>
void run_threads(int T, Fn f) {
  std::vector<std::thread> th;
  for (int t = 1; t < T; ++t) th.emplace_back(f, t);
  f(0);
  for (auto &x : th) x.join();
}

std::string lower(std::string s) {
  for (auto &c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

}  // namespace

using namespace gbs;

extern "C" gbs_status gbs_mtx_read(const char *path, gbs_host_csr *out) {
  clear_error();
  GBS_REQUIRE(path && out, "mtx: null argument");
  std::memset(out, 0, sizeof(*out));
  Reader rd;
  if (!rd.load(path)) return fail(GBS_ERR_INVALID_ARG, std::string("mtx: cannot open ") + path);
  std::string ln;
  if (!rd.line(&ln)) return fail(GBS_ERR_INVALID_ARG, "mtx: empty file");
  char banner[64] = {0}, mtx[64] = {0}, crd[64] = {0}, dtype[64] = {0}, sym[64] = {0};
  if (std::sscanf(ln.c_str(), "%63s %63s %63s %63s %63s", banner, mtx, crd, dtype, sym) != 5)
    return fail(GBS_ERR_INVALID_ARG, "mtx: banner needs 5 fields");
  if (std::strncmp(banner, "%%MatrixMarket", 14) != 0) return fail(GBS_ERR_INVALID_ARG, "mtx: no %%MatrixMarket banner");
  const std::string m = lower(mtx), c = lower(crd), d = lower(dtype), y = lower(sym);
  if (m != "matrix") return fail(GBS_ERR_UNSUPPORTED, "mtx: object must be 'matrix'");
  if (c != "coordinate") return fail(GBS_ERR_UNSUPPORTED, "mtx: only coordinate (sparse) files are supported");
  int kind;  // 0 real, 1 integer, 2 pattern
  if (d == "real") kind = 0;
  else if (d == "integer") kind = 1;
  else if (d == "pattern") kind = 2;
  else return fail(GBS_ERR_UNSUPPORTED, "mtx: data type must be real, integer or pattern");
  if (y != "general" && y != "symmetric" && y != "hermitian" && y != "skew-symmetric")
    return fail(GBS_ERR_UNSUPPORTED, "mtx: unknown symmetry field");

  long M = 0, N = 0, NZ = 0;
  bool have = false;
  while (rd.line(&ln)) {
    if (!ln.empty() && ln[0] == '%') continue;
    if (std::sscanf(ln.c_str(), "%ld %ld %ld", &M, &N, &NZ) == 3) have = true;
    break;
  }
  if (!have) {  // mm_read_mtx_crd_size: keep reading integers until 3
    if (!(rd.read_long(&M) && rd.read_long(&N) && rd.read_long(&NZ)))
      return fail(GBS_ERR_INVALID_ARG, "mtx: missing size line");
  }
  if (M < 0 || N < 0 || NZ < 0 || M > 0x7fffffffL || N > 0x7fffffffL || NZ > 0x7fffffffL)
    return fail(GBS_ERR_INVALID_ARG, "mtx: size out of range");

  RawArray<int> ri((size_t)NZ), ci((size_t)NZ);
  RawArray<float> v((size_t)NZ);
  const int T = host_threads();
  const char *body = rd.buf.data() + rd.pos, *bend = rd.buf.data() + rd.buf.size() - 1;
  bool parallel_done = false;
  if (T > 1 && bend - body > (8l << 20) && NZ > 0) {
    // pieces start right after a newline
    std::vector<const char *> cut(T + 1);
    cut[0] = body;
    cut[T] = bend;
    for (int t = 1; t < T; ++t) {
      const char *q = body + (bend - body) * t / T;
      if (q < cut[t - 1]) q = cut[t - 1];
      while (q < bend && *q != '\n') ++q;
      cut[t] = q < bend ? q + 1 : bend;
    }
    std::vector<Piece> pc(T);
    run_threads(T, [&](int t) { parse_piece(cut[t], cut[t + 1], t == T - 1, kind, M, N, NZ, &pc[t]); });
    // pieces in file order: where each one's entries go, up to NZ entries,
    // the first split entry or the first bad one; then copied in parallel
    long have_n = 0;
    bool split = false;
    int used = 0;
    std::vector<long> off(T, 0), take(T, 0);
    for (int t = 0; t < T && have_n < NZ; ++t) {
      off[t] = have_n;
      take[t] = std::min((long)pc[t].ri.size(), NZ - have_n);
      have_n += take[t];
      used = t + 1;
      if (have_n == NZ) break;
      if (pc[t].split) {
        split = true;
        break;
      }
      if (pc[t].err == 3)
        return fail(GBS_ERR_INVALID_ARG, "mtx: entry " + std::to_string(have_n + 1) + " outside the matrix");
      if (pc[t].err == 2) return fail(GBS_ERR_INVALID_ARG, "mtx: missing value");
      if (pc[t].err == 1) return fail(GBS_ERR_INVALID_ARG, "mtx: fewer entries than the size line states");
    }
    run_threads(used, [&](int t) {
      std::copy(pc[t].ri.begin(), pc[t].ri.begin() + take[t], ri.data() + off[t]);
      std::copy(pc[t].ci.begin(), pc[t].ci.begin() + take[t], ci.data() + off[t]);
      std::copy(pc[t].v.begin(), pc[t].v.begin() + take[t], v.data() + off[t]);
    });
    if (!split) {
      if (have_n < NZ) return fail(GBS_ERR_INVALID_ARG, "mtx: fewer entries than the size line states");
      parallel_done = true;
    }
  }
  for (long e = 0; e < NZ && !parallel_done; ++e) {
    long r, cc;
    if (!rd.read_long(&r) || !rd.read_long(&cc))
      return fail(GBS_ERR_INVALID_ARG, "mtx: fewer entries than the size line states");
    float val = 1.0f;
    if (kind == 0) {
      if (!rd.read_float(&val)) return fail(GBS_ERR_INVALID_ARG, "mtx: missing value");
    } else if (kind == 1) {
      long iv;
      if (!rd.read_long(&iv)) return fail(GBS_ERR_INVALID_ARG, "mtx: missing value");
      val = (float)(int)iv;
    }
    if (r < 1 || r > M || cc < 1 || cc > N)
      return fail(GBS_ERR_INVALID_ARG, "mtx: entry " + std::to_string(e + 1) + " outside the matrix");
    ri[(size_t)e] = (int)(r - 1);
    ci[(size_t)e] = (int)(cc - 1);
    v[(size_t)e] = val;
  }

  // counting sort by row (stable), then stable sort of each row by column.
  // With several threads each counts and scatters its own range of entries
  // (file order), the ranges placed one after another inside every row, as
  // long as the per-thread row counters stay within a few times NZ.
  std::vector<int> rowptr((size_t)M + 1, 0);
  RawArray<int> order((size_t)NZ);
  const int TC = (NZ > (1l << 20) && (long long)T * (M + 1) <= 4ll * NZ) ? T : 1;
  if (TC > 1) {
    std::vector<std::vector<int>> cnt(TC);
    run_threads(TC, [&](int t) {
      cnt[t].assign((size_t)M, 0);
      for (long e = NZ * t / TC; e < NZ * (t + 1) / TC; ++e) cnt[t][(size_t)ri[(size_t)e]]++;
    });
    // rows split over the threads: each row's total, and each thread's start
    // inside the row (relative)
    run_threads(TC, [&](int t) {
      for (long i = M * t / TC; i < M * (t + 1) / TC; ++i) {
        int run = 0;
        for (int u = 0; u < TC; ++u) {
          const int k = cnt[u][(size_t)i];
          cnt[u][(size_t)i] = run;
          run += k;
        }
        rowptr[(size_t)i + 1] = run;
      }
    });
    for (long i = 0; i < M; ++i) rowptr[(size_t)i + 1] += rowptr[(size_t)i];
    run_threads(TC, [&](int t) {
      std::vector<int> &fill = cnt[t];
      for (long e = NZ * t / TC; e < NZ * (t + 1) / TC; ++e) {
        const int r = ri[(size_t)e];
        order[(size_t)rowptr[(size_t)r] + (size_t)fill[(size_t)r]++] = (int)e;
      }
    });
  } else {
    for (long e = 0; e < NZ; ++e) rowptr[(size_t)ri[(size_t)e] + 1]++;
    for (long i = 0; i < M; ++i) rowptr[(size_t)i + 1] += rowptr[(size_t)i];
    std::vector<int> fill(rowptr.begin(), rowptr.end() - 1);
    for (long e = 0; e < NZ; ++e) order[(size_t)fill[(size_t)ri[(size_t)e]]++] = (int)e;
  }
  // per-row sorts on T threads, rows split into ranges of ~NZ / T entries
  std::vector<long> rcut(T + 1, M);
  rcut[0] = 0;
  for (int t = 1; t < T; ++t)
    rcut[t] = std::lower_bound(rowptr.begin(), rowptr.end() - 1, (int)((long long)NZ * t / T)) - rowptr.begin();
  for (int t = 1; t <= T; ++t) rcut[t] = std::max(rcut[t], rcut[t - 1]);
  run_threads(NZ > (1l << 20) ? T : 1, [&](int t) {
    const long i0 = NZ > (1l << 20) ? rcut[t] : 0, i1 = NZ > (1l << 20) ? rcut[t + 1] : M;
    for (long i = i0; i < i1; ++i)
      std::stable_sort(order.data() + rowptr[(size_t)i], order.data() + rowptr[(size_t)i + 1],
                       [&](int a, int b) { return ci[(size_t)a] < ci[(size_t)b]; });
  });

  out->nrows = (int)M;
  out->ncols = (int)N;
  out->nnz = (int)NZ;
  out->rowptr = (int *)std::malloc(sizeof(int) * ((size_t)M + 1));
  out->colind = (int *)std::malloc(sizeof(int) * (size_t)(NZ > 0 ? NZ : 1));
  out->vals = (float *)std::malloc(sizeof(float) * (size_t)(NZ > 0 ? NZ : 1));
  if (!out->rowptr || !out->colind || !out->vals) {
    gbs_host_csr_free(out);
    return fail(GBS_ERR_OOM, "mtx: host allocation failed");
  }
  std::memcpy(out->rowptr, rowptr.data(), sizeof(int) * ((size_t)M + 1));
  const int TG = NZ > (1l << 20) ? T : 1;
  run_threads(TG, [&](int t) {
    for (long e = NZ * t / TG; e < NZ * (t + 1) / TG; ++e) {
      const int k = order[(size_t)e];
      out->colind[e] = ci[(size_t)k];
      out->vals[e] = v[(size_t)k];
    }
  });
  return GBS_OK;
}

extern "C" void gbs_host_csr_free(gbs_host_csr *c) {
  if (!c) return;
  std::free(c->rowptr);
  std::free(c->colind);
  std::free(c->vals);
  c->rowptr = nullptr;
  c->colind = nullptr;
  c->vals = nullptr;
}

// ---------------------------------------------------------------------------
// Binary CSR cache: parsing a large .mtx once and reloading its CSR.  Layout
// (host byte order): 8-byte magic "GBSCSR1\0", int32 nrows, ncols, nnz,
// has_vals, then rowptr[nrows + 1], colind[nnz] (int32) and, if has_vals,
// vals[nnz] (float32).
// ---------------------------------------------------------------------------
namespace {
const char kBinMagic[8] = {'G', 'B', 'S', 'C', 'S', 'R', '1', '\0'};
}

extern "C" gbs_status gbs_csr_write_bin(const char *path, const gbs_host_csr *csr) {
  clear_error();
  GBS_REQUIRE(path && csr, "csr bin: null argument");
  GBS_REQUIRE(csr->nrows >= 0 && csr->ncols >= 0 && csr->nnz >= 0 && csr->rowptr, "csr bin: bad CSR");
  GBS_REQUIRE(csr->nnz == 0 || csr->colind, "csr bin: null colind");
  FILE *f = std::fopen(path, "wb");
  if (!f) return fail(GBS_ERR_INVALID_ARG, std::string("csr bin: cannot create ") + path);
  const int hdr[4] = {csr->nrows, csr->ncols, csr->nnz, csr->vals ? 1 : 0};
  bool ok = std::fwrite(kBinMagic, 1, 8, f) == 8 && std::fwrite(hdr, sizeof(int), 4, f) == 4 &&
            std::fwrite(csr->rowptr, sizeof(int), (size_t)csr->nrows + 1, f) == (size_t)csr->nrows + 1 &&
            std::fwrite(csr->colind, sizeof(int), (size_t)csr->nnz, f) == (size_t)csr->nnz;
  if (ok && csr->vals) ok = std::fwrite(csr->vals, sizeof(float), (size_t)csr->nnz, f) == (size_t)csr->nnz;
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return fail(GBS_ERR_INVALID_ARG, std::string("csr bin: write failed: ") + path);
  return GBS_OK;
}

extern "C" gbs_status gbs_csr_read_bin(const char *path, gbs_host_csr *out) {
  clear_error();
  GBS_REQUIRE(path && out, "csr bin: null argument");
  std::memset(out, 0, sizeof(*out));
  FILE *f = std::fopen(path, "rb");
  if (!f) return fail(GBS_ERR_INVALID_ARG, std::string("csr bin: cannot open ") + path);
  char magic[8];
  int hdr[4];
  if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, kBinMagic, 8) != 0 ||
      std::fread(hdr, sizeof(int), 4, f) != 4) {
    std::fclose(f);
    return fail(GBS_ERR_INVALID_ARG, "csr bin: not a CSR cache file");
  }
  const int n = hdr[0], m = hdr[1], nnz = hdr[2], has_vals = hdr[3];
  if (n < 0 || m < 0 || nnz < 0 || (has_vals != 0 && has_vals != 1)) {
    std::fclose(f);
    return fail(GBS_ERR_INVALID_ARG, "csr bin: corrupt header");
  }
  out->nrows = n;
  out->ncols = m;
  out->nnz = nnz;
  out->rowptr = (int *)std::malloc(sizeof(int) * ((size_t)n + 1));
  out->colind = (int *)std::malloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
  out->vals = (float *)std::malloc(sizeof(float) * (size_t)(nnz > 0 ? nnz : 1));
  if (!out->rowptr || !out->colind || !out->vals) {
    std::fclose(f);
    gbs_host_csr_free(out);
    return fail(GBS_ERR_OOM, "csr bin: host allocation failed");
  }
  bool ok = std::fread(out->rowptr, sizeof(int), (size_t)n + 1, f) == (size_t)n + 1 &&
            std::fread(out->colind, sizeof(int), (size_t)nnz, f) == (size_t)nnz;
  if (ok && has_vals) ok = std::fread(out->vals, sizeof(float), (size_t)nnz, f) == (size_t)nnz;
  if (ok && !has_vals)
    for (int e = 0; e < nnz; ++e) out->vals[e] = 1.0f;
  std::fclose(f);
  // a CSR the rest of the library can trust
  if (ok) ok = out->rowptr[0] == 0 && out->rowptr[n] == nnz;
  for (int i = 0; ok && i < n; ++i) ok = out->rowptr[i] <= out->rowptr[i + 1];
  for (int e = 0; ok && e < nnz; ++e) ok = out->colind[e] >= 0 && out->colind[e] < m;
  if (!ok) {
    gbs_host_csr_free(out);
    std::memset(out, 0, sizeof(*out));
    return fail(GBS_ERR_INVALID_ARG, "csr bin: truncated or inconsistent file");
  }
  return GBS_OK;
}

// ---------------------------------------------------------------------------
// Binary B2SR cache: packed tiles kept between runs.  Layout (host byte
// order): 8-byte magic "GBSB2SR1", int32 nrows, ncols, tile, nblockrows,
// nnzb, then rowptr[nblockrows + 1], colind[nnzb] (int32) and
// val[nnzb * tile] in the tile's element width (1, 1, 2, 4 bytes for tiles
// 4, 8, 16, 32).  Row r of a tile is one element whose bit (tile - 1 - j)
// is column j of the tile, as the packers write it.
// ---------------------------------------------------------------------------
namespace {
const char kB2srMagic[8] = {'G', 'B', 'S', 'B', '2', 'S', 'R', '1'};

size_t tile_elem_bytes(int tile) { return tile == 32 ? 4 : (tile == 16 ? 2 : 1); }

uint32_t tile_row_at(const void *val, int tile, size_t i) {
  if (tile == 32) return static_cast<const uint32_t *>(val)[i];
  if (tile == 16) return static_cast<const uint16_t *>(val)[i];
  return static_cast<const uint8_t *>(val)[i];
}

// A B2SR the kernels can trust: block-row pointers from 0 to nnzb, tile
// columns strictly ascending inside a block-row and inside the matrix, no
// bit outside the tile's width, past the last column or on a row past the
// last row.
bool b2sr_consistent(const gbs_host_b2sr &b) {
  const int T = b.tile, mb = b.nblockrows;
  const int nbc = (b.ncols + T - 1) / T;
  if (b.rowptr[0] != 0 || b.rowptr[mb] != b.nnzb) return false;
  for (int i = 0; i < mb; ++i) {
    const int s = b.rowptr[i], e = b.rowptr[i + 1];
    if (s > e) return false;
    for (int k = s; k < e; ++k) {
      const int bc = b.colind[k];
      if (bc < 0 || bc >= nbc || (k > s && bc <= b.colind[k - 1])) return false;
      const int cols = std::min(T, b.ncols - bc * T);
      const uint32_t allowed = (cols == 32 ? 0xffffffffu : ((1u << cols) - 1u)) << (T - cols);
      const int rows = std::min(T, b.nrows - i * T);
      for (int r = 0; r < T; ++r) {
        const uint32_t w = tile_row_at(b.val, T, (size_t)k * T + r);
        if ((w & ~allowed) != 0 || (r >= rows && w != 0)) return false;
      }
    }
  }
  return true;
}
}  // namespace

extern "C" void gbs_host_b2sr_free(gbs_host_b2sr *b) {
  if (!b) return;
  std::free(b->rowptr);
  std::free(b->colind);
  std::free(b->val);
  b->rowptr = nullptr;
  b->colind = nullptr;
  b->val = nullptr;
}

extern "C" gbs_status gbs_b2sr_write_bin(const char *path, const gbs_host_b2sr *b) {
  clear_error();
  GBS_REQUIRE(path && b && b->rowptr, "b2sr bin: null argument");
  GBS_REQUIRE(b->tile == 4 || b->tile == 8 || b->tile == 16 || b->tile == 32, "b2sr bin: tile must be 4, 8, 16 or 32");
  GBS_REQUIRE(b->nrows >= 0 && b->ncols >= 0 && b->nnzb >= 0 &&
                  b->nblockrows == (b->nrows + b->tile - 1) / b->tile,
              "b2sr bin: bad shape");
  GBS_REQUIRE(b->nnzb == 0 || (b->colind && b->val), "b2sr bin: null colind / val");
  GBS_REQUIRE(b2sr_consistent(*b), "b2sr bin: inconsistent B2SR arrays");
  FILE *f = std::fopen(path, "wb");
  if (!f) return fail(GBS_ERR_INVALID_ARG, std::string("b2sr bin: cannot create ") + path);
  const int hdr[5] = {b->nrows, b->ncols, b->tile, b->nblockrows, b->nnzb};
  const size_t nv = (size_t)b->nnzb * b->tile, eb = tile_elem_bytes(b->tile);
  bool ok = std::fwrite(kB2srMagic, 1, 8, f) == 8 && std::fwrite(hdr, sizeof(int), 5, f) == 5 &&
            std::fwrite(b->rowptr, sizeof(int), (size_t)b->nblockrows + 1, f) == (size_t)b->nblockrows + 1 &&
            std::fwrite(b->colind, sizeof(int), (size_t)b->nnzb, f) == (size_t)b->nnzb &&
            std::fwrite(b->val, eb, nv, f) == nv;
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return fail(GBS_ERR_INVALID_ARG, std::string("b2sr bin: write failed: ") + path);
  return GBS_OK;
}

extern "C" gbs_status gbs_b2sr_read_bin(const char *path, gbs_host_b2sr *out) {
  clear_error();
  GBS_REQUIRE(path && out, "b2sr bin: null argument");
  std::memset(out, 0, sizeof(*out));
  FILE *f = std::fopen(path, "rb");
  if (!f) return fail(GBS_ERR_INVALID_ARG, std::string("b2sr bin: cannot open ") + path);
  char magic[8];
  int hdr[5];
  if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, kB2srMagic, 8) != 0 ||
      std::fread(hdr, sizeof(int), 5, f) != 5) {
    std::fclose(f);
    return fail(GBS_ERR_INVALID_ARG, "b2sr bin: not a B2SR cache file");
  }
  const int n = hdr[0], m = hdr[1], T = hdr[2], mb = hdr[3], nnzb = hdr[4];
  if (n < 0 || m < 0 || nnzb < 0 || !(T == 4 || T == 8 || T == 16 || T == 32) || mb != (n + T - 1) / T) {
    std::fclose(f);
    return fail(GBS_ERR_INVALID_ARG, "b2sr bin: corrupt header");
  }
  out->nrows = n;
  out->ncols = m;
  out->tile = T;
  out->nblockrows = mb;
  out->nnzb = nnzb;
  const size_t nv = (size_t)nnzb * T, eb = tile_elem_bytes(T);
  out->rowptr = (int *)std::malloc(sizeof(int) * ((size_t)mb + 1));
  out->colind = (int *)std::malloc(sizeof(int) * (size_t)(nnzb > 0 ? nnzb : 1));
  out->val = std::malloc(eb * (nv > 0 ? nv : 1));
  if (!out->rowptr || !out->colind || !out->val) {
    std::fclose(f);
    gbs_host_b2sr_free(out);
    return fail(GBS_ERR_OOM, "b2sr bin: host allocation failed");
  }
  bool ok = std::fread(out->rowptr, sizeof(int), (size_t)mb + 1, f) == (size_t)mb + 1 &&
            std::fread(out->colind, sizeof(int), (size_t)nnzb, f) == (size_t)nnzb &&
            std::fread(out->val, eb, nv, f) == nv;
  std::fclose(f);
  if (!ok || !b2sr_consistent(*out)) {
    gbs_host_b2sr_free(out);
    std::memset(out, 0, sizeof(*out));
    return fail(GBS_ERR_INVALID_ARG, "b2sr bin: truncated or inconsistent file");
  }
  return GBS_OK;
}
