// Matrix Market coordinate files -> CSR pattern, on the host.
//
// Replaces read_mtx_file (test-cg/include/dataloader/dataloader.hpp:22-107,
// banner and size parsing as in mmio.hpp:203-300): the pattern of a
// coordinate file (values are not kept; the SpMM paths read a null value
// array as ones), 1-based indices made 0-based, symmetric files expanded
// with the mirrored off-diagonal entries and de-duplicated, entries sorted
// by (row, column).  SS_MTX_REFERENCE reproduces the reference's result
// exactly, including that its CSR build stops after as many entries as the
// file declares (dataloader.hpp:93-101 bounds the walk by the file's count,
// so an expanded symmetric matrix loses its last rows' entries);
// SS_MTX_FULL keeps every expanded entry and also expands skew-symmetric and
// hermitian files (the reference treats those as general).
//
// Sorting is a counting sort by row followed by a sort of each row's
// columns: the same order as sorting (row, column) pairs, in linear time
// plus the short per-row sorts.
#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "internal.h"

struct ss_mtx {
  int nrow = 0, ncol = 0;
  std::vector<int32_t> indptr, indices;
};

namespace ss {
namespace {

struct Reader {
  const char *p, *end;
  bool eol() const { return p >= end || *p == '\n'; }
  void skip_blanks() {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\r')) p++;
  }
  void skip_space() {
    while (p < end && isspace((unsigned char)*p)) p++;
  }
  void skip_line() {
    while (p < end && *p != '\n') p++;
    if (p < end) p++;
  }
  std::string token() {  // next blank-separated token on this line
    skip_blanks();
    const char *s = p;
    while (p < end && !isspace((unsigned char)*p)) p++;
    return std::string(s, p);
  }
  bool integer(long long &v) {  // next whitespace-separated integer
    skip_space();
    bool neg = false;
    if (p < end && (*p == '+' || *p == '-')) neg = *p++ == '-';
    if (p >= end || !isdigit((unsigned char)*p)) return false;
    long long x = 0;
    while (p < end && isdigit((unsigned char)*p)) {
      x = x * 10 + (*p++ - '0');
      if (x > (1LL << 40)) return false;
    }
    v = neg ? -x : x;
    return true;
  }
  bool skip_token() {  // a value: any non-blank run
    skip_space();
    if (p >= end) return false;
    while (p < end && !isspace((unsigned char)*p)) p++;
    return true;
  }
};

std::string lower(std::string s) {
  for (char &c : s) c = (char)tolower((unsigned char)c);
  return s;
}

// The body of ss_mtx_read.  Host allocations may throw std::bad_alloc; the
// entry point turns that into a status, since no exception may cross the C
// boundary.
ss_status mtx_read(const char *path, int mode, ss_mtx **out) {
  FILE *f = fopen(path, "rb");
  if (!f) return fail(SS_ERR_INVALID_ARG, "cannot open %s", path);
  std::vector<char> buf;
  {
    char chunk[1 << 16];
    size_t n;
    while ((n = fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + n);
  }
  fclose(f);
  Reader r{buf.data(), buf.data() + buf.size()};

  // banner: %%MatrixMarket matrix coordinate <field> <symmetry>
  const std::string banner = r.token();
  const std::string object = lower(r.token()), format = lower(r.token());
  const std::string field = lower(r.token()), symmetry = lower(r.token());
  if (banner.compare(0, 14, "%%MatrixMarket") != 0) return fail(SS_ERR_BAD_DATA, "%s: no Matrix Market banner", path);
  if (object != "matrix") return fail(SS_ERR_BAD_DATA, "%s: object '%s' is not 'matrix'", path, object.c_str());
  if (format != "coordinate")
    return fail(SS_ERR_BAD_DATA, "%s: format '%s' unsupported (coordinate only)", path, format.c_str());
  int values_per_entry;
  if (field == "real" || field == "integer") values_per_entry = 1;
  else if (field == "complex") values_per_entry = 2;
  else if (field == "pattern") values_per_entry = 0;
  else return fail(SS_ERR_BAD_DATA, "%s: field '%s' unknown", path, field.c_str());
  const bool symmetric = symmetry == "symmetric";
  const bool mirrored = symmetric || symmetry == "skew-symmetric" || symmetry == "hermitian";
  if (!mirrored && symmetry != "general") return fail(SS_ERR_BAD_DATA, "%s: symmetry '%s' unknown", path, symmetry.c_str());
  const bool expand = mode == SS_MTX_FULL ? mirrored : symmetric;
  r.skip_line();
  // comments, then the size line
  while (r.p < r.end) {
    r.skip_blanks();
    if (r.p < r.end && *r.p == '%') { r.skip_line(); continue; }
    if (r.eol()) { r.skip_line(); continue; }
    break;
  }
  long long M, K, Z;
  if (!r.integer(M) || !r.integer(K) || !r.integer(Z) || M < 0 || K < 0 || Z < 0 || M > 0x7fffffff ||
      K > 0x7fffffff || Z > 0x7fffffff)
    return fail(SS_ERR_BAD_DATA, "%s: bad size line", path);

  // Each entry takes at least three bytes of text ("i j" and a separator,
  // the last one possibly without), so a file holds at most size / 3 + 1 of
  // them whatever its size line declares: reserve no more than that, so a
  // short file with a huge declared count fails on its missing entries
  // instead of on a huge allocation.
  std::vector<int32_t> rows, cols;
  const size_t fit = std::min((size_t)Z, buf.size() / 3 + 1);
  const size_t cap = fit * (expand ? 2 : 1);
  rows.reserve(cap);
  cols.reserve(cap);
  for (long long e = 0; e < Z; e++) {
    long long i, j;
    if (!r.integer(i) || !r.integer(j)) return fail(SS_ERR_BAD_DATA, "%s: entry %lld missing or malformed", path, e + 1);
    for (int v = 0; v < values_per_entry; v++)
      if (!r.skip_token()) return fail(SS_ERR_BAD_DATA, "%s: entry %lld has no value", path, e + 1);
    if (i < 1 || i > M || j < 1 || j > K)
      return fail(SS_ERR_BAD_DATA, "%s: entry %lld (%lld, %lld) outside %lld x %lld", path, e + 1, i, j, M, K);
    rows.push_back((int32_t)(i - 1));
    cols.push_back((int32_t)(j - 1));
    if (expand && i != j) {
      rows.push_back((int32_t)(j - 1));
      cols.push_back((int32_t)(i - 1));
    }
  }
  if (expand && M != K) return fail(SS_ERR_BAD_DATA, "%s: %s matrix is not square", path, symmetry.c_str());

  // counting sort by row, then each row's columns sorted (and de-duplicated
  // when the file was expanded, as the reference does for symmetric files)
  const size_t n = rows.size();
  std::vector<int64_t> start((size_t)M + 1, 0);
  for (size_t e = 0; e < n; e++) start[(size_t)rows[e] + 1]++;
  for (long long i = 0; i < M; i++) start[(size_t)i + 1] += start[(size_t)i];
  std::vector<int32_t> sorted(n);
  {
    std::vector<int64_t> cur(start.begin(), start.end() - 1);
    for (size_t e = 0; e < n; e++) sorted[(size_t)cur[(size_t)rows[e]]++] = cols[e];
  }
  std::unique_ptr<ss_mtx> m(new ss_mtx);
  m->nrow = (int)M;
  m->ncol = (int)K;
  m->indptr.assign((size_t)M + 1, 0);
  m->indices.reserve(n);
  // the reference builds CSR from at most the file's entry count
  const size_t limit = mode == SS_MTX_REFERENCE ? (size_t)Z : (size_t)-1;
  for (long long i = 0; i < M; i++) {
    int32_t *a = sorted.data() + start[(size_t)i];
    int32_t *b = sorted.data() + start[(size_t)i + 1];
    std::sort(a, b);
    if (expand) b = std::unique(a, b);
    for (int32_t *q = a; q < b && m->indices.size() < limit; q++) m->indices.push_back(*q);
    // int32 row pointers: a symmetric expansion (full mode) can double the
    // declared count past them
    if (m->indices.size() > (size_t)0x7fffffff)
      return fail(SS_ERR_CAPACITY, "%s: more than 2^31 - 1 entries after symmetric expansion", path);
    m->indptr[(size_t)i + 1] = (int32_t)m->indices.size();
  }
  *out = m.release();
  return SS_OK;
}

}  // namespace
}  // namespace ss

using namespace ss;

extern "C" {

ss_status ss_mtx_read(const char *path, int mode, ss_mtx **out) {
  if (!path || !out) return fail(SS_ERR_INVALID_ARG, "null path or output");
  if (mode != SS_MTX_REFERENCE && mode != SS_MTX_FULL) return fail(SS_ERR_INVALID_ARG, "mode %d unknown", mode);
  *out = nullptr;
  try {
    return mtx_read(path, mode, out);
  } catch (const std::bad_alloc &) {
    return fail(SS_ERR_CAPACITY, "%s: out of host memory while reading", path);
  }
}

ss_status ss_mtx_shape(const ss_mtx *m, int *nrow, int *ncol, int *nnz) {
  if (!m || !nrow || !ncol || !nnz) return fail(SS_ERR_INVALID_ARG, "null argument");
  *nrow = m->nrow;
  *ncol = m->ncol;
  *nnz = (int)m->indices.size();
  return SS_OK;
}

ss_status ss_mtx_csr(const ss_mtx *m, int32_t *indptr, int32_t *indices) {
  if (!m || !indptr || (!indices && !m->indices.empty())) return fail(SS_ERR_INVALID_ARG, "null argument");
  memcpy(indptr, m->indptr.data(), m->indptr.size() * sizeof(int32_t));
  if (!m->indices.empty()) memcpy(indices, m->indices.data(), m->indices.size() * sizeof(int32_t));
  return SS_OK;
}

void ss_mtx_free(ss_mtx *m) { delete m; }

}  // extern "C"
