// gg_io.cu -- graph file input on the host: Rutherford-Boeing matrices (the files the
// reference's benchmark loads through HarwellRutherfordBoeing.jl's RutherfordBoeingData,
// benchmark/benchmarks.jl:262-266; Harwell-Boeing files without right-hand sides share
// the layout) and whitespace-separated edge lists (GraphIO.EdgeList,
// benchmark/benchmarks.jl:12-14).
//
// Matrix Market coordinate files are read too (gg_read_mtx).
//
// Rutherford-Boeing, assembled matrices:
//   line 1  title (columns 1-72) and key
//   line 2  card counts (total, pointer, index, value[, right-hand side])
//   line 3  type (3 letters: r/p/i value kind, u/s/z/r/h structure, a assembled),
//           nrow, ncol, nnz[, nelt]
//   line 4  Fortran formats of the pointer, index and value cards, e.g. (10I8) (3E26.16)
//   then ncol+1 column pointers, nnz row indices and (unless pattern) nnz values, each
//   card holding as many fixed-width fields as its format says.
// Fields are read by width, as Fortran does, so adjacent numbers without spaces parse.
// Symmetric (s) and skew-symmetric (z) files store one triangle; with expand != 0 the
// other triangle is added (negated for z), diagonal entries once.  The result is CSC
// with 1-based Int32 colptr / rowval, rows ascending within each column, and Float64
// values (1 for pattern files).
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gg_common.cuh"

namespace gg {

struct FortranFmt {
  int per_line = 0;  // fields per card
  int width = 0;     // characters per field
};

// (10I8), (3E26.16), (1P,3E26.16), (1P3D25.17), (8F10.3): repeat count and width of the
// first I / E / D / F / G descriptor
static bool parse_fmt(const std::string& f, FortranFmt* out) {
  size_t i = 0;
  while (i < f.size()) {
    const char c = (char)std::toupper((unsigned char)f[i]);
    if (c == 'I' || c == 'E' || c == 'D' || c == 'F' || c == 'G') {
      // repeat count: digits right before the letter, after a 'P' scale factor or a
      // comma / parenthesis
      size_t j = i;
      while (j > 0 && std::isdigit((unsigned char)f[j - 1])) --j;
      const int rep = (j < i) ? std::atoi(f.substr(j, i - j).c_str()) : 1;
      size_t k = i + 1;
      size_t w0 = k;
      while (k < f.size() && std::isdigit((unsigned char)f[k])) ++k;
      if (k == w0) return false;
      out->per_line = rep > 0 ? rep : 1;
      out->width = std::atoi(f.substr(w0, k - w0).c_str());
      return out->width > 0;
    }
    ++i;
  }
  return false;
}

struct LineReader {
  FILE* f;
  std::string line;
  bool next() {
    line.clear();
    int c;
    bool any = false;
    while ((c = std::fgetc(f)) != EOF) {
      any = true;
      if (c == '\n') break;
      if (c != '\r') line.push_back((char)c);
    }
    return any;
  }
};

// reads `count` fields of format fmt, card by card.  A card whose blank-separated
// tokens are exactly the fields it should hold is read token by token (some writers
// pad fields to other widths than their format states); otherwise by the format's
// field width, as Fortran does (adjacent fields without blanks between them).
template <typename T, typename Conv>
static bool read_fields(LineReader& R, const FortranFmt& fmt, int64_t count, std::vector<T>* out,
                        Conv conv) {
  out->resize((size_t)count);
  int64_t got = 0;
  while (got < count) {
    if (!R.next()) return false;
    std::string card = R.line;
    for (auto& ch : card)
      if (ch == 'D' || ch == 'd') ch = 'E';
    const int64_t want = (count - got) < fmt.per_line ? (count - got) : fmt.per_line;
    std::vector<std::string> tok;
    {
      size_t p = 0;
      while (p < card.size()) {
        while (p < card.size() && card[p] == ' ') ++p;
        size_t q = p;
        while (q < card.size() && card[q] != ' ') ++q;
        if (q > p) tok.push_back(card.substr(p, q - p));
        p = q;
      }
    }
    if ((int64_t)tok.size() == want) {
      for (const auto& t : tok)
        if (!conv(t.c_str(), &(*out)[(size_t)got++])) return false;
      continue;
    }
    for (int k = 0; k < fmt.per_line && got < count; ++k) {
      const size_t a = (size_t)k * fmt.width;
      if (a >= card.size()) break;
      const std::string fld = card.substr(a, (size_t)fmt.width);
      const char* s = fld.c_str();
      while (*s == ' ') ++s;
      if (!*s) break;  // a short card: the remaining fields are blank
      if (!conv(s, &(*out)[(size_t)got])) return false;
      ++got;
    }
  }
  return true;
}

static bool conv_int(const char* s, int64_t* v) {
  char* e = nullptr;
  *v = std::strtoll(s, &e, 10);
  return e != s;
}
static bool conv_real(const char* s, double* v) {
  char* e = nullptr;
  *v = std::strtod(s, &e);
  if (e == s) return false;
  // Fortran may drop the 'E' before a signed exponent: 1.5-003
  if (*e == '+' || *e == '-') {
    char* e2 = nullptr;
    const long ex = std::strtol(e, &e2, 10);
    if (e2 != e) {
      double p = 1.0;
      for (long i = 0; i < (ex < 0 ? -ex : ex); ++i) p *= 10.0;
      *v = ex < 0 ? *v / p : *v * p;
    }
  }
  return true;
}

// CSC (0-based, arbitrary order inside columns, possibly with repeated or mirrored
// entries) -> 1-based CSC with rows ascending in each column; of repeated (row, column)
// pairs the first in input order is kept (as a graph keeps the first edge added)
static void finish_csc(int64_t nrow, int64_t ncol, const std::vector<int64_t>& col,
                       const std::vector<int64_t>& row, const std::vector<double>& val,
                       std::vector<int32_t>* colptr, std::vector<int32_t>* rowval,
                       std::vector<double>* vals) {
  const size_t nz = row.size();
  // two stable counting sorts: by row, then by column -> (column, row, input order)
  std::vector<size_t> by_row(nz), order(nz);
  {
    std::vector<int64_t> rc((size_t)nrow + 1, 0);
    for (size_t k = 0; k < nz; ++k) rc[(size_t)row[k] + 1]++;
    for (int64_t r = 0; r < nrow; ++r) rc[(size_t)r + 1] += rc[(size_t)r];
    for (size_t k = 0; k < nz; ++k) by_row[(size_t)rc[(size_t)row[k]]++] = k;
  }
  {
    std::vector<int64_t> cc((size_t)ncol + 1, 0);
    for (size_t k = 0; k < nz; ++k) cc[(size_t)col[k] + 1]++;
    for (int64_t j = 0; j < ncol; ++j) cc[(size_t)j + 1] += cc[(size_t)j];
    for (size_t q = 0; q < nz; ++q) {
      const size_t k = by_row[q];
      order[(size_t)cc[(size_t)col[k]]++] = k;
    }
  }
  colptr->assign((size_t)ncol + 1, 1);
  rowval->clear();
  vals->clear();
  rowval->reserve(nz);
  vals->reserve(nz);
  int64_t pc = -1, pr = -1;
  for (size_t q = 0; q < nz; ++q) {
    const size_t k = order[q];
    if (col[k] == pc && row[k] == pr) continue;  // a repeat of the entry just kept
    pc = col[k];
    pr = row[k];
    rowval->push_back((int32_t)(row[k] + 1));
    vals->push_back(val[k]);
    (*colptr)[(size_t)col[k] + 1]++;
  }
  for (int64_t j = 0; j < ncol; ++j) (*colptr)[(size_t)j + 1] += (*colptr)[(size_t)j] - 1;
}

struct HostMatrix {
  int64_t m = 0, n = 0;
  std::vector<int32_t> ptr, idx;
  std::vector<double> val;
};

static int read_rb(const char* path, int expand, HostMatrix* H, int* kind_out) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return set_error(GG_ERR_ARGUMENT, "cannot open %s", path);
  LineReader R{f, {}};
  int rc = GG_OK;
  do {
    if (!R.next() || !R.next()) { rc = set_error(GG_ERR_ARGUMENT, "%s: truncated header", path); break; }
    long long cards[5] = {0, 0, 0, 0, 0};
    const int ncards = std::sscanf(R.line.c_str(), "%lld %lld %lld %lld %lld", cards, cards + 1,
                                   cards + 2, cards + 3, cards + 4);
    if (!R.next()) { rc = set_error(GG_ERR_ARGUMENT, "%s: truncated header", path); break; }
    std::string l3 = R.line;
    if (l3.size() < 3) { rc = set_error(GG_ERR_ARGUMENT, "%s: no matrix type", path); break; }
    const char vk = (char)std::tolower((unsigned char)l3[0]);
    const char sk = (char)std::tolower((unsigned char)l3[1]);
    const char ak = (char)std::tolower((unsigned char)l3[2]);
    if (ak != 'a') { rc = set_error(GG_ERR_UNSUPPORTED, "%s: only assembled matrices are read", path); break; }
    if (vk == 'c') { rc = set_error(GG_ERR_UNSUPPORTED, "%s: complex values", path); break; }
    if (vk != 'r' && vk != 'p' && vk != 'i') { rc = set_error(GG_ERR_ARGUMENT, "%s: value kind %c", path, vk); break; }
    long long nrow = 0, ncol = 0, nnz = 0;
    if (std::sscanf(l3.c_str() + 3, "%lld %lld %lld", &nrow, &ncol, &nnz) != 3 || nrow < 0 ||
        ncol < 0 || nnz < 0) {
      rc = set_error(GG_ERR_ARGUMENT, "%s: bad sizes", path);
      break;
    }
    if (nnz >= (1LL << 31) || nrow >= (1LL << 31) || ncol >= (1LL << 31)) {
      rc = set_error(GG_ERR_ARGUMENT, "%s: sizes do not fit Int32 indices", path);
      break;
    }
    if (!R.next()) { rc = set_error(GG_ERR_ARGUMENT, "%s: truncated header", path); break; }
    // the formats: parenthesised groups in order
    std::vector<std::string> fmts;
    {
      const std::string& l4 = R.line;
      size_t p = 0;
      while ((p = l4.find('(', p)) != std::string::npos) {
        size_t q = l4.find(')', p);
        if (q == std::string::npos) break;
        fmts.push_back(l4.substr(p, q - p + 1));
        p = q + 1;
      }
    }
    // a Harwell-Boeing file with right-hand sides has one more header line
    if (ncards == 5 && cards[4] > 0 && !R.next()) {
      rc = set_error(GG_ERR_ARGUMENT, "%s: truncated header", path);
      break;
    }
    FortranFmt fp, fi, fv;
    if (fmts.size() < 2 || !parse_fmt(fmts[0], &fp) || !parse_fmt(fmts[1], &fi) ||
        (vk != 'p' && (fmts.size() < 3 || !parse_fmt(fmts[2], &fv)))) {
      rc = set_error(GG_ERR_ARGUMENT, "%s: bad Fortran formats", path);
      break;
    }
    std::vector<int64_t> cp, ri;
    std::vector<double> vv;
    if (!read_fields(R, fp, ncol + 1, &cp, conv_int) || !read_fields(R, fi, nnz, &ri, conv_int)) {
      rc = set_error(GG_ERR_ARGUMENT, "%s: truncated pointer / index cards", path);
      break;
    }
    if (vk == 'p') vv.assign((size_t)nnz, 1.0);
    else if (!read_fields(R, fv, nnz, &vv, conv_real)) {
      rc = set_error(GG_ERR_ARGUMENT, "%s: truncated value cards", path);
      break;
    }
    if (cp[0] != 1 || cp[(size_t)ncol] != nnz + 1) {
      rc = set_error(GG_ERR_ARGUMENT, "%s: column pointers do not span 1:nnz+1", path);
      break;
    }
    // every pointer in 1:nnz+1 and non-decreasing before any entry is read through them
    bool ptr_ok = true;
    for (int64_t j = 0; j < ncol && ptr_ok; ++j)
      ptr_ok = cp[(size_t)j] >= 1 && cp[(size_t)j] <= cp[(size_t)j + 1] && cp[(size_t)j + 1] <= nnz + 1;
    if (!ptr_ok) {
      rc = set_error(GG_ERR_ARGUMENT, "%s: column pointers out of range or decreasing", path);
      break;
    }
    std::vector<int64_t> col, row;
    std::vector<double> val;
    col.reserve((size_t)nnz * (expand ? 2 : 1));
    row.reserve(col.capacity());
    val.reserve(col.capacity());
    bool bad = false;
    for (int64_t j = 0; j < ncol && !bad; ++j) {
      if (cp[(size_t)j + 1] < cp[(size_t)j]) { bad = true; break; }
      for (int64_t k = cp[(size_t)j] - 1; k < cp[(size_t)j + 1] - 1; ++k) {
        const int64_t r = ri[(size_t)k] - 1;
        if (r < 0 || r >= nrow) { bad = true; break; }
        col.push_back(j);
        row.push_back(r);
        val.push_back(vv[(size_t)k]);
        if (expand && (sk == 's' || sk == 'z' || sk == 'h') && r != j) {
          col.push_back(r);
          row.push_back(j);
          val.push_back(sk == 'z' ? -vv[(size_t)k] : vv[(size_t)k]);
        }
      }
    }
    if (bad) { rc = set_error(GG_ERR_ARGUMENT, "%s: row index or pointer out of range", path); break; }
    if ((int64_t)col.size() >= (1LL << 31) - 1) {
      rc = set_error(GG_ERR_ARGUMENT, "%s: %lld entries after symmetric expansion do not fit Int32 indices",
                     path, (long long)col.size());
      break;
    }
    H->m = nrow;
    H->n = ncol;
    finish_csc(nrow, ncol, col, row, val, &H->ptr, &H->idx, &H->val);
    *kind_out = (vk == 'p' ? 1 : vk == 'i' ? 2 : 0) | (sk == 's' ? 4 : sk == 'z' ? 8 : sk == 'h' ? 16 : 0);
  } while (0);
  std::fclose(f);
  return rc;
}

static int read_edgelist(const char* path, int base, HostMatrix* H, int* weighted) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return set_error(GG_ERR_ARGUMENT, "cannot open %s", path);
  LineReader R{f, {}};
  std::vector<int64_t> src, dst;
  std::vector<double> w;
  int64_t nv = 0, lineno = 0;
  int cols = -1;
  int rc = GG_OK;
  while (R.next()) {
    ++lineno;
    const char* s = R.line.c_str();
    while (*s == ' ' || *s == '\t') ++s;
    if (!*s || *s == '#' || *s == '%') continue;
    char* e = nullptr;
    const long long a = std::strtoll(s, &e, 10);
    if (e == s) { rc = set_error(GG_ERR_ARGUMENT, "%s:%lld: expected a vertex id", path, (long long)lineno); break; }
    while (*e == ' ' || *e == '\t' || *e == ',') ++e;
    const char* s2 = e;
    const long long b = std::strtoll(s2, &e, 10);
    if (e == s2) { rc = set_error(GG_ERR_ARGUMENT, "%s:%lld: expected two vertex ids", path, (long long)lineno); break; }
    while (*e == ' ' || *e == '\t' || *e == ',') ++e;
    double wt = 1.0;
    int c = 2;
    if (*e) {
      char* e3 = nullptr;
      wt = std::strtod(e, &e3);
      if (e3 != e) c = 3;
    }
    if (cols < 0) cols = c;
    const long long u = a - base, v = b - base;
    if (u < 0 || v < 0) { rc = set_error(GG_ERR_ARGUMENT, "%s:%lld: vertex id below %d", path, (long long)lineno, base); break; }
    if (u >= (1LL << 31) - 1 || v >= (1LL << 31) - 1) { rc = set_error(GG_ERR_ARGUMENT, "%s:%lld: vertex id too large", path, (long long)lineno); break; }
    src.push_back(u);
    dst.push_back(v);
    w.push_back(wt);
    nv = u + 1 > nv ? u + 1 : nv;
    nv = v + 1 > nv ? v + 1 : nv;
  }
  std::fclose(f);
  if (rc != GG_OK) return rc;
  if ((int64_t)src.size() >= (1LL << 31) - 1) return set_error(GG_ERR_ARGUMENT, "%s: too many edges", path);
  // adjacency A[u, v] for edge u -> v, as CSC (column v lists its in-neighbours u):
  // the CSR storage of A_T, the form every graph call takes
  H->m = nv;
  H->n = nv;
  finish_csc(nv, nv, dst, src, w, &H->ptr, &H->idx, &H->val);
  *weighted = cols == 3 ? 1 : 0;
  return GG_OK;
}

// Matrix Market coordinate files (the other format SuiteSparse matrices are published
// in): "%%MatrixMarket matrix coordinate <real|integer|pattern> <general|symmetric|
// skew-symmetric>", '%' comment lines, a size line "m n nnz", then nnz lines "i j [v]"
// with 1-based indices.  Symmetric / skew files store one triangle, expanded like the
// Rutherford-Boeing ones when expand != 0.
static int read_mtx(const char* path, int expand, HostMatrix* H, int* kind_out) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return set_error(GG_ERR_ARGUMENT, "cannot open %s", path);
  LineReader R{f, {}};
  int rc = GG_OK;
  do {
    if (!R.next()) { rc = set_error(GG_ERR_ARGUMENT, "%s: empty file", path); break; }
    std::string banner = R.line;
    for (auto& ch : banner) ch = (char)std::tolower((unsigned char)ch);
    if (banner.compare(0, 14, "%%matrixmarket") != 0) {
      rc = set_error(GG_ERR_ARGUMENT, "%s: no %%%%MatrixMarket banner", path);
      break;
    }
    if (banner.find("coordinate") == std::string::npos) {
      rc = set_error(GG_ERR_UNSUPPORTED, "%s: only coordinate (sparse) files are read", path);
      break;
    }
    if (banner.find("complex") != std::string::npos) {
      rc = set_error(GG_ERR_UNSUPPORTED, "%s: complex values", path);
      break;
    }
    const bool pattern = banner.find("pattern") != std::string::npos;
    const bool integer = banner.find("integer") != std::string::npos;
    const bool skew = banner.find("skew-symmetric") != std::string::npos;
    const bool herm = banner.find("hermitian") != std::string::npos;
    const bool sym = !skew && !herm && banner.find("symmetric") != std::string::npos;
    long long m = -1, n = -1, nnz = -1;
    while (R.next()) {
      const char* s = R.line.c_str();
      while (*s == ' ' || *s == '\t') ++s;
      if (!*s || *s == '%') continue;
      if (std::sscanf(s, "%lld %lld %lld", &m, &n, &nnz) != 3) m = -1;
      break;
    }
    if (m < 0 || n < 0 || nnz < 0) { rc = set_error(GG_ERR_ARGUMENT, "%s: bad size line", path); break; }
    if (m >= (1LL << 31) || n >= (1LL << 31) || nnz >= (1LL << 31)) {
      rc = set_error(GG_ERR_ARGUMENT, "%s: sizes do not fit Int32 indices", path);
      break;
    }
    std::vector<int64_t> col, row;
    std::vector<double> val;
    const size_t cap = (size_t)nnz * ((expand && (sym || skew || herm)) ? 2 : 1);
    col.reserve(cap);
    row.reserve(cap);
    val.reserve(cap);
    long long got = 0;
    while (got < nnz && R.next()) {
      const char* s = R.line.c_str();
      while (*s == ' ' || *s == '\t') ++s;
      if (!*s || *s == '%') continue;
      char* e = nullptr;
      const long long i = std::strtoll(s, &e, 10);
      const char* s2 = e;
      const long long j = std::strtoll(s2, &e, 10);
      if (e == s2) { rc = set_error(GG_ERR_ARGUMENT, "%s: bad entry line", path); break; }
      double v = 1.0;
      if (!pattern) {
        const char* s3 = e;
        v = std::strtod(s3, &e);
        if (e == s3) { rc = set_error(GG_ERR_ARGUMENT, "%s: entry without a value", path); break; }
      }
      if (i < 1 || i > m || j < 1 || j > n) {
        rc = set_error(GG_ERR_ARGUMENT, "%s: entry (%lld, %lld) outside %lldx%lld", path, i, j, m, n);
        break;
      }
      col.push_back(j - 1);
      row.push_back(i - 1);
      val.push_back(v);
      if (expand && (sym || skew || herm) && i != j) {
        col.push_back(i - 1);
        row.push_back(j - 1);
        val.push_back(skew ? -v : v);
      }
      ++got;
    }
    if (rc != GG_OK) break;
    if (got < nnz) { rc = set_error(GG_ERR_ARGUMENT, "%s: %lld of %lld entries", path, got, nnz); break; }
    if ((int64_t)col.size() >= (1LL << 31) - 1) {
      rc = set_error(GG_ERR_ARGUMENT, "%s: %lld entries after symmetric expansion do not fit Int32 indices",
                     path, (long long)col.size());
      break;
    }
    H->m = m;
    H->n = n;
    finish_csc(m, n, col, row, val, &H->ptr, &H->idx, &H->val);
    *kind_out = (pattern ? 1 : 0) | (integer ? 2 : 0) | (sym ? 4 : 0) | (skew ? 8 : 0) | (herm ? 16 : 0);
  } while (0);
  std::fclose(f);
  return rc;
}

static int export_matrix(HostMatrix& H, int64_t* m, int64_t* n, int64_t* nnz, int32_t** colptr,
                         int32_t** rowval, double** values) {
  const size_t nz = H.idx.size();
  int32_t* p = (int32_t*)std::malloc((H.ptr.size() > 0 ? H.ptr.size() : 1) * sizeof(int32_t));
  int32_t* r = (int32_t*)std::malloc((nz > 0 ? nz : 1) * sizeof(int32_t));
  double* v = (double*)std::malloc((nz > 0 ? nz : 1) * sizeof(double));
  if (!p || !r || !v) {
    std::free(p);
    std::free(r);
    std::free(v);
    return set_error(GG_ERR_OOM, "host allocation failed");
  }
  if (!H.ptr.empty()) std::memcpy(p, H.ptr.data(), H.ptr.size() * sizeof(int32_t));
  else p[0] = 1;
  if (nz) std::memcpy(r, H.idx.data(), nz * sizeof(int32_t));
  if (nz) std::memcpy(v, H.val.data(), nz * sizeof(double));
  *m = H.m;
  *n = H.n;
  *nnz = (int64_t)nz;
  *colptr = p;
  *rowval = r;
  *values = v;
  return GG_OK;
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_read_rb(const char* path, int expand_symmetric, int64_t* m, int64_t* n, int64_t* nnz,
               int32_t** colptr, int32_t** rowval, double** values, int* kind) {
  if (!path || !m || !n || !nnz || !colptr || !rowval || !values)
    return set_error(GG_ERR_ARGUMENT, "NULL argument");
  HostMatrix H;
  int k = 0;
  GG_CHECK(read_rb(path, expand_symmetric, &H, &k));
  if (kind) *kind = k;
  return export_matrix(H, m, n, nnz, colptr, rowval, values);
}

int gg_read_mtx(const char* path, int expand_symmetric, int64_t* m, int64_t* n, int64_t* nnz,
                int32_t** colptr, int32_t** rowval, double** values, int* kind) {
  if (!path || !m || !n || !nnz || !colptr || !rowval || !values)
    return set_error(GG_ERR_ARGUMENT, "NULL argument");
  HostMatrix H;
  int k = 0;
  GG_CHECK(read_mtx(path, expand_symmetric, &H, &k));
  if (kind) *kind = k;
  return export_matrix(H, m, n, nnz, colptr, rowval, values);
}

int gg_read_edgelist(const char* path, int base, int64_t* nv, int64_t* nnz, int32_t** colptr,
                     int32_t** rowval, double** values, int* weighted) {
  if (!path || !nv || !nnz || !colptr || !rowval || !values)
    return set_error(GG_ERR_ARGUMENT, "NULL argument");
  if (base != 0 && base != 1) return set_error(GG_ERR_ARGUMENT, "base must be 0 or 1");
  HostMatrix H;
  int w = 0;
  GG_CHECK(read_edgelist(path, base, &H, &w));
  if (weighted) *weighted = w;
  int64_t m2 = 0;
  return export_matrix(H, nv, &m2, nnz, colptr, rowval, values);
}

int gg_host_free(void* p) {
  std::free(p);
  return GG_OK;
}

}  // extern "C"
