// Matrix Market coordinate reader: MtxReader::parse of the reference
// (crates/core/src/mtx.rs:124-275, errors crates/core/src/error.rs:43-81).
//
// Same acceptance rules and error kinds/texts: the first non-empty line is
// the `%%MatrixMarket matrix <format> <field> <symmetry>` banner (case
// insensitive, 5 tokens, `array` unsupported); the dimension line is the
// first non-empty, non-comment line after it (`rows cols nnz`); symmetric,
// skew-symmetric and hermitian matrices must be square and every
// off-diagonal entry (i, j) also yields (j, i); coordinates are 1-based and
// bounds-checked, extra tokens (values) are ignored, self-loops dropped, and
// the graph has max(rows, cols) vertices with sorted, deduplicated
// adjacency (CsrGraph::from_edge_list).
//
// Unlike the reference's line-by-line stream, the entry section is parsed by
// all host threads at once: the text is cut into chunks at line breaks, each
// thread parses its chunk into its own pair list, and the first failing
// line in file order is reported with the line number it has in the file.
#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/msbfs.h"
#include "host_graph.h"

namespace {

bool is_ws(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }

struct Line {
  const char* b;
  const char* e;  // trimmed [b, e)
};

Line trim(const char* b, const char* e) {
  while (b < e && is_ws(*b)) ++b;
  while (e > b && is_ws(e[-1])) --e;
  return {b, e};
}

// Next whitespace-separated token of [*p, e); empty when none.
Line token(const char** p, const char* e) {
  const char* b = *p;
  while (b < e && is_ws(*b)) ++b;
  const char* t = b;
  while (t < e && !is_ws(*t)) ++t;
  *p = t;
  return {b, t};
}

std::string str(Line l) { return std::string(l.b, l.e - l.b); }

bool ieq(Line l, const char* s) {
  const size_t n = strlen(s);
  if ((size_t)(l.e - l.b) != n) return false;
  for (size_t i = 0; i < n; ++i) {
    char c = l.b[i];
    if (c >= 'A' && c <= 'Z') c = (char)(c - 'A' + 'a');
    if (c != s[i]) return false;
  }
  return true;
}

std::string lower(Line l) {
  std::string s = str(l);
  for (char& c : s)
    if (c >= 'A' && c <= 'Z') c = (char)(c - 'A' + 'a');
  return s;
}

// usize::from_str semantics: optional '+', decimal digits, no overflow.
// Returns nullptr on success, else the ParseIntError text.
const char* parse_usize(Line t, uint64_t* out) {
  const char* p = t.b;
  if (p == t.e) return "cannot parse integer from empty string";
  if (*p == '+') {
    ++p;
    if (p == t.e) return "invalid digit found in string";
  }
  uint64_t v = 0;
  for (; p < t.e; ++p) {
    if (*p < '0' || *p > '9') return "invalid digit found in string";
    const uint64_t d = (uint64_t)(*p - '0');
    if (v > (UINT64_MAX - d) / 10) return "number too large to fit in target type";
    v = v * 10 + d;
  }
  *out = v;
  return nullptr;
}

struct Err {
  int kind = MSBFS_MTX_OK;
  uint64_t line = 0, row = 0, col = 0, max_rows = 0, max_cols = 0;
  std::string msg;
};

void set_msg(Err* e) {
  char buf[512];
  switch (e->kind) {
    case MSBFS_MTX_ZERO_INDEX:
      snprintf(buf, sizeof buf,
               "Matrix Market coordinates are 1-based, but found 0 at line %llu: row=%llu, "
               "col=%llu",
               (unsigned long long)e->line, (unsigned long long)e->row,
               (unsigned long long)e->col);
      e->msg = buf;
      break;
    case MSBFS_MTX_INDEX_OUT_OF_BOUNDS:
      snprintf(buf, sizeof buf,
               "Coordinate out of bounds at line %llu: entry (%llu, %llu) exceeds matrix "
               "dimensions (%llu, %llu)",
               (unsigned long long)e->line, (unsigned long long)e->row,
               (unsigned long long)e->col, (unsigned long long)e->max_rows,
               (unsigned long long)e->max_cols);
      e->msg = buf;
      break;
    default:
      break;
  }
}

Err header_err(uint64_t line, const std::string& reason) {
  Err e;
  e.kind = MSBFS_MTX_INVALID_HEADER;
  e.line = line;
  e.msg = "Invalid Matrix Market header at line " + std::to_string(line) + ": " + reason;
  return e;
}

Err dims_err(uint64_t line, const std::string& reason) {
  Err e;
  e.kind = MSBFS_MTX_INVALID_DIMENSIONS;
  e.line = line;
  e.msg = "Invalid dimensions at line " + std::to_string(line) + ": " + reason;
  return e;
}

Err unsupported(const std::string& what) {
  Err e;
  e.kind = MSBFS_MTX_UNSUPPORTED_FORMAT;
  e.msg = "Unsupported Matrix Market format '" + what +
          "': only sparse 'coordinate' format is supported";
  return e;
}

struct Chunk {
  const char* b;
  const char* e;
  uint64_t lines = 0;  // lines fully scanned
  bool failed = false;
  Err err;             // line holds the chunk-local line index
  std::vector<uint64_t> pairs;
};

void parse_entries(Chunk* c, uint64_t rows, uint64_t cols, bool sym) {
  const char* p = c->b;
  while (p < c->e) {
    const char* nl = static_cast<const char*>(memchr(p, '\n', (size_t)(c->e - p)));
    const char* le = nl ? nl : c->e;
    const Line l = trim(p, le);
    const uint64_t local = c->lines;
    ++c->lines;
    p = nl ? nl + 1 : c->e;
    if (l.b == l.e || *l.b == '%') continue;
    const char* q = l.b;
    const Line rt = token(&q, l.e);
    const Line ct = token(&q, l.e);
    uint64_t r = 0, col = 0;
    if (ct.b == ct.e || parse_usize(rt, &r) || parse_usize(ct, &col)) {
      c->failed = true;
      c->err.kind = MSBFS_MTX_INVALID_COORDINATE_LINE;
      c->err.line = local;
      c->err.msg = str(l);  // completed with the file line number later
      return;
    }
    if (r == 0 || col == 0 || r > rows || col > cols) {
      c->failed = true;
      c->err.kind = (r == 0 || col == 0) ? MSBFS_MTX_ZERO_INDEX : MSBFS_MTX_INDEX_OUT_OF_BOUNDS;
      c->err.line = local;
      c->err.row = r;
      c->err.col = col;
      c->err.max_rows = rows;
      c->err.max_cols = cols;
      return;
    }
    const uint64_t u = r - 1, v = col - 1;
    if (u == v) continue;  // self-loops are dropped
    c->pairs.push_back(u << 32 | v);
    if (sym) c->pairs.push_back(v << 32 | u);
  }
}

bool parse(const char* text, size_t len, msbfs::HostCsr* out, Err* err) {
  const char* p = text;
  const char* end = text + len;
  uint64_t line_no = 0;
  auto next_line = [&](Line* l) {
    if (p >= end) return false;
    const char* nl = static_cast<const char*>(memchr(p, '\n', (size_t)(end - p)));
    const char* le = nl ? nl : end;
    *l = trim(p, le);
    p = nl ? nl + 1 : end;
    ++line_no;
    return true;
  };
  // 1. banner
  Line l{};
  for (;;) {
    if (!next_line(&l)) {
      *err = header_err(line_no + 1, "Empty input: no MatrixMarket header found");
      return false;
    }
    if (l.b != l.e) break;
  }
  Line tok[6];
  int nt = 0;
  {
    const char* q = l.b;
    for (;;) {
      Line t = token(&q, l.e);
      if (t.b == t.e) break;
      if (nt < 6) tok[nt] = t;
      ++nt;
    }
  }
  if (nt != 5) {
    *err = header_err(line_no, "Expected 5 tokens in header line, found " + std::to_string(nt) +
                                   ": '" + str(l) + "'");
    return false;
  }
  if (!ieq(tok[0], "%%matrixmarket")) {
    *err = header_err(line_no, "Missing '%%MatrixMarket' banner: '" + str(tok[0]) + "'");
    return false;
  }
  if (!ieq(tok[1], "matrix")) {
    *err = header_err(line_no, "Unsupported object '" + str(tok[1]) +
                                   "', only 'matrix' is supported");
    return false;
  }
  const std::string fmt = lower(tok[2]);
  if (fmt == "array") {
    *err = unsupported("array");
    return false;
  }
  if (fmt != "coordinate") {
    *err = header_err(line_no, "Unknown format '" + fmt + "'");
    return false;
  }
  const std::string field = lower(tok[3]);
  if (field != "pattern" && field != "real" && field != "integer" && field != "complex") {
    *err = header_err(line_no, "Unknown field '" + field + "'");
    return false;
  }
  const std::string symm = lower(tok[4]);
  if (symm != "general" && symm != "symmetric" && symm != "skew-symmetric" &&
      symm != "hermitian") {
    *err = header_err(line_no, "Unknown symmetry '" + symm + "'");
    return false;
  }
  const bool sym = symm != "general";
  // 2. dimension line
  for (;;) {
    if (!next_line(&l)) {
      *err = dims_err(line_no + 1, "Unexpected end of file while searching for dimension line");
      return false;
    }
    if (l.b != l.e && *l.b != '%') break;
  }
  nt = 0;
  {
    const char* q = l.b;
    for (;;) {
      Line t = token(&q, l.e);
      if (t.b == t.e) break;
      if (nt < 6) tok[nt] = t;
      ++nt;
    }
  }
  if (nt != 3) {
    *err = dims_err(line_no, "Expected 3 integer tokens (rows cols nnz), got " +
                                 std::to_string(nt) + ": '" + str(l) + "'");
    return false;
  }
  uint64_t dim[3];
  const char* names[3] = {"rows", "cols", "nnz"};
  for (int i = 0; i < 3; ++i)
    if (const char* why = parse_usize(tok[i], &dim[i])) {
      *err = dims_err(line_no, std::string("Failed to parse ") + names[i] + " count '" +
                                   str(tok[i]) + "': " + why);
      return false;
    }
  const uint64_t rows = dim[0], cols = dim[1];
  if (sym && rows != cols) {
    *err = dims_err(line_no, "Symmetric matrix must be square, but got " +
                                 std::to_string(rows) + " rows and " + std::to_string(cols) +
                                 " cols");
    return false;
  }
  const uint64_t V = std::max(rows, cols);
  if (V >= 0xFFFFFFFFull) {
    *err = dims_err(line_no, "graph exceeds u32 vertex indices");
    return false;
  }
  // 3. entries, in parallel chunks cut at line breaks
  const size_t rest = (size_t)(end - p);
  const int nthreads =
      (int)std::max<size_t>(1, std::min<size_t>(msbfs::host_threads(), rest / (1 << 20) + 1));
  std::vector<Chunk> chunks(nthreads);
  const char* cb = p;
  for (int t = 0; t < nthreads; ++t) {
    const char* ce = t + 1 == nthreads ? end : std::max(cb, p + rest * (t + 1) / nthreads);
    if (ce < end && ce > cb) {
      const char* nl = static_cast<const char*>(memchr(ce, '\n', (size_t)(end - ce)));
      ce = nl ? nl + 1 : end;
    }
    chunks[t].b = cb;
    chunks[t].e = ce;
    cb = ce;
  }
  {
    std::vector<std::thread> th;
    for (int t = 1; t < nthreads; ++t)
      th.emplace_back(parse_entries, &chunks[t], rows, cols, sym);
    parse_entries(&chunks[0], rows, cols, sym);
    for (auto& x : th) x.join();
  }
  uint64_t base = line_no;  // lines before the entry section
  for (Chunk& c : chunks) {
    if (c.failed) {
      Err e = c.err;
      e.line = base + e.line + 1;
      if (e.kind == MSBFS_MTX_INVALID_COORDINATE_LINE)
        e.msg = "Invalid coordinate entry at line " + std::to_string(e.line) + ": '" + e.msg +
                "'";
      else
        set_msg(&e);
      *err = e;
      return false;
    }
    base += c.lines;
  }
  std::vector<const std::vector<uint64_t>*> lists;
  for (const Chunk& c : chunks) lists.push_back(&c.pairs);
  *out = msbfs::csr_from_pair_lists((size_t)V, lists);
  return true;
}

int export_err(const Err& e, msbfs_mtx_error* out) {
  if (out) {
    memset(out, 0, sizeof *out);
    out->kind = e.kind;
    out->line_number = e.line;
    out->row = e.row;
    out->col = e.col;
    out->max_rows = e.max_rows;
    out->max_cols = e.max_cols;
    snprintf(out->message, sizeof out->message, "%s", e.msg.c_str());
  }
  return e.kind == MSBFS_MTX_OK ? MSBFS_OK : MSBFS_ERR_PARSE;
}

int export_graph(const msbfs::HostCsr& g, msbfs_csr* out) {
  out->num_vertices = g.V;
  out->num_edges = g.E;
  out->row_offsets = (uint32_t*)malloc((g.V + 1) * sizeof(uint32_t));
  out->col_indices = (uint32_t*)malloc((g.E ? g.E : 1) * sizeof(uint32_t));
  if (!out->row_offsets || !out->col_indices) {
    free(out->row_offsets);
    free(out->col_indices);
    out->row_offsets = out->col_indices = nullptr;
    return MSBFS_ERR_OOM;
  }
  if (g.off.empty())
    out->row_offsets[0] = 0;
  else
    memcpy(out->row_offsets, g.off.data(), (g.V + 1) * sizeof(uint32_t));
  if (g.E) memcpy(out->col_indices, g.idx.data(), g.E * sizeof(uint32_t));
  return MSBFS_OK;
}

}  // namespace

extern "C" {

int msbfs_mtx_parse(const char* text, size_t len, msbfs_csr* out, msbfs_mtx_error* err) {
  if (!out || (len && !text)) return MSBFS_ERR_INVALID_ARGUMENT;
  try {
    Err e;
    msbfs::HostCsr g;
    if (!parse(text ? text : "", len, &g, &e)) return export_err(e, err);
    export_err(Err{}, err);
    return export_graph(g, out);
  } catch (const std::bad_alloc&) {
    return MSBFS_ERR_OOM;
  }
}

int msbfs_mtx_read(const char* path, msbfs_csr* out, msbfs_mtx_error* err) {
  if (!path || !out) return MSBFS_ERR_INVALID_ARGUMENT;
  FILE* f = fopen(path, "rb");
  Err e;
  if (!f) {
    e.kind = MSBFS_MTX_IO;
    e.msg = std::string("I/O error during Matrix Market parsing: ") + strerror(errno);
    return export_err(e, err);
  }
  std::vector<char> buf;
  try {
    fseek(f, 0, SEEK_END);
    const long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    buf.resize(n > 0 ? (size_t)n : 0);
    if (n > 0 && fread(buf.data(), 1, (size_t)n, f) != (size_t)n) {
      fclose(f);
      e.kind = MSBFS_MTX_IO;
      e.msg = "I/O error during Matrix Market parsing: short read";
      return export_err(e, err);
    }
  } catch (const std::bad_alloc&) {
    fclose(f);
    return MSBFS_ERR_OOM;
  }
  fclose(f);
  return msbfs_mtx_parse(buf.data(), buf.size(), out, err);
}

}  // extern "C"
