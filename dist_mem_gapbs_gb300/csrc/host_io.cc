// Graph file input/output for the host side of the BFS path.
//
// Formats follow the reference's Reader / Writer: ".sg" serialized graphs
// (src/writer.h:39-69, src/reader.h:291-345), ".el" and ".wel" edge lists,
// DIMACS ".gr" files (gapbs-verify/reader.h:49-84), METIS ".graph" files
// (gapbs-verify/reader.h:88-140) and Matrix Market ".mtx" coordinate files
// (src/reader.h:186-256).  Edge lists go through
// gbbfs_build_csr, the same construction the synthetic graphs use.

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gbbfs.h"

namespace {

std::string Suffix(const std::string& path) {
  const size_t p = path.rfind('.');
  return p == std::string::npos ? std::string() : path.substr(p);
}

// Read whitespace-separated integers; `per_edge` values per record, of which
// the first two are the endpoints.  For ".gr", only lines starting with 'a'.
int ReadEdgeText(const std::string& path, bool dimacs, int per_edge,
                 std::vector<int32_t>* el) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return GBBFS_ERR_IO;
  char* lp = nullptr;
  size_t cap = 0;
  ssize_t len;
  int rc = GBBFS_OK;
  while ((len = getline(&lp, &cap, f)) >= 0) {
    const char* p = lp;
    while (*p == ' ' || *p == '\t') p++;
    if (*p == '\n' || *p == '\0' || *p == '\r') continue;
    if (dimacs) {
      if (*p != 'a') continue;
      p++;
    } else if (*p == '#' || *p == '%') {
      continue;
    }
    long long vals[3] = {0, 0, 0};
    int got = 0;
    char* end = nullptr;
    for (; got < per_edge; got++) {
      vals[got] = strtoll(p, &end, 10);
      if (end == p) break;
      p = end;
    }
    if (got < 2) {
      rc = GBBFS_ERR_IO;
      break;
    }
    long long u = vals[0], v = vals[1];
    if (dimacs) {
      u -= 1;
      v -= 1;
    }
    if (u < 0 || v < 0 || u > INT32_MAX || v > INT32_MAX) {
      rc = GBBFS_ERR_IO;
      break;
    }
    el->push_back(static_cast<int32_t>(u));
    el->push_back(static_cast<int32_t>(v));
  }
  free(lp);
  fclose(f);
  return rc;
}

// Matrix Market coordinate files (src/reader.h:186-256): a header line
// "%%MatrixMarket matrix coordinate <field> <symmetry>", '%' comment lines,
// "rows cols entries" (square only), then one 1-based "row col [value]" entry
// per line.  Fields pattern / real / double / integer (values are ignored),
// symmetries symmetric (undirected) / general / skew-symmetric.
int ReadMTX(const std::string& path, std::vector<int32_t>* el, bool* undirected) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return GBBFS_ERR_IO;
  char start[64] = {0}, object[64] = {0}, format[64] = {0}, field[64] = {0}, sym[64] = {0};
  int rc = GBBFS_OK;
  if (fscanf(f, "%63s %63s %63s %63s %63s", start, object, format, field, sym) != 5 ||
      strcmp(start, "%%MatrixMarket") != 0 || strcmp(object, "matrix") != 0 ||
      strcmp(format, "coordinate") != 0)
    rc = GBBFS_ERR_IO;
  bool weighted = false;
  if (rc == GBBFS_OK) {
    if (strcmp(field, "pattern") == 0)
      weighted = false;
    else if (!strcmp(field, "real") || !strcmp(field, "double") || !strcmp(field, "integer"))
      weighted = true;
    else
      rc = GBBFS_ERR_IO;   // complex or unknown
    if (strcmp(sym, "symmetric") == 0)
      *undirected = true;
    else if (!strcmp(sym, "general") || !strcmp(sym, "skew-symmetric"))
      *undirected = false;
    else
      rc = GBBFS_ERR_IO;
  }
  char* lp = nullptr;
  size_t cap = 0;
  bool sized = false;
  while (rc == GBBFS_OK && getline(&lp, &cap, f) >= 0) {
    const char* p = lp;
    while (*p == ' ' || *p == '\t') p++;
    if (*p == '%' || *p == '\n' || *p == '\r' || *p == '\0') continue;
    long long a = 0, b = 0;
    char* end = nullptr;
    a = strtoll(p, &end, 10);
    if (end == p) {
      rc = GBBFS_ERR_IO;
      break;
    }
    p = end;
    b = strtoll(p, &end, 10);
    if (end == p) {
      rc = GBBFS_ERR_IO;
      break;
    }
    p = end;
    if (!sized) {
      strtoll(p, &end, 10);   // the entry count: present, not used
      if (end == p || a != b) rc = GBBFS_ERR_IO;   // square only
      sized = true;
      continue;
    }
    (void)weighted;   // a value, if present, is ignored
    const long long u = a - 1, v = b - 1;
    if (u < 0 || v < 0 || u > INT32_MAX || v > INT32_MAX) {
      rc = GBBFS_ERR_IO;
      break;
    }
    el->push_back(static_cast<int32_t>(u));
    el->push_back(static_cast<int32_t>(v));
  }
  if (rc == GBBFS_OK && !sized) rc = GBBFS_ERR_IO;
  free(lp);
  fclose(f);
  return rc;
}

// METIS graph files (gapbs-verify/reader.h:88-140, src/reader.h ".graph"): '%'
// comment lines; a header "num_nodes num_edges [fmt]" with fmt 1 for edge
// weights (0 or 100: none; other codes are refused); then one line per vertex
// u (1-based neighbour ids, "neighbour weight" pairs when weighted), an empty
// line being a vertex without neighbours.  Every entry of a line is read.
// (The reference's own loop drops a line's last entry unless whitespace
// follows it; files whose lines end in a space read the same in both.)
int ReadMetis(const std::string& path, std::vector<int32_t>* el) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return GBBFS_ERR_IO;
  char* lp = nullptr;
  size_t cap = 0;
  int rc = GBBFS_OK;
  bool header = false, weighted = false;
  long long num_nodes = 0, u = 0;
  while (rc == GBBFS_OK && (!header || u < num_nodes) && getline(&lp, &cap, f) >= 0) {
    if (lp[0] == '%') continue;
    const char* p = lp;
    char* end = nullptr;
    if (!header) {
      num_nodes = strtoll(p, &end, 10);
      if (end == p || num_nodes < 0 || num_nodes > INT32_MAX) {
        rc = GBBFS_ERR_IO;
        break;
      }
      p = end;
      (void)strtoll(p, &end, 10);   // num_edges: not needed
      if (end == p) {
        rc = GBBFS_ERR_IO;
        break;
      }
      p = end;
      const long long fmt = strtoll(p, &end, 10);
      if (end != p) {
        if (fmt == 1)
          weighted = true;
        else if (fmt != 0 && fmt != 100)
          rc = GBBFS_ERR_IO;
      }
      header = true;
      continue;
    }
    for (;;) {
      const long long v = strtoll(p, &end, 10);
      if (end == p) break;
      p = end;
      if (weighted) {
        (void)strtoll(p, &end, 10);
        if (end == p) {
          rc = GBBFS_ERR_IO;
          break;
        }
        p = end;
      }
      if (v < 1 || v - 1 > INT32_MAX) {
        rc = GBBFS_ERR_IO;
        break;
      }
      el->push_back(static_cast<int32_t>(u));
      el->push_back(static_cast<int32_t>(v - 1));
    }
    u++;
  }
  if (rc == GBBFS_OK && !header) rc = GBBFS_ERR_IO;
  free(lp);
  fclose(f);
  return rc;
}

int ReadSG(const std::string& path, int64_t** offsets_out, int32_t** neigh_out,
           int64_t* n_out, int64_t* m_out) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return GBBFS_ERR_IO;
  unsigned char directed = 0;
  int64_t m = 0, n = 0;
  if (fread(&directed, 1, 1, f) != 1 || fread(&m, 8, 1, f) != 1 || fread(&n, 8, 1, f) != 1 ||
      n <= 0 || n > INT32_MAX || m < 0) {
    fclose(f);
    return GBBFS_ERR_IO;
  }
  if (directed) {
    fclose(f);
    return GBBFS_ERR_ARG;  // directed CSR is outside this engine
  }
  int64_t* off = static_cast<int64_t*>(malloc(sizeof(int64_t) * (n + 1)));
  int32_t* nbr = static_cast<int32_t*>(malloc(sizeof(int32_t) * (m > 0 ? m : 1)));
  if (!off || !nbr) {
    free(off);
    free(nbr);
    fclose(f);
    return GBBFS_ERR_NOMEM;
  }
  bool ok = fread(off, sizeof(int64_t), n + 1, f) == static_cast<size_t>(n + 1) &&
            (m == 0 || fread(nbr, sizeof(int32_t), m, f) == static_cast<size_t>(m));
  fclose(f);
  // The offsets written by the reference are relative to the first vertex.
  ok = ok && off[0] == 0 && off[n] == m;
  for (int64_t i = 0; ok && i < n; i++) ok = off[i] <= off[i + 1];
  for (int64_t e = 0; ok && e < m; e++) ok = nbr[e] >= 0 && nbr[e] < n;
  if (!ok) {
    free(off);
    free(nbr);
    return GBBFS_ERR_IO;
  }
  *offsets_out = off;
  *neigh_out = nbr;
  *n_out = n;
  *m_out = m;
  return GBBFS_OK;
}

}  // namespace

extern "C" {

int gbbfs_read_graph(const char* path, int symmetrize, int64_t** offsets_out,
                     int32_t** neigh_out, int64_t* n_out, int64_t* m_dir_out) {
  if (!path || !offsets_out || !neigh_out || !n_out || !m_dir_out) return GBBFS_ERR_ARG;
  const std::string p(path), suf = Suffix(p);
  if (suf == ".sg") return ReadSG(p, offsets_out, neigh_out, n_out, m_dir_out);
  std::vector<int32_t> el;
  bool undirected = false;
  int rc;
  if (suf == ".el")
    rc = ReadEdgeText(p, false, 2, &el);
  else if (suf == ".wel")
    rc = ReadEdgeText(p, false, 3, &el);
  else if (suf == ".gr")
    rc = ReadEdgeText(p, true, 3, &el);
  else if (suf == ".mtx")
    rc = ReadMTX(p, &el, &undirected);
  else if (suf == ".graph") {
    rc = ReadMetis(p, &el);
    undirected = true;   // METIS lists every edge on both endpoints' lines
  } else
    return GBBFS_ERR_ARG;
  if (rc != GBBFS_OK) return rc;
  // directed graphs are outside this engine; a symmetric .mtx is undirected
  if (!symmetrize && !undirected) return GBBFS_ERR_ARG;
  if (el.empty()) return GBBFS_ERR_IO;
  return gbbfs_build_csr(el.data(), static_cast<int64_t>(el.size() / 2), -1, offsets_out,
                         neigh_out, n_out, m_dir_out);
}

int gbbfs_write_sg(const char* path, const int64_t* offsets, const int32_t* neigh, int64_t n,
                   int64_t m_dir) {
  if (!path || !offsets || n <= 0 || m_dir < 0 || (m_dir > 0 && !neigh)) return GBBFS_ERR_ARG;
  FILE* f = fopen(path, "wb");
  if (!f) return GBBFS_ERR_IO;
  const unsigned char directed = 0;
  bool ok = fwrite(&directed, 1, 1, f) == 1 && fwrite(&m_dir, 8, 1, f) == 1 &&
            fwrite(&n, 8, 1, f) == 1 &&
            fwrite(offsets, sizeof(int64_t), n + 1, f) == static_cast<size_t>(n + 1) &&
            (m_dir == 0 ||
             fwrite(neigh, sizeof(int32_t), m_dir, f) == static_cast<size_t>(m_dir));
  if (fclose(f) != 0) ok = false;
  return ok ? GBBFS_OK : GBBFS_ERR_IO;
}

}  // extern "C"
