// GALES mesh files (the MESH! text format) read into the arrays of gales_mesh_desc.
// Host code only.
//
// Format and semantics follow src/fem/mesh/mesh.hpp:
//   header (read_header, 147-167): "MESH! 2D|3D", "nodes N", "elements N", "sides N",
//     then one bounds line per dimension ("X lo hi", ...);
//   "Node gid x y [z] flag" lines (read_nodes, 294-370: coordinates, flag; a node is on
//     the boundary when flag > 0);
//   "Element gid pid nnodes n_0 .. n_{k-1} flag" lines (read_elements, 184-242: only
//     the elements of the requested pid; on the boundary when flag > 0);
//   "Side gid pid nsn n_0 .. flag" lines (read_sides, 253-277: only the requested pid).
// Tokens are separated by any run of spaces and commas (algorithm.hpp:219-225).  The
// nodes of a pid are the sorted distinct gids its elements use and a node's local id is
// its position in that list (read_elements 239, read_nodes 303-331).  A boundary
// element's local side gets the flag of the Side line with the same node set, but only
// when every node of that side is a boundary node (el_side_info, 409-456; the last
// matching Side line wins); sides left with flag 0 are not boundary sides.
//
// Differences, all on inputs the reference cannot read: Node lines may come in any
// order (the reference needs them sorted by gid), a pid < 0 reads every element and
// side, and malformed lines are reported with their line number instead of aborting.
// Side lookup uses a hash of the sorted node set, and node lookup a sorted array, where
// the reference scans linearly (its cost is quadratic in the mesh size per rank).
#include <cuda_runtime.h>

#include <algorithm>
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/gales_asm.h"

struct gales_mesh_file {
  int32_t dim = 0, nen = 0;
  std::vector<double> coords;
  std::vector<int32_t> conn, node_flag, bd_el, bd_loc, bd_flag;
  std::vector<uint8_t> el_on_boundary;
  std::vector<int64_t> node_gid, el_gid;
};

namespace {

// local side tables of element.hpp:100-104 (quad), 145-149 (tri), 401-408 (hex), 455-460 (tet)
const int kTriSides[3][4] = {{1, 2}, {2, 0}, {0, 1}};
const int kQuadSides[4][4] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};
const int kTetSides[4][4] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};
const int kHexSides[6][4] = {{4, 5, 6, 7}, {0, 3, 2, 1}, {0, 4, 7, 3}, {1, 2, 6, 5}, {2, 3, 7, 6}, {1, 5, 4, 0}};

bool side_table(int dim, int nen, const int (**tab)[4], int& ns, int& nsn) {
  if (dim == 2 && nen == 3) { *tab = kTriSides; ns = 3; nsn = 2; return true; }
  if (dim == 2 && nen == 4) { *tab = kQuadSides; ns = 4; nsn = 2; return true; }
  if (dim == 3 && nen == 4) { *tab = kTetSides; ns = 4; nsn = 3; return true; }
  if (dim == 3 && nen == 8) { *tab = kHexSides; ns = 6; nsn = 4; return true; }
  return false;
}

// The whole file in memory (NUL-terminated); lines and tokens are views into it.
struct Reader {
  std::vector<char> buf;
  size_t pos = 0;
  long long line_no = 0;
  std::vector<std::pair<const char*, const char*>> tok;  // [begin, end) per token
  std::string err;

  static bool is_sep(char c) { return c == ' ' || c == ',' || c == '\t' || c == '\r'; }
  bool load(FILE* f) {
    char chunk[1 << 16];
    size_t n;
    while ((n = fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + n);
    if (ferror(f)) return false;
    buf.push_back('\0');
    return true;
  }
  bool next() {  // next line split into tokens; false at end of file
    const size_t end = buf.size() - 1;
    if (pos >= end) return false;
    ++line_no;
    tok.clear();
    const char* p = buf.data() + pos;
    const char* stop = buf.data() + end;
    while (p < stop && *p != '\n') {
      while (p < stop && *p != '\n' && is_sep(*p)) ++p;
      const char* q = p;
      while (q < stop && *q != '\n' && !is_sep(*q)) ++q;
      if (q > p) tok.emplace_back(p, q);
      p = q;
    }
    pos = (size_t)(p - buf.data()) + (p < stop ? 1 : 0);
    return true;
  }
  std::string str(size_t i) const { return std::string(tok[i].first, tok[i].second); }
  bool fail(const std::string& what) {
    err = "line " + std::to_string(line_no) + ": " + what;
    return false;
  }
  bool int_at(size_t i, long long& v) {
    if (i >= tok.size()) return fail("missing field " + std::to_string(i));
    const char* p = tok[i].first;
    const char* e = tok[i].second;
    const bool neg = *p == '-';
    if (*p == '-' || *p == '+') ++p;
    if (p == e || e - p > 18) {  // up to 18 digits fit int64; longer or empty: strtoll decides
      char* end = nullptr;
      errno = 0;
      v = strtoll(tok[i].first, &end, 10);
      if (errno || end != e || p == e) return fail("not an integer: '" + str(i) + "'");
      return true;
    }
    long long x = 0;
    for (; p < e; ++p) {
      const unsigned d = (unsigned)(*p - '0');
      if (d > 9) return fail("not an integer: '" + str(i) + "'");
      x = x * 10 + (long long)d;
    }
    v = neg ? -x : x;
    return true;
  }
  bool dbl_at(size_t i, double& v) {
    if (i >= tok.size()) return fail("missing field " + std::to_string(i));
    char* end = nullptr;
    errno = 0;
    v = strtod(tok[i].first, &end);
    if (errno == ERANGE && v != 0.0) return fail("number out of range: '" + str(i) + "'");
    if (end != tok[i].second) return fail("not a number: '" + str(i) + "'");
    return true;
  }
  bool is(size_t i, const char* word) const {
    const size_t n = strlen(word);
    return i < tok.size() && (size_t)(tok[i].second - tok[i].first) == n && memcmp(tok[i].first, word, n) == 0;
  }
  bool keyword(const char* kw) {
    if (!is(0, kw)) return fail(std::string("expected '") + kw + "'");
    return true;
  }
};

struct VecHash {
  size_t operator()(const std::vector<int64_t>& v) const {
    size_t h = 1469598103934665603ull;
    for (int64_t x : v) h = (h ^ (size_t)x) * 1099511628211ull;
    return h;
  }
};

int read_impl(const char* path, int32_t pid, gales_mesh_file& m, std::string& err) {
  Reader r;
  {
    FILE* f = fopen(path, "rb");
    if (!f) {
      err = std::string("cannot open ") + path;
      return GALES_ERR_BAD_INPUT;
    }
    const bool ok = r.load(f);
    fclose(f);
    if (!ok) {
      err = std::string("cannot read ") + path;
      return GALES_ERR_BAD_INPUT;
    }
  }
  auto bad = [&](void) {
    err = r.err;
    return GALES_ERR_BAD_INPUT;
  };
  // header
  if (!r.next()) {
    err = "empty file";
    return GALES_ERR_BAD_INPUT;
  }
  if (!r.keyword("MESH!")) return bad();
  if (!r.is(1, "2D") && !r.is(1, "3D")) {
    r.fail("expected 'MESH! 2D' or 'MESH! 3D'");
    return bad();
  }
  m.dim = r.is(1, "2D") ? 2 : 3;
  long long counts[3];
  const char* names[3] = {"nodes", "elements", "sides"};
  for (int i = 0; i < 3; ++i) {
    if (!r.next()) return (err = "file ends in the header", GALES_ERR_BAD_INPUT);
    if (!r.keyword(names[i]) || !r.int_at(1, counts[i])) return bad();
    if (counts[i] < 0) {
      r.fail("negative count");
      return bad();
    }
  }
  for (int d = 0; d < m.dim; ++d)
    if (!r.next()) return (err = "file ends in the header", GALES_ERR_BAD_INPUT);
  const long long n_nodes_tot = counts[0], n_el_tot = counts[1], n_sides_tot = counts[2];
  // nodes: kept in file order with their gid; matched to the elements' gids below
  std::vector<int64_t> f_gid;
  std::vector<double> f_xyz;
  std::vector<int32_t> f_flag;
  f_gid.reserve(n_nodes_tot);
  f_xyz.reserve(n_nodes_tot * m.dim);
  f_flag.reserve(n_nodes_tot);
  for (long long i = 0; i < n_nodes_tot; ++i) {
    if (!r.next()) return (err = "file ends in the Node lines", GALES_ERR_BAD_INPUT);
    long long gid, flag;
    if (!r.keyword("Node") || !r.int_at(1, gid) || !r.int_at(m.dim + 2, flag)) return bad();
    double x[3] = {0, 0, 0};
    for (int d = 0; d < m.dim; ++d)
      if (!r.dbl_at(2 + d, x[d])) return bad();
    f_gid.push_back(gid);
    for (int d = 0; d < m.dim; ++d) f_xyz.push_back(x[d]);
    f_flag.push_back((int32_t)flag);
  }
  // elements of the pid
  std::vector<int64_t> el_nodes_gid;
  std::vector<int32_t> el_flag;
  for (long long i = 0; i < n_el_tot; ++i) {
    if (!r.next()) return (err = "file ends in the Element lines", GALES_ERR_BAD_INPUT);
    long long gid, epid, nn, flag;
    if (!r.keyword("Element") || !r.int_at(1, gid) || !r.int_at(2, epid) || !r.int_at(3, nn)) return bad();
    if (pid >= 0 && epid != pid) continue;
    if (nn <= 0 || nn > 8) {
      r.fail("unsupported node count " + std::to_string(nn));
      return bad();
    }
    if (m.nen == 0) m.nen = (int32_t)nn;
    if (nn != m.nen) {
      r.fail("elements of different node counts in one mesh");
      return bad();
    }
    for (long long j = 0; j < nn; ++j) {
      long long g;
      if (!r.int_at(4 + j, g)) return bad();
      el_nodes_gid.push_back(g);
    }
    if (!r.int_at(4 + nn, flag)) return bad();
    m.el_gid.push_back(gid);
    el_flag.push_back((int32_t)flag);
  }
  // sides of the pid: sorted node set -> flag (the last matching line wins)
  std::unordered_map<std::vector<int64_t>, int32_t, VecHash> side_flag;
  for (long long i = 0; i < n_sides_tot; ++i) {
    if (!r.next()) return (err = "file ends in the Side lines", GALES_ERR_BAD_INPUT);
    long long gid, spid, nsn, flag;
    if (!r.keyword("Side") || !r.int_at(1, gid) || !r.int_at(2, spid) || !r.int_at(3, nsn)) return bad();
    if (pid >= 0 && spid != pid) continue;
    if (nsn <= 0 || nsn > 4) {
      r.fail("unsupported side node count " + std::to_string(nsn));
      return bad();
    }
    std::vector<int64_t> key((size_t)nsn);
    for (long long j = 0; j < nsn; ++j) {
      long long g;
      if (!r.int_at(4 + j, g)) return bad();
      key[j] = g;
    }
    if (!r.int_at(4 + nsn, flag)) return bad();
    std::sort(key.begin(), key.end());
    side_flag[key] = (int32_t)flag;
  }
  const int64_t n_el = (int64_t)m.el_gid.size();
  if (n_el == 0) {
    err = "no elements for this pid";
    return GALES_ERR_BAD_INPUT;
  }
  const int(*tab)[4] = nullptr;
  int ns = 0, nsn = 0;
  if (!side_table(m.dim, m.nen, &tab, ns, nsn)) {
    err = "unsupported element: " + std::to_string(m.dim) + "D with " + std::to_string(m.nen) + " nodes";
    return GALES_ERR_UNSUPPORTED;
  }
  // the pid's nodes: sorted distinct gids of its elements; local id = position.  Dense
  // gid ranges (the usual case) use a table over [lo, hi], sparse ones a sorted list.
  const auto mm = std::minmax_element(el_nodes_gid.begin(), el_nodes_gid.end());
  const int64_t lo = *mm.first, hi = *mm.second;
  std::vector<int32_t> table;
  const bool dense = lo >= 0 && (uint64_t)(hi - lo) <= 4 * (uint64_t)el_nodes_gid.size() + 1024;
  if (dense) {
    table.assign((size_t)(hi - lo + 1), -1);
    for (int64_t g : el_nodes_gid) table[(size_t)(g - lo)] = 0;
    int64_t next = 0;
    for (size_t i = 0; i < table.size(); ++i)
      if (table[i] == 0) {
        if (next > INT32_MAX) {
          err = "too many nodes for 32-bit node ids";
          return GALES_ERR_UNSUPPORTED;
        }
        table[i] = (int32_t)next++;
        m.node_gid.push_back(lo + (int64_t)i);
      }
  } else {
    m.node_gid = el_nodes_gid;
    std::sort(m.node_gid.begin(), m.node_gid.end());
    m.node_gid.erase(std::unique(m.node_gid.begin(), m.node_gid.end()), m.node_gid.end());
  }
  const size_t nn = m.node_gid.size();
  auto local_of = [&](int64_t g) -> int64_t {
    if (dense) return (g >= lo && g <= hi) ? (int64_t)table[(size_t)(g - lo)] : -1;
    auto it = std::lower_bound(m.node_gid.begin(), m.node_gid.end(), g);
    return (it != m.node_gid.end() && *it == g) ? (int64_t)(it - m.node_gid.begin()) : -1;
  };
  m.coords.assign(nn * m.dim, 0.0);
  m.node_flag.assign(nn, 0);
  std::vector<uint8_t> seen(nn, 0);
  for (size_t i = 0; i < f_gid.size(); ++i) {
    const int64_t l = local_of(f_gid[i]);
    if (l < 0) continue;
    if (seen[l]) {
      err = "node " + std::to_string(f_gid[i]) + " appears twice";
      return GALES_ERR_BAD_INPUT;
    }
    seen[l] = 1;
    for (int d = 0; d < m.dim; ++d) m.coords[l * m.dim + d] = f_xyz[i * m.dim + d];
    m.node_flag[l] = f_flag[i];
  }
  for (size_t l = 0; l < nn; ++l)
    if (!seen[l]) {
      err = "element node " + std::to_string(m.node_gid[l]) + " has no Node line";
      return GALES_ERR_BAD_INPUT;
    }
  if ((int64_t)nn > INT32_MAX) {
    err = "too many nodes for 32-bit node ids";
    return GALES_ERR_UNSUPPORTED;
  }
  m.conn.resize((size_t)n_el * m.nen);
  for (size_t i = 0; i < m.conn.size(); ++i) m.conn[i] = (int32_t)local_of(el_nodes_gid[i]);
  m.el_on_boundary.resize(n_el);
  for (int64_t e = 0; e < n_el; ++e) m.el_on_boundary[e] = el_flag[e] > 0 ? 1 : 0;
  // boundary sides of the boundary elements
  std::vector<int64_t> key(nsn);
  for (int64_t e = 0; e < n_el; ++e) {
    if (!m.el_on_boundary[e]) continue;
    const int32_t* en = &m.conn[(size_t)e * m.nen];
    for (int s = 0; s < ns; ++s) {
      bool all_bd = true;
      for (int j = 0; j < nsn; ++j) {
        const int32_t l = en[tab[s][j]];
        all_bd = all_bd && m.node_flag[l] > 0;
        key[j] = m.node_gid[l];
      }
      if (!all_bd) continue;
      std::sort(key.begin(), key.end());
      auto it = side_flag.find(key);
      if (it == side_flag.end() || it->second <= 0) continue;
      if (it->second >= GALES_MAX_FLAGS) {
        err = "side flag " + std::to_string(it->second) + " exceeds the supported range";
        return GALES_ERR_UNSUPPORTED;
      }
      m.bd_el.push_back((int32_t)e);
      m.bd_loc.push_back(s);
      m.bd_flag.push_back(it->second);
    }
  }
  return 0;
}

void copy_err(const std::string& s, char* err, int32_t err_len) {
  if (!err || err_len <= 0) return;
  const size_t n = std::min<size_t>(s.size(), (size_t)err_len - 1);
  memcpy(err, s.data(), n);
  err[n] = '\0';
}

}  // namespace

extern "C" {

int gales_mesh_read(const char* path, int32_t pid, gales_mesh_file** out, char* err, int32_t err_len) {
  if (out) *out = nullptr;
  if (!path || !out) {
    copy_err("null argument", err, err_len);
    return GALES_ERR_BAD_INPUT;
  }
  gales_mesh_file* m = new gales_mesh_file();
  std::string e;
  const int rc = read_impl(path, pid, *m, e);
  if (rc) {
    copy_err(e, err, err_len);
    delete m;
    return rc;
  }
  copy_err("", err, err_len);
  *out = m;
  return 0;
}

int gales_mesh_file_desc(const gales_mesh_file* m, gales_mesh_desc* desc, const int64_t** node_gid,
                         const int64_t** el_gid) {
  if (!m || !desc) return GALES_ERR_BAD_INPUT;
  memset(desc, 0, sizeof(*desc));
  desc->dim = m->dim;
  desc->nen = m->nen;
  desc->n_nodes = (int64_t)m->node_gid.size();
  desc->n_elements = (int64_t)m->el_gid.size();
  desc->coords = m->coords.data();
  desc->conn = m->conn.data();
  desc->node_flag = m->node_flag.data();
  desc->el_on_boundary = m->el_on_boundary.data();
  desc->n_bd_sides = (int64_t)m->bd_el.size();
  desc->bd_side_el = m->bd_el.data();
  desc->bd_side_local = m->bd_loc.data();
  desc->bd_side_flag = m->bd_flag.data();
  if (node_gid) *node_gid = m->node_gid.data();
  if (el_gid) *el_gid = m->el_gid.data();
  return 0;
}

void gales_mesh_file_free(gales_mesh_file* m) { delete m; }

}  // extern "C"
