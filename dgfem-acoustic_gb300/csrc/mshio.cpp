#include "mshio.h"

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <deque>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <thread>
#include <type_traits>
#include <unordered_map>

namespace dgmsh {

namespace {

struct TypeInfo {
  int type, dim, order, nodes;
};
// Gmsh element type ids (complete Lagrange simplices only).
const TypeInfo kTypes[] = {
    {15, 0, 0, 1},  {1, 1, 1, 2},   {8, 1, 2, 3},   {26, 1, 3, 4},  {27, 1, 4, 5},
    {2, 2, 1, 3},   {9, 2, 2, 6},   {21, 2, 3, 10}, {23, 2, 4, 15}, {4, 3, 1, 4},
    {11, 3, 2, 10}, {29, 3, 3, 20}, {30, 3, 4, 35},
};

const TypeInfo* find_type(int type) {
  for (const auto& t : kTypes)
    if (t.type == type) return &t;
  return nullptr;
}

[[noreturn]] void fail(const std::string& path, const std::string& msg) {
  throw std::runtime_error("msh '" + path + "': " + msg);
}

// Token cursor over the whole file held in memory (msh ASCII is whitespace
// separated apart from the quoted names in $PhysicalNames, which are read
// line-wise).
struct WsTable {
  bool t[256];
  WsTable() {
    for (int i = 0; i < 256; ++i) t[i] = i == ' ' || i == '\n' || i == '\r' || i == '\t' || i == '\v' || i == '\f';
  }
};
const WsTable kWs;
inline bool is_ws(char c) { return kWs.t[(unsigned char)c]; }

// Integer token at p (after whitespace); sets ok = false when there is none.
inline int64_t parse_int(const char*& p, const char* end, bool& ok) {
  while (p < end && is_ws(*p)) ++p;
  bool neg = false;
  if (p < end && (*p == '-' || *p == '+')) neg = *p == '-', ++p;
  const char* d0 = p;
  int64_t v = 0;
  while (p < end && *p >= '0' && *p <= '9') v = v * 10 + (*p - '0'), ++p;
  if (p == d0 || (p < end && !is_ws(*p))) {
    ok = false;
    return 0;
  }
  return neg ? -v : v;
}

// Floating-point token at p (correctly rounded by strtod; the file buffer
// ends with a NUL, so strtod cannot run past it).
inline double parse_double(const char*& p, const char* end, bool& ok) {
  while (p < end && is_ws(*p)) ++p;
  char* q = nullptr;
  const double v = std::strtod(p, &q);
  if (q == p || (q < end && !is_ws(*q))) {
    ok = false;
    return 0.0;
  }
  p = q;
  return v;
}

struct Reader {
  const char* p;
  const char* end;
  std::string path;
  bool at_end() {
    while (p < end && is_ws(*p)) ++p;
    return p >= end;
  }
  std::string token() {
    while (p < end && is_ws(*p)) ++p;
    const char* t = p;
    while (p < end && !is_ws(*p)) ++p;
    return std::string(t, p);
  }
  template <class T>
  T get() {
    bool ok = true;
    T v;
    if constexpr (std::is_floating_point<T>::value)
      v = (T)parse_double(p, end, ok);
    else
      v = (T)parse_int(p, end, ok);
    if (!ok) fail(path, at_end() ? "unexpected end of data" : "malformed number '" + token() + "'");
    return v;
  }
  void expect(const std::string& tok) {
    const std::string s = token();
    if (s != tok) fail(path, "expected '" + tok + "', got '" + s + "'");
  }
  void skip_to(const std::string& end_tok) {
    while (!at_end())
      if (token() == end_tok) return;
    fail(path, "missing " + end_tok);
  }
  std::string line() {  // rest of the current line
    const char* t = p;
    while (p < end && *p != '\n') ++p;
    std::string s(t, p);
    if (p < end) ++p;
    if (!s.empty() && s.back() == '\r') s.pop_back();
    return s;
  }
  // Skips n tokens; every `every` tokens records where the next one starts.
  void skip_tokens(int64_t n, int64_t every, std::vector<const char*>& marks) {
    for (int64_t k = 0; k < n; ++k) {
      while (p < end && is_ws(*p)) ++p;
      if (p >= end) fail(path, "unexpected end of data");
      if (k % every == 0) marks.push_back(p);
      while (p < end && !is_ws(*p)) ++p;
    }
  }
};

// A run of tokens to parse: `n` tokens from `start`, the first being token
// `first` of its section; `kind` says what they are.
struct Span {
  const char* start;
  int64_t first, n;
  int kind;       // 0: node tags, 1: node coordinates, 2: 4.0 node records (tag x y z), 3: element records
  int64_t base;   // first node index (kinds 0-2) or first element of the block (kind 3)
  int per;        // tokens per element record (kind 3)
  ElementBlock* blk;
};

constexpr int64_t kSpan = 1 << 16;  // tokens per parallel task

void parse_spans(const std::vector<Span>& spans, MshFile& f, const std::string& path, const char* end) {
  std::atomic<size_t> next{0};
  std::atomic<bool> bad{false};
  auto work = [&] {
    for (;;) {
      const size_t i = next.fetch_add(1);
      if (i >= spans.size() || bad.load()) return;
      const Span& s = spans[i];
      const char* p = s.start;
      bool ok = true;
      for (int64_t k = 0; k < s.n && ok; ++k) {
        const int64_t t = s.first + k;
        switch (s.kind) {
          case 0: f.node_tags[s.base + t] = parse_int(p, end, ok); break;
          case 1: f.node_xyz[3 * s.base + t] = parse_double(p, end, ok); break;
          case 2: {
            const int64_t node = s.base + t / 4, c = t % 4;
            if (c == 0)
              f.node_tags[node] = parse_int(p, end, ok);
            else
              f.node_xyz[3 * node + c - 1] = parse_double(p, end, ok);
            break;
          }
          default: {
            const int64_t e = t / s.per, c = t % s.per;
            if (c == 0)
              s.blk->tags[e] = parse_int(p, end, ok);
            else
              s.blk->nodes[e * (s.per - 1) + c - 1] = parse_int(p, end, ok);
          }
        }
      }
      if (!ok) bad = true;
    }
  };
  const unsigned hw = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  const unsigned nt = (unsigned)std::min<size_t>(hw, std::max<size_t>(1, spans.size()));
  if (nt <= 1) {
    work();
  } else {
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < nt; ++t) pool.emplace_back(work);
    for (auto& th : pool) th.join();
  }
  if (bad) fail(path, "malformed number in $Nodes or $Elements");
}

// Records spans of n tokens from the reader's position, then skips them.
void add_spans(Reader& r, std::vector<Span>& spans, Span proto, int64_t n) {
  std::vector<const char*> marks;
  r.skip_tokens(n, kSpan, marks);
  for (size_t k = 0; k < marks.size(); ++k) {
    Span s = proto;
    s.start = marks[k];
    s.first = (int64_t)k * kSpan;
    s.n = std::min<int64_t>(kSpan, n - s.first);
    spans.push_back(s);
  }
}

}  // namespace

int gmsh_type_nodes(int type) {
  auto t = find_type(type);
  return t ? t->nodes : 0;
}
int gmsh_type_dim(int type) {
  auto t = find_type(type);
  return t ? t->dim : -1;
}
int gmsh_type_order(int type) {
  auto t = find_type(type);
  return t ? t->order : -1;
}
int gmsh_type_for(int dim, int order) {
  for (const auto& t : kTypes)
    if (t.dim == dim && t.order == order) return t.type;
  return 0;
}

MshFile read_msh(const std::string& path) {
  // the whole file in memory, NUL-terminated
  std::string buf;
  {
    FILE* fp = std::fopen(path.c_str(), "rb");
    if (!fp) fail(path, "cannot open file");
    std::fseek(fp, 0, SEEK_END);
    const long sz = std::ftell(fp);
    std::fseek(fp, 0, SEEK_SET);
    buf.resize(sz > 0 ? (size_t)sz : 0);
    const size_t got = sz > 0 ? std::fread(&buf[0], 1, (size_t)sz, fp) : 0;
    std::fclose(fp);
    if (got != buf.size()) fail(path, "read error");
  }
  MshFile f;
  Reader r{buf.data(), buf.data() + buf.size(), path};
  std::vector<Span> spans;
  // element blocks are filled in place by the parallel pass: keep their storage stable
  std::deque<ElementBlock> blocks;
  bool have_nodes = false, have_elems = false;
  while (!r.at_end()) {
    const std::string tok = r.token();
    if (tok == "$MeshFormat") {
      f.version = r.get<double>();
      int ftype = r.get<int>();
      r.get<int>();  // data size
      if (ftype != 0) fail(path, "binary .msh files are not supported");
      if (f.version < 4.0 || f.version >= 5.0) fail(path, "only msh 4.x is supported");
      r.expect("$EndMeshFormat");
    } else if (tok == "$PhysicalNames") {
      int n = r.get<int>();
      r.line();
      for (int i = 0; i < n; ++i) {
        if (r.at_end()) fail(path, "truncated $PhysicalNames");
        const std::string line = r.line();
        std::istringstream ls(line);
        PhysicalGroup g;
        ls >> g.dim >> g.tag;
        auto q0 = line.find('"'), q1 = line.rfind('"');
        if (q0 == std::string::npos || q1 == q0) fail(path, "bad physical name line");
        g.name = line.substr(q0 + 1, q1 - q0 - 1);
        f.physicals.push_back(g);
      }
      r.expect("$EndPhysicalNames");
    } else if (tok == "$Entities") {
      int64_t counts[4];
      for (auto& c : counts) c = r.get<int64_t>();
      for (int d = 0; d < 4; ++d) {
        if (counts[d] > 0) f.model_dim = std::max(f.model_dim, d);
        for (int64_t i = 0; i < counts[d]; ++i) {
          int tag = r.get<int>();
          // 4.1 points carry X Y Z, everything else (and 4.0 points) a box.
          int ncoord = (d == 0 && f.version >= 4.1) ? 3 : 6;
          for (int k = 0; k < ncoord; ++k) r.get<double>();
          int nphys = r.get<int>();
          std::vector<int> phys(nphys);
          for (auto& p : phys) p = r.get<int>();
          f.entity_phys[d][tag] = phys;
          if (d > 0) {
            int nb = r.get<int>();
            for (int k = 0; k < nb; ++k) r.get<int>();
          }
        }
      }
      r.expect("$EndEntities");
    } else if (tok == "$Nodes") {
      have_nodes = true;
      int64_t nblocks = r.get<int64_t>(), nnodes = r.get<int64_t>();
      if (f.version >= 4.1) {
        r.get<int64_t>();
        r.get<int64_t>();
      }
      if (nnodes < 0) fail(path, "node count mismatch");
      f.node_tags.assign(nnodes, 0);
      f.node_xyz.assign(3 * nnodes, 0.0);
      int64_t base = 0;
      for (int64_t b = 0; b < nblocks; ++b) {
        r.get<int>();
        r.get<int>();
        int parametric = r.get<int>();
        int64_t n = r.get<int64_t>();
        if (n < 0 || base + n > nnodes) fail(path, "node count mismatch");
        if (parametric && n > 0) fail(path, "parametric node coordinates are not supported");
        if (f.version >= 4.1) {
          add_spans(r, spans, Span{nullptr, 0, 0, 0, base, 0, nullptr}, n);
          add_spans(r, spans, Span{nullptr, 0, 0, 1, base, 0, nullptr}, 3 * n);
        } else {
          add_spans(r, spans, Span{nullptr, 0, 0, 2, base, 0, nullptr}, 4 * n);
        }
        base += n;
      }
      if (base != nnodes) fail(path, "node count mismatch");
      r.expect("$EndNodes");
    } else if (tok == "$Elements") {
      have_elems = true;
      int64_t nblocks = r.get<int64_t>();
      r.get<int64_t>();
      if (f.version >= 4.1) {
        r.get<int64_t>();
        r.get<int64_t>();
      }
      for (int64_t b = 0; b < nblocks; ++b) {
        blocks.emplace_back();
        ElementBlock& blk = blocks.back();
        int a = r.get<int>(), c = r.get<int>();
        if (f.version >= 4.1) {
          blk.dim = a;
          blk.entity = c;
        } else {
          blk.entity = a;
          blk.dim = c;
        }
        blk.type = r.get<int>();
        int64_t n = r.get<int64_t>();
        blk.nodes_per_elem = gmsh_type_nodes(blk.type);
        if (blk.nodes_per_elem == 0) fail(path, "unsupported element type " + std::to_string(blk.type));
        if (n < 0) fail(path, "bad element count");
        blk.tags.resize(n);
        blk.nodes.resize(n * blk.nodes_per_elem);
        const int per = 1 + blk.nodes_per_elem;
        add_spans(r, spans, Span{nullptr, 0, 0, 3, 0, per, &blk}, n * per);
      }
      r.expect("$EndElements");
    } else if (!tok.empty() && tok[0] == '$' && tok.rfind("$End", 0) != 0) {
      r.skip_to("$End" + tok.substr(1));
    }
  }
  if (!have_nodes || !have_elems) fail(path, "missing $Nodes or $Elements");
  parse_spans(spans, f, path, buf.data() + buf.size());
  for (auto& b : blocks) f.blocks.push_back(std::move(b));
  if (f.model_dim == 0)
    for (const auto& b : f.blocks) f.model_dim = std::max(f.model_dim, b.dim);
  return f;
}

VolumeMesh to_volume_mesh(MshFile f) {
  VolumeMesh m;
  m.dim = f.model_dim;
  if (m.dim < 1 || m.dim > 3) throw std::runtime_error("mesh dimension must be 1, 2 or 3");
  for (const auto& b : f.blocks)
    if (b.dim == m.dim) {
      m.type = b.type;
      break;
    }
  if (m.type == 0) throw std::runtime_error("mesh has no elements of its model dimension");
  m.order = gmsh_type_order(m.type);
  m.nodes_per_elem = gmsh_type_nodes(m.type);
  if (gmsh_type_dim(m.type) != m.dim) throw std::runtime_error("element type does not match model dimension");
  m.node_tags = f.node_tags;
  m.xyz = std::move(f.node_xyz);
  int64_t max_tag = 0;
  for (auto t : f.node_tags) max_tag = std::max(max_tag, t);
  std::vector<int64_t> tag2idx;
  std::unordered_map<int64_t, int64_t> sparse;
  bool dense = max_tag <= 4 * (int64_t)f.node_tags.size() + 16;
  if (dense) {
    tag2idx.assign(max_tag + 1, -1);
    for (size_t i = 0; i < f.node_tags.size(); ++i) tag2idx[f.node_tags[i]] = (int64_t)i;
  } else {
    for (size_t i = 0; i < f.node_tags.size(); ++i) sparse[f.node_tags[i]] = (int64_t)i;
  }
  auto idx = [&](int64_t tag) -> int64_t {
    int64_t v = -1;
    if (dense) {
      if (tag >= 0 && tag <= max_tag) v = tag2idx[tag];
    } else {
      auto it = sparse.find(tag);
      if (it != sparse.end()) v = it->second;
    }
    if (v < 0) throw std::runtime_error("element references unknown node tag " + std::to_string(tag));
    return v;
  };
  for (const auto& b : f.blocks) {
    if (b.dim != m.dim || b.type != m.type) continue;
    m.elem_tags.insert(m.elem_tags.end(), b.tags.begin(), b.tags.end());
    for (auto t : b.nodes) m.elem_nodes.push_back(idx(t));
  }
  // Boundary groups of dimension dim-1 in ascending tag order.
  std::vector<PhysicalGroup> groups;
  for (const auto& g : f.physicals)
    if (g.dim == m.dim - 1) groups.push_back(g);
  // Physical groups may also exist only through entity tags (no name).
  for (const auto& kv : f.entity_phys[m.dim - 1])
    for (int ptag : kv.second) {
      bool known = false;
      for (const auto& g : groups) known |= (g.tag == ptag);
      if (!known) groups.push_back(PhysicalGroup{m.dim - 1, ptag, ""});
    }
  std::sort(groups.begin(), groups.end(), [](const PhysicalGroup& a, const PhysicalGroup& b) { return a.tag < b.tag; });
  for (const auto& g : groups) {
    std::vector<int64_t> nodes;
    for (const auto& b : f.blocks) {
      if (b.dim != m.dim - 1) continue;
      auto it = f.entity_phys[m.dim - 1].find(b.entity);
      if (it == f.entity_phys[m.dim - 1].end()) continue;
      if (std::find(it->second.begin(), it->second.end(), g.tag) == it->second.end()) continue;
      for (auto t : b.nodes) nodes.push_back(idx(t));
    }
    std::sort(nodes.begin(), nodes.end());
    nodes.erase(std::unique(nodes.begin(), nodes.end()), nodes.end());
    m.bc_groups.push_back(g);
    m.bc_group_nodes.push_back(std::move(nodes));
  }
  return m;
}

VolumeMesh load_volume_mesh(const std::string& path) { return to_volume_mesh(read_msh(path)); }

void write_msh41(const std::string& path, int dim, int order, const std::vector<double>& xyz,
                 const std::vector<int64_t>& elem_nodes, const std::vector<WriteGroup>& groups) {
  FILE* fp = std::fopen(path.c_str(), "w");
  if (!fp) throw std::runtime_error("cannot write " + path);
  int vtype = gmsh_type_for(dim, order), ftype = gmsh_type_for(dim - 1, order);
  int vn = gmsh_type_nodes(vtype), fn = gmsh_type_nodes(ftype);
  int64_t nnodes = (int64_t)xyz.size() / 3, nelem = (int64_t)elem_nodes.size() / vn;
  std::fprintf(fp, "$MeshFormat\n4.1 0 8\n$EndMeshFormat\n$PhysicalNames\n%zu\n", groups.size() + 1);
  for (const auto& g : groups) std::fprintf(fp, "%d %d \"%s\"\n", dim - 1, g.tag, g.name.c_str());
  std::fprintf(fp, "%d %d \"Domain\"\n$EndPhysicalNames\n", dim, 1000000);
  // One boundary entity per group, one volume entity.
  int64_t counts[4] = {0, 0, 0, 0};
  counts[dim - 1] = (int64_t)groups.size();
  counts[dim] = 1;
  std::fprintf(fp, "$Entities\n%lld %lld %lld %lld\n", (long long)counts[0], (long long)counts[1],
               (long long)counts[2], (long long)counts[3]);
  for (size_t i = 0; i < groups.size(); ++i)
    std::fprintf(fp, "%zu 0 0 0 0 0 0 1 %d 0\n", i + 1, groups[i].tag);
  std::fprintf(fp, "1 0 0 0 0 0 0 1 %d 0\n$EndEntities\n", 1000000);
  std::fprintf(fp, "$Nodes\n1 %lld 1 %lld\n%d 1 0 %lld\n", (long long)nnodes, (long long)nnodes, dim,
               (long long)nnodes);
  for (int64_t i = 0; i < nnodes; ++i) std::fprintf(fp, "%lld\n", (long long)(i + 1));
  for (int64_t i = 0; i < nnodes; ++i)
    std::fprintf(fp, "%.17g %.17g %.17g\n", xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
  int64_t nface = 0;
  for (const auto& g : groups) nface += (int64_t)g.face_nodes.size() / fn;
  std::fprintf(fp, "$EndNodes\n$Elements\n%zu %lld 1 %lld\n", groups.size() + 1, (long long)(nelem + nface),
               (long long)(nelem + nface));
  int64_t etag = 1;
  for (size_t i = 0; i < groups.size(); ++i) {
    int64_t n = (int64_t)groups[i].face_nodes.size() / fn;
    std::fprintf(fp, "%d %zu %d %lld\n", dim - 1, i + 1, ftype, (long long)n);
    for (int64_t e = 0; e < n; ++e) {
      std::fprintf(fp, "%lld", (long long)etag++);
      for (int k = 0; k < fn; ++k) std::fprintf(fp, " %lld", (long long)(groups[i].face_nodes[e * fn + k] + 1));
      std::fprintf(fp, "\n");
    }
  }
  std::fprintf(fp, "%d 1 %d %lld\n", dim, vtype, (long long)nelem);
  for (int64_t e = 0; e < nelem; ++e) {
    std::fprintf(fp, "%lld", (long long)etag++);
    for (int k = 0; k < vn; ++k) std::fprintf(fp, " %lld", (long long)(elem_nodes[e * vn + k] + 1));
    std::fprintf(fp, "\n");
  }
  std::fprintf(fp, "$EndElements\n");
  std::fclose(fp);
}

}  // namespace dgmsh
