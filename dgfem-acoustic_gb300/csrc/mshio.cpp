#include "mshio.h"

#include <algorithm>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <stdexcept>
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

// Token stream over the whole file (msh ASCII is whitespace separated apart
// from the quoted names in $PhysicalNames, which are handled line-wise).
struct Reader {
  std::istream& in;
  std::string path;
  template <class T>
  T get() {
    T v;
    if (!(in >> v)) fail(path, "unexpected end of data");
    return v;
  }
  void expect(const std::string& tok) {
    std::string s;
    if (!(in >> s) || s != tok) fail(path, "expected '" + tok + "', got '" + s + "'");
  }
  void skip_to(const std::string& end) {
    std::string s;
    while (in >> s)
      if (s == end) return;
    fail(path, "missing " + end);
  }
};

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
  std::ifstream in(path);
  if (!in.is_open()) fail(path, "cannot open file");
  MshFile f;
  Reader r{in, path};
  std::string tok;
  bool have_nodes = false, have_elems = false;
  while (in >> tok) {
    if (tok == "$MeshFormat") {
      f.version = r.get<double>();
      int ftype = r.get<int>();
      r.get<int>();  // data size
      if (ftype != 0) fail(path, "binary .msh files are not supported");
      if (f.version < 4.0 || f.version >= 5.0) fail(path, "only msh 4.x is supported");
      r.expect("$EndMeshFormat");
    } else if (tok == "$PhysicalNames") {
      int n = r.get<int>();
      std::string line;
      std::getline(in, line);
      for (int i = 0; i < n; ++i) {
        if (!std::getline(in, line)) fail(path, "truncated $PhysicalNames");
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
      f.node_tags.reserve(nnodes);
      f.node_xyz.reserve(3 * nnodes);
      for (int64_t b = 0; b < nblocks; ++b) {
        int a = r.get<int>(), c = r.get<int>();
        (void)a;
        (void)c;
        int parametric = r.get<int>();
        int64_t n = r.get<int64_t>();
        if (f.version >= 4.1) {
          size_t base = f.node_tags.size();
          for (int64_t i = 0; i < n; ++i) f.node_tags.push_back(r.get<int64_t>());
          for (int64_t i = 0; i < n; ++i) {
            for (int k = 0; k < 3; ++k) f.node_xyz.push_back(r.get<double>());
            if (parametric) fail(path, "parametric node coordinates are not supported");
          }
          (void)base;
        } else {
          for (int64_t i = 0; i < n; ++i) {
            f.node_tags.push_back(r.get<int64_t>());
            for (int k = 0; k < 3; ++k) f.node_xyz.push_back(r.get<double>());
            if (parametric) fail(path, "parametric node coordinates are not supported");
          }
        }
      }
      if ((int64_t)f.node_tags.size() != nnodes) fail(path, "node count mismatch");
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
        ElementBlock blk;
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
        blk.tags.resize(n);
        blk.nodes.resize(n * blk.nodes_per_elem);
        for (int64_t i = 0; i < n; ++i) {
          blk.tags[i] = r.get<int64_t>();
          for (int k = 0; k < blk.nodes_per_elem; ++k) blk.nodes[i * blk.nodes_per_elem + k] = r.get<int64_t>();
        }
        f.blocks.push_back(std::move(blk));
      }
      r.expect("$EndElements");
    } else if (!tok.empty() && tok[0] == '$' && tok.rfind("$End", 0) != 0) {
      r.skip_to("$End" + tok.substr(1));
    }
  }
  if (!have_nodes || !have_elems) fail(path, "missing $Nodes or $Elements");
  if (f.model_dim == 0)
    for (const auto& b : f.blocks) f.model_dim = std::max(f.model_dim, b.dim);
  return f;
}

VolumeMesh to_volume_mesh(const MshFile& f) {
  VolumeMesh m;
  m.dim = f.model_dim;
  if (m.dim != 2 && m.dim != 3) throw std::runtime_error("mesh dimension must be 2 or 3");
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
  m.xyz = f.node_xyz;
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
