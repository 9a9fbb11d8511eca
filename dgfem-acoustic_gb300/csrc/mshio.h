// Gmsh .msh 4.0 / 4.1 ASCII reader and 4.1 writer.
//
// The solver reads its mesh the way the reference obtains it through the Gmsh
// SDK (src/Mesh.cpp:40-48, src/configParser.cpp:197-223):
//   * the model dimension is the largest entity dimension in $Entities;
//   * only the first element type of that dimension is used;
//   * boundary conditions come from physical groups of dimension dim-1, and a
//     group's node set is every node of every element of the entities that
//     carry the group's tag (gmsh::model::mesh::getNodesForPhysicalGroup).
#pragma once
#include <cstddef>
#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace dgmsh {

struct ElementBlock {
  int dim = 0, entity = 0, type = 0, nodes_per_elem = 0;
  std::vector<int64_t> tags;   // element tags
  std::vector<int64_t> nodes;  // node tags, nodes_per_elem per element
};

struct PhysicalGroup {
  int dim = 0, tag = 0;
  std::string name;
};

struct MshFile {
  double version = 0.0;
  int model_dim = 0;                               // max entity dimension
  std::vector<PhysicalGroup> physicals;            // from $PhysicalNames
  std::map<int, std::vector<int>> entity_phys[4];  // entity tag -> physical tags
  std::vector<int64_t> node_tags;                  // file order
  std::vector<double> node_xyz;                    // 3 per node, file order
  std::vector<ElementBlock> blocks;                // file order
};

// Throws std::runtime_error with a message on malformed input.
MshFile read_msh(const std::string& path);

// Nodes per element for the Gmsh element types the solver understands
// (points, lines, triangles, tetrahedra of order 1..4); 0 if unknown.
int gmsh_type_nodes(int type);
// Topological dimension and order of a Gmsh element type (-1 if unknown).
int gmsh_type_dim(int type);
int gmsh_type_order(int type);
// Gmsh type id for (dim, order), 0 if unsupported.
int gmsh_type_for(int dim, int order);

// Volume mesh in solver form: node index = position in node_tags (file order),
// elements of the first element type of the model dimension, boundary groups
// of dimension dim-1 sorted by ascending physical tag (Gmsh's
// getPhysicalGroups order), each with the sorted node indices of its elements.
struct VolumeMesh {
  int dim = 0, order = 0, type = 0, nodes_per_elem = 0;
  std::vector<int64_t> node_tags;   // index -> tag
  std::vector<double> xyz;          // index -> coordinates
  std::vector<int64_t> elem_tags;   // element tags
  std::vector<int64_t> elem_nodes;  // node indices, nodes_per_elem per element
  std::vector<PhysicalGroup> bc_groups;             // dim-1 groups, ascending tag
  std::vector<std::vector<int64_t>> bc_group_nodes; // node indices per group
};

VolumeMesh to_volume_mesh(MshFile f);
VolumeMesh load_volume_mesh(const std::string& path);

// Writes a 4.1 ASCII mesh: one volume entity holding all elements and one
// boundary entity per physical group (each with its line/triangle elements).
struct WriteGroup {
  int tag = 0;
  std::string name;
  std::vector<int64_t> face_nodes;  // node indices, (dim-1)-simplices of the same order
};
void write_msh41(const std::string& path, int dim, int order, const std::vector<double>& xyz,
                 const std::vector<int64_t>& elem_nodes, const std::vector<WriteGroup>& groups);

}  // namespace dgmsh
