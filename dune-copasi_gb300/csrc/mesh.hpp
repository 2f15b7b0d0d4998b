// Structured simplex grid, compartments and codim-1 faces.
//
// Grid construction follows dune/copasi/grid/make_multi_domain_grid.hh:76-100:
// "grid.cells" (default 1 per axis) cubes between "grid.origin" and origin +
// "grid.extensions", each cube split into simplices by StructuredGridFactory::
// createSimplexGrid (one simplex per axis permutation: the Kuhn split), then
// "grid.refinement_level" global refinements, which for this split equal the Kuhn split
// with cells * 2^level per axis.  Compartments are marked by evaluating each
// "compartments.<name>.expression" at the cell centre (make_multi_domain_grid.hh:118-154).
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "expr.hpp"
#include "ini.hpp"

namespace dcgpu {

struct Mesh {
  int dim = 2;
  int64_t nv = 0, ne = 0;
  std::vector<double> coords;    // nv * dim
  std::vector<int32_t> cells;    // ne * (dim + 1)
  std::vector<int> cells_per_axis;
  // per-cell data visible to compartment expressions ("gmsh_id" of Gmsh grids)
  std::map<std::string, std::vector<double>> cell_data;
};
Mesh read_gmsh(const std::string& path, int dim);

Mesh make_structured_simplex_mesh(int dim, const std::vector<int>& cells,
                                  const std::vector<double>& origin,
                                  const std::vector<double>& extensions);
Mesh make_mesh_from_config(const Ini& grid);

// codim-1 faces: face vertices (dim per face), the two neighbouring cells (e1 = -1 on
// the domain boundary) and the local index of the vertex opposite the face in each cell
struct Faces {
  int64_t nf = 0;
  std::vector<int32_t> verts;    // nf * dim (sorted)
  std::vector<int32_t> e0, e1;   // e0 < e1 when both exist
  std::vector<int8_t> l0, l1;    // local index of the opposite vertex
};
Faces compute_faces(const Mesh& m);

}  // namespace dcgpu
