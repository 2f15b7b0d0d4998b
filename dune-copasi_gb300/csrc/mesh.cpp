#include "mesh.hpp"

#include <algorithm>
#include <fstream>
#include <numeric>
#include <sstream>
#include <unordered_map>

namespace dcgpu {

Mesh make_structured_simplex_mesh(int dim, const std::vector<int>& cells,
                                  const std::vector<double>& origin,
                                  const std::vector<double>& extensions) {
  if (dim != 2 && dim != 3) throw ConfigError("only 2D triangle and 3D tetrahedral grids are supported");
  Mesh m;
  m.dim = dim;
  m.cells_per_axis = cells;
  std::vector<int64_t> npts(dim), stride(dim);
  int64_t nv = 1, ncube = 1;
  for (int d = 0; d < dim; ++d) {
    if (cells[d] < 1) throw ConfigError("grid.cells must be positive");
    npts[d] = cells[d] + 1;
    stride[d] = nv;
    nv *= npts[d];
    ncube *= cells[d];
  }
  if (nv > INT32_MAX / 2) throw ConfigError("grid too large for 32-bit vertex indices");
  m.nv = nv;
  m.coords.resize(nv * dim);
  for (int64_t v = 0; v < nv; ++v) {
    int64_t r = v;
    for (int d = 0; d < dim; ++d) {
      int64_t i = r % npts[d];
      r /= npts[d];
      // same spacing as numpy.linspace(origin, origin + extension, n)
      const double upper = origin[d] + extensions[d];
      const double step = (upper - origin[d]) / static_cast<double>(cells[d]);
      double x = (i == cells[d]) ? upper : static_cast<double>(i) * step + origin[d];
      m.coords[v * dim + d] = x;
    }
  }
  std::vector<std::vector<int>> perms;
  std::vector<int> p(dim);
  std::iota(p.begin(), p.end(), 0);
  do perms.push_back(p); while (std::next_permutation(p.begin(), p.end()));
  const int nl = dim + 1;
  m.ne = ncube * static_cast<int64_t>(perms.size());
  m.cells.resize(m.ne * nl);
  int64_t e = 0;
  for (int64_t c = 0; c < ncube; ++c) {
    int64_t r = c, base = 0;
    for (int d = 0; d < dim; ++d) {
      base += (r % cells[d]) * stride[d];
      r /= cells[d];
    }
    for (const auto& perm : perms) {
      int64_t cur = base;
      m.cells[e * nl] = static_cast<int32_t>(cur);
      for (int k = 0; k < dim; ++k) {
        cur += stride[perm[k]];
        m.cells[e * nl + k + 1] = static_cast<int32_t>(cur);
      }
      ++e;
    }
  }
  return m;
}

// Gmsh MSH 2.x ASCII (the format Dune's GmshReader reads, make_multi_domain_grid.hh:66-76):
// nodes in file order (ids mapped to 0..n-1), the elements of the grid's dimension (type 2
// triangles, type 4 tetrahedra) in file order, lower-dimensional elements skipped; the first
// tag of an element is its physical entity, kept as the cell data "gmsh_id".
Mesh read_gmsh(const std::string& path, int dim) {
  std::ifstream in(path);
  if (!in) throw ConfigError("cannot open grid file '" + path + "'");
  Mesh m;
  m.dim = dim;
  std::unordered_map<long, int32_t> idmap;
  std::vector<double> phys;
  const int want = dim == 2 ? 2 : 4;
  std::string line;
  bool have_nodes = false;
  while (std::getline(in, line)) {
    line = trim(line);
    if (line == "$MeshFormat") {
      std::getline(in, line);
      std::istringstream ss(line);
      std::string ver;
      int ftype = 1;
      ss >> ver >> ftype;
      if (ver.empty() || ver[0] != '2' || ftype != 0) throw ConfigError("only ASCII Gmsh MSH 2.x files are supported");
    } else if (line == "$Nodes") {
      std::getline(in, line);
      const long n = std::stol(line);
      m.coords.assign(static_cast<size_t>(n) * dim, 0.0);
      for (long k = 0; k < n; ++k) {
        std::getline(in, line);
        std::istringstream ss(line);
        long id;
        double xyz[3] = {0, 0, 0};
        ss >> id >> xyz[0] >> xyz[1] >> xyz[2];
        if (!ss && !(dim == 2 && ss.eof())) throw ConfigError("malformed node line in '" + path + "'");
        idmap[id] = static_cast<int32_t>(k);
        for (int d = 0; d < dim; ++d) m.coords[k * dim + d] = xyz[d];
      }
      m.nv = n;
      have_nodes = true;
    } else if (line == "$Elements") {
      std::getline(in, line);
      const long n = std::stol(line);
      for (long k = 0; k < n; ++k) {
        std::getline(in, line);
        std::istringstream ss(line);
        long id, typ, ntags;
        ss >> id >> typ >> ntags;
        std::vector<long> tags(ntags);
        for (auto& t : tags) ss >> t;
        if (typ != want) continue;
        for (int a = 0; a <= dim; ++a) {
          long v;
          ss >> v;
          auto it = idmap.find(v);
          if (!ss || it == idmap.end()) throw ConfigError("malformed element line in '" + path + "'");
          m.cells.push_back(it->second);
        }
        phys.push_back(ntags > 0 ? static_cast<double>(tags[0]) : 0.0);
      }
    }
  }
  if (!have_nodes || phys.empty())
    throw ConfigError("grid file '" + path + "' has no nodes or no " + std::to_string(dim) + "D elements");
  m.ne = static_cast<int64_t>(phys.size());
  m.cell_data["gmsh_id"] = phys;
  return m;
}

Mesh make_mesh_from_config(const Ini& grid) {
  if (grid.has_key("path")) {
    const int dim = static_cast<int>(grid.get_long("dimension", 2));
    if (dim != 2 && dim != 3) throw ConfigError("only grid.dimension 2 or 3 is supported");
    if (grid.get_long("refinement_level", 0) != 0)
      throw ConfigError("grid.refinement_level is not supported together with grid.path");
    return read_gmsh(grid.get("path", ""), dim);
  }
  int dim = 2;
  if (grid.has_key("dimension")) dim = static_cast<int>(grid.get_long("dimension", 2));
  else if (grid.has_key("extensions")) dim = static_cast<int>(grid.get_doubles("extensions", {}).size());
  if (dim != 2 && dim != 3) throw ConfigError("only grid.dimension 2 or 3 is supported");
  auto cd = grid.get_doubles("cells", std::vector<double>(dim, 1.0));
  auto ext = grid.get_doubles("extensions", std::vector<double>(dim, 1.0));
  auto org = grid.get_doubles("origin", std::vector<double>(dim, 0.0));
  if (static_cast<int>(cd.size()) != dim || static_cast<int>(ext.size()) != dim || static_cast<int>(org.size()) != dim)
    throw ConfigError("grid.cells/extensions/origin must have 'dimension' entries");
  long level = grid.get_long("refinement_level", 0);
  std::vector<int> cells(dim);
  for (int d = 0; d < dim; ++d) cells[d] = static_cast<int>(cd[d]) << level;
  return make_structured_simplex_mesh(dim, cells, org, ext);
}

Faces compute_faces(const Mesh& m) {
  const int d = m.dim, nl = d + 1;
  const int64_t n = m.ne * nl;
  struct Rec { int32_t v[3]; int32_t e; int8_t l; };
  std::vector<Rec> recs(n);
  for (int64_t e = 0; e < m.ne; ++e) {
    for (int k = 0; k < nl; ++k) {
      Rec r{};
      int c = 0;
      for (int j = 0; j < nl; ++j)
        if (j != k) r.v[c++] = m.cells[e * nl + j];
      for (int i = 1; i < d; ++i)  // insertion sort of the d face vertices
        for (int j = i; j > 0 && r.v[j - 1] > r.v[j]; --j) std::swap(r.v[j - 1], r.v[j]);
      if (d == 2) r.v[2] = -1;
      r.e = static_cast<int32_t>(e);
      r.l = static_cast<int8_t>(k);
      recs[e * nl + k] = r;
    }
  }
  auto key_less = [](const Rec& a, const Rec& b) {
    if (a.v[0] != b.v[0]) return a.v[0] < b.v[0];
    if (a.v[1] != b.v[1]) return a.v[1] < b.v[1];
    if (a.v[2] != b.v[2]) return a.v[2] < b.v[2];
    return a.e < b.e;
  };
  std::sort(recs.begin(), recs.end(), key_less);
  Faces f;
  auto same = [&](const Rec& a, const Rec& b) { return a.v[0] == b.v[0] && a.v[1] == b.v[1] && a.v[2] == b.v[2]; };
  for (int64_t i = 0; i < n;) {
    bool pair = (i + 1 < n) && same(recs[i], recs[i + 1]);
    for (int k = 0; k < d; ++k) f.verts.push_back(recs[i].v[k]);
    f.e0.push_back(recs[i].e);
    f.l0.push_back(recs[i].l);
    if (pair) {
      f.e1.push_back(recs[i + 1].e);
      f.l1.push_back(recs[i + 1].l);
      i += 2;
    } else {
      f.e1.push_back(-1);
      f.l1.push_back(-1);
      i += 1;
    }
  }
  f.nf = static_cast<int64_t>(f.e0.size());
  return f;
}

}  // namespace dcgpu
