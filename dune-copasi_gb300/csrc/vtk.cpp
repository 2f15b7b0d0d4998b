// VTK output of the state, replacing ModelMultiCompartment::write_vtk /
// ModelSingleCompartment::write_vtk (dune/copasi/model/diffusion_reaction/
// model_multi_compartment.impl.hh:219-293, model_single_compartment.impl.hh:251-300).
//
// Per compartment with species, one unstructured-grid piece of the compartment's cells with
// one scalar vertex field per species is written to "<dir>/<stem>-<compartment>-NNNNN.vtu",
// NNNNN counting the calls for that path, and the time series "<dir>/<stem>-<compartment>.pvd"
// is rewritten to list every file so far with its time (Dune's VTKSequenceWriter naming;
// data are written as ASCII rather than base64).  append = 0 restarts the series.
#include <cerrno>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <sys/stat.h>

#include "model.hpp"

namespace dcgpu {

namespace {

void make_dirs(const std::string& path) {
  std::string cur;
  for (size_t i = 0; i < path.size(); ++i) {
    cur += path[i];
    if ((path[i] == '/' || i + 1 == path.size()) && !cur.empty() && cur != "/") {
      if (mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST)
        throw ConfigError("cannot create output directory '" + cur + "'");
    }
  }
}

}  // namespace

void Model::write_vtk(const std::vector<double>& x_ref, double t, const std::string& path, bool append) const {
  if (path.empty()) throw ConfigError("empty VTK output path");
  make_dirs(path);
  std::string dir = path;
  while (dir.size() > 1 && dir.back() == '/') dir.pop_back();
  const auto slash = dir.find_last_of('/');
  const std::string stem = slash == std::string::npos ? dir : dir.substr(slash + 1);
  auto& steps = vtk_steps[dir];
  if (!append) steps.clear();
  const size_t index = steps.size();
  steps.push_back(t);
  const int nl = dim + 1;
  const int cell_type = dim == 2 ? 5 : 10;  // VTK_TRIANGLE / VTK_TETRA

  for (size_t c = 0; c < comp_names.size(); ++c) {
    if (ns[c] == 0 || comp_vertices[c].empty()) continue;
    const std::string name = stem + "-" + comp_names[c];
    char num[16];
    std::snprintf(num, sizeof num, "%05zu", index);
    const std::string file = name + "-" + num + ".vtu";
    std::ofstream o(dir + "/" + file);
    if (!o) throw ConfigError("cannot write '" + dir + "/" + file + "'");
    o << std::setprecision(17);
    const auto& verts = comp_vertices[c];
    std::vector<int64_t> cells;
    for (int64_t e = 0; e < mesh.ne; ++e)
      if (elem_comp[e] == static_cast<int>(c)) cells.push_back(e);
    o << "<?xml version=\"1.0\"?>\n"
      << "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n"
      << "<UnstructuredGrid>\n"
      << "<Piece NumberOfPoints=\"" << verts.size() << "\" NumberOfCells=\"" << cells.size() << "\">\n"
      << "<PointData Scalars=\"" << species[0].name << "\">\n";
    int64_t off = 0;
    for (size_t k = 0; k < c; ++k) off += static_cast<int64_t>(comp_vertices[k].size()) * ns[k];
    for (const auto& sp : species) {
      if (sp.comp != static_cast<int>(c)) continue;
      o << "<DataArray type=\"Float64\" Name=\"" << sp.name << "\" NumberOfComponents=\"1\" format=\"ascii\">\n";
      for (size_t k = 0; k < verts.size(); ++k) o << x_ref[off + static_cast<int64_t>(k) * ns[c] + sp.local] << "\n";
      o << "</DataArray>\n";
    }
    o << "</PointData>\n<Points>\n"
      << "<DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">\n";
    for (int32_t v : verts) {
      for (int d = 0; d < 3; ++d) o << (d < dim ? mesh.coords[static_cast<int64_t>(v) * dim + d] : 0.0) << (d < 2 ? " " : "\n");
    }
    o << "</DataArray>\n</Points>\n<Cells>\n"
      << "<DataArray type=\"Int64\" Name=\"connectivity\" format=\"ascii\">\n";
    const int64_t base = comp_node_offset[c];
    for (int64_t e : cells) {
      for (int a = 0; a < nl; ++a)
        o << (comp_vnode[c][mesh.cells[e * nl + a]] - base) << (a + 1 < nl ? " " : "\n");
    }
    o << "</DataArray>\n<DataArray type=\"Int64\" Name=\"offsets\" format=\"ascii\">\n";
    for (size_t k = 0; k < cells.size(); ++k) o << (static_cast<int64_t>(k) + 1) * nl << "\n";
    o << "</DataArray>\n<DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">\n";
    for (size_t k = 0; k < cells.size(); ++k) o << cell_type << "\n";
    o << "</DataArray>\n</Cells>\n</Piece>\n</UnstructuredGrid>\n</VTKFile>\n";
    if (!o) throw ConfigError("error while writing '" + dir + "/" + file + "'");

    std::ofstream pvd(dir + "/" + name + ".pvd");
    pvd << std::setprecision(17)
        << "<?xml version=\"1.0\"?>\n<VTKFile type=\"Collection\" version=\"0.1\" byte_order=\"LittleEndian\">\n"
        << "<Collection>\n";
    for (size_t k = 0; k < steps.size(); ++k) {
      std::snprintf(num, sizeof num, "%05zu", k);
      pvd << "<DataSet timestep=\"" << steps[k] << "\" group=\"\" part=\"0\" file=\"" << name << "-" << num
          << ".vtu\"/>\n";
    }
    pvd << "</Collection>\n</VTKFile>\n";
    if (!pvd) throw ConfigError("error while writing '" + dir + "/" + name + ".pvd'");
  }
}

}  // namespace dcgpu
