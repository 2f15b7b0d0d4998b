#include "model.hpp"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <map>
#include <numeric>
#include <set>

#include "assemble.cuh"

namespace dcgpu {

int64_t& device_bytes_this_thread() {
  static thread_local int64_t bytes = 0;
  return bytes;
}

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

DevProgram ProgramBundle::view() const {
  DevProgram p;
  p.code = code.get();
  p.consts = consts.get();
  p.consts32 = consts32.get();
  p.inputs = inputs.get();
  p.outputs = outputs.get();
  p.ncode = static_cast<int>(host.code.size());
  p.ninputs = static_cast<int>(host.inputs.size());
  p.noutputs = static_cast<int>(host.outputs.size());
  p.nregs = host.nregs;
  return p;
}

void ProgramBundle::upload() {
  if (host.nregs > kMaxDevRegisters) throw ConfigError("expression program needs too many registers");
  code.upload(host.code);
  consts.upload(host.consts);
  consts32.upload(std::vector<float>(host.consts.begin(), host.consts.end()));
  inputs.upload(host.inputs);
  outputs.upload(host.outputs);
}

namespace {

const char* kAxes[3] = {"x", "y", "z"};

std::optional<std::string> expr_of(const Ini& sub) {
  std::string t = trim(sub.get("expression", ""));
  if (is_zero_expression(t)) return std::nullopt;
  return t;
}

struct ScalarFn {
  std::string value;
  std::vector<std::pair<std::string, std::string>> jac;  // (species, expression)
};
struct TensorFn {
  bool tensor = false;
  std::vector<std::string> entries;  // 1 (scalar) or dim*dim ("" absent)
};

std::optional<ScalarFn> scalar_fn(const Ini& c, const std::vector<SpeciesInfo>& all) {
  auto v = expr_of(c);
  if (!v) return std::nullopt;
  ScalarFn f;
  f.value = *v;
  Ini jc = c.sub("jacobian");
  for (const auto& s : all)
    if (jc.has_sub(s.name))
      if (auto j = expr_of(jc.sub(s.name))) f.jac.emplace_back(s.name, *j);
  return f;
}

std::optional<std::vector<std::string>> vector_fn(const Ini& c, int dim) {
  std::vector<std::string> comps(dim);
  bool active = false;
  for (int d = 0; d < dim; ++d) {
    if (auto e = expr_of(c.sub(kAxes[d]))) { comps[d] = *e; active = true; }
  }
  if (!active) return std::nullopt;
  return comps;
}

std::optional<TensorFn> tensor_fn(const Ini& c, int dim) {
  std::string type = c.get("type", "scalar");
  TensorFn t;
  if (type == "scalar") {
    auto e = expr_of(c);
    if (!e) return std::nullopt;
    t.entries = {*e};
    return t;
  }
  if (type == "tensor") {
    t.tensor = true;
    t.entries.assign(dim * dim, "");
    bool active = false;
    for (int i = 0; i < dim; ++i)
      for (int j = 0; j < dim; ++j) {
        std::string key = std::string(kAxes[i]) + kAxes[j];
        if (c.has_sub(key))
          if (auto e = expr_of(c.sub(key))) { t.entries[i * dim + j] = *e; active = true; }
      }
    if (!active) return std::nullopt;
    return t;
  }
  throw ConfigError("not known type 'scalar_field diffusion type = " + type + "'");
}

}  // namespace

Model::Model(const std::string& ini_text, const std::string& overrides) {
  cfg = Ini::parse(ini_text);
  if (!overrides.empty()) cfg.apply_overrides(overrides);
  if (cfg.has_sub("parser_context")) ctx = ParserContext(cfg.sub("parser_context"));
  mesh = make_mesh_from_config(cfg.sub("grid"));
  dim = mesh.dim;
  build_species();
  build_nodes();
  build_pattern();
  upload_geometry();
  build_volume_groups();
  build_face_groups();
  if (numerical_jacobian)
    for (const auto& g : fgroups)
      for (int side = 0; side < 2; ++side)
        for (uint16_t id : g.prog[side].host.inputs)
          if (id >= IN_GRAD && id < IN_POSITION)
            throw ConfigError("model.jacobian.type = numerical: outflow expressions that read a gradient are not "
                              "supported");
  build_static_matrices();
  build_constraints();
  setup_volume_jit();
  for (const auto& g : vgroups) {
    dynamic_mass = dynamic_mass || g.has_mass;
    for (const Program* pr : {&g.prog_res.host, &g.prog_all.host})
      for (uint16_t id : pr->inputs) dynamic_time = dynamic_time || id == IN_TIME;
  }
  for (const auto& f : fgroups)
    for (int side = 0; side < 2; ++side)
      for (uint16_t id : f.prog[side].host.inputs) dynamic_time = dynamic_time || id == IN_TIME;
}

// model.assembly.jit = auto | true | false: the compartments' volume kernels compiled at
// set-up for their own programs (volume_jit.hpp); auto compiles them for compartments of at
// least kJitAutoCells cells, where the compilation (about a second) is small against the
// assembly time it saves.  Without NVRTC, or when a compilation fails, the interpreter
// kernels stay in use (jit_status says why); `true` makes that a configuration error.
void Model::setup_volume_jit() {
  constexpr int64_t kJitAutoCells = int64_t{1} << 18;
  const std::string mode = cfg.get("model.assembly.jit", "auto");
  if (mode != "auto" && mode != "true" && mode != "false")
    throw ConfigError("model.assembly.jit must be auto, true or false");
  jit_status = "off";
  if (mode == "false" || numerical_jacobian) return;
  for (auto& g : vgroups) {
    if (mode == "auto" && g.ne < kJitAutoCells) continue;
    JitVolumeInput in;
    in.dim = dim;
    in.ns = g.ns;
    in.species_offset = species_offset[g.comp];
    in.n_slots = g.slots_dyn;
    in.all_mass = g.dyn_all_mass;
    in.prog_res = &g.prog_res.host;
    in.prog_all = &g.prog_all.host;
    in.res_terms_r = &g.res_terms_r;
    in.res_terms_a = &g.res_terms_a;
    in.jac_terms = &g.jac_terms;
    std::string why;
    g.jit = build_volume_jit(in, &why);
    if (!g.jit) {
      if (mode == "true") throw ConfigError("model.assembly.jit = true: " + why);
      jit_status = "interpreter (" + why + ")";
      for (auto& h : vgroups) h.jit.reset();
      return;
    }
    jit_status = "compiled";
  }
}

// uniform skip flags of the volume kernel for one program and its term lists, and the
// number of per-element Jacobian coefficients of the terms (k_volume's shared-memory size:
// NQ point weights + one for mass-type terms, 1 for scalar diffusion, dim^2 for tensor
// diffusion, (dim + 1) dim for the vector terms)
void set_volume_flags(VolumeParams& p, const Program& prog, const std::vector<Term>& res, const std::vector<Term>& jac,
                      int dim) {
  const int nq = dim == 2 ? 3 : 4;
  p.ncoef = 0;
  for (const Term& T : jac) {
    const int sz = (T.kind == J_MASS || T.kind == J_MASS_U || T.kind == J_STORAGE_SELF) ? nq + 1
                   : T.kind == J_DIFF_SCALAR                                             ? 1
                   : T.kind == J_DIFF_TENSOR                                             ? dim * dim
                                                                                         : (dim + 1) * dim;
    p.ncoef = std::max(p.ncoef, static_cast<int>(T.coef) + sz);
  }
  p.need_pos = p.need_grad = p.has_flux = p.need_vol = 0;
  for (uint16_t id : prog.inputs) {
    if (id == IN_ENTITY_VOLUME) p.need_vol = 1;
    if (id >= IN_POSITION && id < IN_NORMAL) p.need_pos = 1;
    if (id >= IN_GRAD && id < IN_POSITION) p.need_grad = 1;
  }
  for (const Term& T : res) {
    if (T.kind == R_VELOCITY || T.kind == R_DIFF_SCALAR || T.kind == R_DIFF_TENSOR) p.has_flux = 1;
    if (T.kind == R_DIFF_SCALAR || T.kind == R_DIFF_TENSOR) p.need_grad = 1;
  }
  for (const Term& T : jac)
    if (T.kind == J_DIFFJAC_SCALAR || T.kind == J_DIFFJAC_TENSOR) p.need_grad = 1;
}

void Model::build_static_matrices() {
  const int64_t nvals = nnzb() * bs * bs;
  for (const auto& g : vgroups) {
    has_Ms |= g.static_mass;
    has_Ks |= g.static_stiffness;
  }
  if (has_Ms) {
    d_Ms.resize(nvals);
    cuda_check(cudaMemset(d_Ms.get(), 0, nvals * sizeof(double)), "memset");
  }
  if (has_Ks) {
    d_Ks.resize(nvals);
    cuda_check(cudaMemset(d_Ks.get(), 0, nvals * sizeof(double)), "memset");
  }
  if (has_Ms || has_Ks) d_Cs.resize(nvals);
  for (const auto& g : vgroups) {
    if (g.static_terms.empty()) continue;
    VolumeParams p{};
    p.coords = d_coords.get();
    p.verts = g.verts.get();
    p.nodes = g.nodes.get();
    p.bpos = g.bpos.get();
    p.prog = g.prog_static.view();
    p.res_terms = nullptr;
    p.n_res_terms = 0;
    p.jac_terms = g.d_static.get();
    p.n_jac_terms = static_cast<int>(g.static_terms.size());
    p.tables = tables;
    p.x = nullptr;
    p.r = nullptr;
    p.bs = bs;
    p.species_offset = species_offset[g.comp];
    p.t = 0.0;
    p.er = d_er.get();
    p.ej = d_ej.get();
    p.n_slots = g.slots_static;
    p.all_mass = g.static_all_mass ? 1 : 0;
    set_volume_flags(p, g.prog_static.host, {}, g.static_terms, dim);
    for (int form = 0; form < 2; ++form) {
      if ((form == 0 && !g.static_mass) || (form == 1 && !g.static_stiffness)) continue;
      double* target = form == 0 ? d_Ms.get() : d_Ks.get();
      p.J = target;
      p.cm = form == 0 ? 1.0 : 0.0;
      p.ca = form == 0 ? 0.0 : 1.0;
      launch_volume(dim, g.ns, p, 0, static_cast<int>(g.ne), 2, nullptr);
      launch_gather_jacobian(target, bs, g.slots_static, g.slot_pos_static.get(), g.block_begin, g.nblocks,
                             g.blist_ptr.get(), g.blist.get(), d_ej.get(), false, nullptr);
    }
  }
  // Every set-up copy, memset and kernel of the model went to the legacy default stream,
  // which does not order against the non-blocking streams the solvers run on (and a
  // pageable cudaMemcpy may return before its DMA lands): wait for all of it here.
  cuda_check(cudaStreamSynchronize(cudaStreamLegacy), "model set-up");
}

void Model::build_species() {
  Ini comps = cfg.sub("compartments");
  comp_names = comps.sub_keys();
  if (comp_names.empty()) throw ConfigError("no compartments defined ('[compartments]')");
  if (comp_names.size() > 64) throw ConfigError("at most 64 compartments are supported");
  // mark cells by their centre (make_multi_domain_grid.hh:118-154)
  const int nl = dim + 1;
  std::vector<std::vector<char>> mask(comp_names.size(), std::vector<char>(mesh.ne, 0));
  for (size_t c = 0; c < comp_names.size(); ++c) {
    Ini sub = comps.sub(comp_names[c]);
    std::string type = sub.get("type", "expression");
    if (type != "expression") throw ConfigError("Not know type '" + type + "' of compartment");
    ProgramBuilder pb(ctx);
    // cell-data keys (Gmsh "gmsh_id") are variables, given as inputs after the position
    std::vector<const std::vector<double>*> cdata;
    Resolver res = [&](const std::string& nm) -> std::optional<Symbol> {
      for (int d = 0; d < 3; ++d)
        if (nm == std::string("position_") + kAxes[d]) {
          Symbol s;
          if (d < dim) { s.is_input = true; s.input = static_cast<uint16_t>(IN_POSITION + d); }
          return s;
        }
      auto it = mesh.cell_data.find(nm);
      if (it != mesh.cell_data.end()) {
        Symbol s;
        s.is_input = true;
        size_t k = std::find(cdata.begin(), cdata.end(), &it->second) - cdata.begin();
        if (k == cdata.size()) cdata.push_back(&it->second);
        s.input = static_cast<uint16_t>(IN_SPECIES + k);
        return s;
      }
      return std::nullopt;
    };
    pb.add_output(pb.compile_text(sub.at("expression"), res));
    Program p = pb.finish();
    std::vector<double> in(p.inputs.size());
    for (int64_t e = 0; e < mesh.ne; ++e) {
      double ctr[3] = {0, 0, 0};
      for (int a = 0; a < nl; ++a)
        for (int d = 0; d < dim; ++d) ctr[d] += mesh.coords[mesh.cells[e * nl + a] * dim + d];
      for (int d = 0; d < dim; ++d) ctr[d] /= nl;
      for (size_t i = 0; i < p.inputs.size(); ++i)
        in[i] = p.inputs[i] >= IN_POSITION ? ctr[p.inputs[i] - IN_POSITION] : (*cdata[p.inputs[i] - IN_SPECIES])[e];
      mask[c][e] = run_program_host(p, ctx, in.data()) != 0.0;
    }
  }
  elem_comp.assign(mesh.ne, -1);
  for (int64_t e = 0; e < mesh.ne; ++e) {
    for (size_t c = 0; c < comp_names.size(); ++c) {
      if (!mask[c][e]) continue;
      if (elem_comp[e] >= 0)
        throw ConfigError("overlapping compartments ('" + comp_names[elem_comp[e]] + "' and '" + comp_names[c] +
                          "') are not supported by the GPU engine");
      elem_comp[e] = static_cast<int32_t>(c);
    }
  }
  // species per compartment in configuration order
  Ini sf = cfg.sub("model").sub("scalar_field");
  std::vector<std::vector<std::string>> per(comp_names.size());
  std::set<std::string> seen;
  for (const auto& name : sf.sub_keys()) {
    std::string cn = sf.sub(name).get("compartment", "");
    if (cn.empty()) continue;
    auto it = std::find(comp_names.begin(), comp_names.end(), cn);
    if (it == comp_names.end()) throw ConfigError("scalar field '" + name + "' refers to unknown compartment '" + cn + "'");
    if (!seen.insert(name).second) throw ConfigError("Variable with name '" + name + "' is repeated");
    per[it - comp_names.begin()].push_back(name);
  }
  ns.assign(comp_names.size(), 0);
  species_offset.assign(comp_names.size(), 0);
  int g = 0;
  for (size_t c = 0; c < comp_names.size(); ++c) {
    species_offset[c] = g;
    ns[c] = static_cast<int>(per[c].size());
    if (ns[c] > 8) throw ConfigError("at most 8 species per compartment are supported");
    for (int k = 0; k < ns[c]; ++k) species.push_back({per[c][k], static_cast<int>(c), k, g++});
  }
  if (species.empty())
    throw ConfigError("Basis has dimension 0, make sure to have at least one 'scalar_field' with a non-empty 'compartment'");
  bs = *std::max_element(ns.begin(), ns.end());
  Ini mcfg = cfg.sub("model");
  is_linear = mcfg.get_bool("is_linear", false);
  std::string jt = mcfg.get("jacobian.type", "analytical");
  if (jt != "analytical" && jt != "numerical")
    throw ConfigError("The option 'model.jacobian.type' must be either 'analytical' or 'numerical'");
  numerical_jacobian = (jt == "numerical") && !is_linear;
  fd_eps = mcfg.get_double("jacobian.epsilon", 1e-7);
  if (cfg.has_sub("model.domain.deformation") || mcfg.has_sub("domain"))
    if (mcfg.sub("domain").has_sub("deformation"))
      throw ConfigError("model.domain.deformation is not supported by the GPU engine");
  if (mcfg.get_long("order", 1) != 1) throw ConfigError("only model.order = 1 (P1) is supported");
}

void Model::build_nodes() {
  const int nl = dim + 1;
  const size_t nc = comp_names.size();
  comp_vertices.assign(nc, {});
  comp_vnode.assign(nc, std::vector<int32_t>(mesh.nv, -1));
  comp_node_offset.assign(nc + 1, 0);
  std::vector<std::vector<char>> used(nc, std::vector<char>(mesh.nv, 0));
  for (int64_t e = 0; e < mesh.ne; ++e) {
    int c = elem_comp[e];
    if (c < 0 || ns[c] == 0) continue;
    for (int a = 0; a < nl; ++a) used[c][mesh.cells[e * nl + a]] = 1;
  }
  int64_t off = 0;
  ndof = 0;
  for (size_t c = 0; c < nc; ++c) {
    comp_node_offset[c] = off;
    for (int64_t v = 0; v < mesh.nv; ++v)
      if (used[c][v]) {
        comp_vnode[c][v] = static_cast<int32_t>(off + comp_vertices[c].size());
        comp_vertices[c].push_back(static_cast<int32_t>(v));
      }
    off += static_cast<int64_t>(comp_vertices[c].size());
    ndof += static_cast<int64_t>(comp_vertices[c].size()) * ns[c];
  }
  comp_node_offset[nc] = off;
  nnodes = off;
  if (nnodes * bs > INT32_MAX) throw ConfigError("problem too large for 32-bit row indices");
  row_ns.assign(nnodes, 0);
  for (size_t c = 0; c < nc; ++c)
    for (int64_t k = comp_node_offset[c]; k < comp_node_offset[c + 1]; ++k) row_ns[k] = static_cast<int8_t>(ns[c]);
  padded = false;
  for (size_t c = 0; c < nc; ++c)
    if (!comp_vertices[c].empty() && ns[c] != bs) padded = true;
}

int64_t Model::ref_dof(int comp, int32_t vloc, int local) const {
  int64_t off = 0;
  for (int c = 0; c < comp; ++c) off += static_cast<int64_t>(comp_vertices[c].size()) * ns[c];
  return off + static_cast<int64_t>(vloc) * ns[comp] + local;
}

void Model::to_blocked(const std::vector<double>& ref, std::vector<double>& blk) const {
  blk.assign(nnodes * bs, 0.0);
  int64_t off = 0;
  for (size_t c = 0; c < comp_names.size(); ++c) {
    const int64_t nvc = static_cast<int64_t>(comp_vertices[c].size());
    for (int64_t k = 0; k < nvc; ++k)
      for (int s = 0; s < ns[c]; ++s) blk[(comp_node_offset[c] + k) * bs + s] = ref[off + k * ns[c] + s];
    off += nvc * ns[c];
  }
}

void Model::from_blocked(const std::vector<double>& blk, std::vector<double>& ref) const {
  ref.assign(ndof, 0.0);
  int64_t off = 0;
  for (size_t c = 0; c < comp_names.size(); ++c) {
    const int64_t nvc = static_cast<int64_t>(comp_vertices[c].size());
    for (int64_t k = 0; k < nvc; ++k)
      for (int s = 0; s < ns[c]; ++s) ref[off + k * ns[c] + s] = blk[(comp_node_offset[c] + k) * bs + s];
    off += nvc * ns[c];
  }
}

std::vector<double> Model::initial_state() const {
  // make_initial.hh:24-90 + interpolate.hh:21-78: nodal values of initial.expression
  std::vector<double> x(ndof, 0.0);
  Ini mcfg = cfg.sub("model");
  Ini sf = mcfg.sub("scalar_field");
  const double t0 = mcfg.get_double("time_step_operator.time_begin", 0.0);
  for (const auto& sp : species) {
    Ini c = sf.sub(sp.name);
    if (!c.has_sub("initial")) continue;
    auto txt = expr_of(c.sub("initial"));
    if (!txt) continue;
    ProgramBuilder pb(ctx);
    Resolver res = [&](const std::string& nm) -> std::optional<Symbol> {
      Symbol s;
      for (int d = 0; d < 3; ++d)
        if (nm == std::string("position_") + kAxes[d]) {
          if (d < dim) { s.is_input = true; s.input = static_cast<uint16_t>(IN_POSITION + d); }
          return s;
        }
      if (nm == "time") { s.value = t0; return s; }
      if (nm == "integration_factor" || nm == "entity_volume" || nm == "in_volume" || nm == "in_boundary" ||
          nm == "in_skeleton")
        return s;
      if (nm == "no_value") { s.value = DBL_MAX; return s; }
      return std::nullopt;
    };
    pb.add_output(pb.compile_text(*txt, res));
    Program p = pb.finish();
    std::vector<double> in(p.inputs.size());
    const auto& verts = comp_vertices[sp.comp];
    for (size_t k = 0; k < verts.size(); ++k) {
      for (size_t i = 0; i < p.inputs.size(); ++i) in[i] = mesh.coords[verts[k] * dim + (p.inputs[i] - IN_POSITION)];
      x[ref_dof(sp.comp, static_cast<int32_t>(k), sp.local)] = run_program_host(p, ctx, in.data());
    }
  }
  return x;
}

// ------------------------------------------------------------------ pattern

void Model::build_pattern() {
  const int nl = dim + 1;
  // element couplings
  std::vector<int64_t> cnt(nnodes + 1, 0);
  for (int64_t e = 0; e < mesh.ne; ++e) {
    int c = elem_comp[e];
    if (c < 0 || ns[c] == 0) continue;
    for (int a = 0; a < nl; ++a) cnt[comp_vnode[c][mesh.cells[e * nl + a]]] += nl;
  }
  // interface couplings: faces between two compartments with species on both sides, or
  // with any outflow configured (computed conservatively here; the face groups use a
  // subset of these blocks)
  std::vector<std::pair<int32_t, int32_t>> extra;
  Ini sf = cfg.sub("model").sub("scalar_field");
  bool any_outflow = false;
  for (const auto& sp : species)
    if (sf.sub(sp.name).has_sub("outflow")) any_outflow = true;
  if (any_outflow && comp_names.size() > 1) {
    Faces F = compute_faces(mesh);
    for (int64_t f = 0; f < F.nf; ++f) {
      if (F.e1[f] < 0) continue;
      int ci = elem_comp[F.e0[f]], co = elem_comp[F.e1[f]];
      if (ci == co || ci < 0 || co < 0 || ns[ci] == 0 || ns[co] == 0) continue;
      for (int k = 0; k < dim; ++k)
        for (int l = 0; l < dim; ++l) {
          int32_t vk = F.verts[f * dim + k], vl = F.verts[f * dim + l];
          int32_t a = comp_vnode[ci][vk], b = comp_vnode[co][vl];
          int32_t a2 = comp_vnode[co][vk], b2 = comp_vnode[ci][vl];
          extra.emplace_back(a, b);
          extra.emplace_back(a2, b2);
        }
    }
    for (const auto& pr : extra) cnt[pr.first] += 1;
  }
  std::vector<int64_t> start(nnodes + 1, 0);
  for (int64_t i = 0; i < nnodes; ++i) start[i + 1] = start[i] + cnt[i];
  std::vector<int32_t> buf(start[nnodes]);
  std::vector<int64_t> fillp(start.begin(), start.end() - 1);
  for (int64_t e = 0; e < mesh.ne; ++e) {
    int c = elem_comp[e];
    if (c < 0 || ns[c] == 0) continue;
    for (int a = 0; a < nl; ++a) {
      int32_t ra = comp_vnode[c][mesh.cells[e * nl + a]];
      for (int b = 0; b < nl; ++b) buf[fillp[ra]++] = comp_vnode[c][mesh.cells[e * nl + b]];
    }
  }
  for (const auto& pr : extra) buf[fillp[pr.first]++] = pr.second;
  rowptr.assign(nnodes + 1, 0);
  colidx.clear();
  colidx.reserve(static_cast<size_t>(nnodes) * (dim == 2 ? 7 : 15));
  diag.assign(nnodes, -1);
  for (int64_t i = 0; i < nnodes; ++i) {
    auto b = buf.begin() + start[i], e = buf.begin() + start[i + 1];
    std::sort(b, e);
    auto u = std::unique(b, e);
    for (auto it = b; it != u; ++it) {
      if (*it == i) diag[i] = static_cast<int32_t>(colidx.size());
      colidx.push_back(*it);
    }
    rowptr[i + 1] = static_cast<int32_t>(colidx.size());
    if (colidx.size() > static_cast<size_t>(INT32_MAX)) throw ConfigError("pattern too large");
  }
  for (int64_t i = 0; i < nnodes; ++i)
    if (diag[i] < 0) throw ConfigError("internal: missing diagonal block");
  d_rowptr.upload(rowptr);
  d_colidx.upload(colidx);
  d_diag.upload(diag);

  // SELL-32 slices of the same pattern: slot offsets and block columns (padding slots point
  // at the lane's own row, or at row 0 past the last row)
  const int64_t nsl = (nnodes + 31) / 32;
  std::vector<int64_t> soff(nsl + 1, 0);
  for (int64_t sl = 0; sl < nsl; ++sl) {
    int w = 0;
    for (int64_t br = sl * 32; br < std::min<int64_t>(nnodes, sl * 32 + 32); ++br)
      w = std::max(w, rowptr[br + 1] - rowptr[br]);
    soff[sl + 1] = soff[sl] + w;
  }
  std::vector<int32_t> scols(static_cast<size_t>(soff[nsl]) * 32);
  for (int64_t sl = 0; sl < nsl; ++sl) {
    const int w = static_cast<int>(soff[sl + 1] - soff[sl]);
    for (int lane = 0; lane < 32; ++lane) {
      const int64_t br = sl * 32 + lane;
      const int len = br < nnodes ? rowptr[br + 1] - rowptr[br] : 0;
      for (int k = 0; k < w; ++k)
        scols[(soff[sl] + k) * 32 + lane] =
            k < len ? colidx[rowptr[br] + k] : static_cast<int32_t>(br < nnodes ? br : 0);
    }
  }
  std::vector<int64_t> sbpos(colidx.size());
  for (int64_t br = 0; br < nnodes; ++br)
    for (int k = 0; k < rowptr[br + 1] - rowptr[br]; ++k)
      sbpos[rowptr[br] + k] = (soff[br / 32] + k) * 32 + (br % 32);
  sell_slots = soff[nsl];
  d_sell_off.upload(soff);
  d_sell_cols.upload(scols);
  d_sell_bpos.upload(sbpos);
  d_row_ns.upload(row_ns);
  // reference DOF -> blocked index (the layout map of to_blocked / from_blocked, on the device)
  {
    std::vector<int64_t> r2b;
    r2b.reserve(ndof);
    for (size_t c = 0; c < comp_names.size(); ++c)
      for (int64_t k = 0; k < static_cast<int64_t>(comp_vertices[c].size()); ++k)
        for (int s = 0; s < ns[c]; ++s) r2b.push_back((comp_node_offset[c] + k) * bs + s);
    d_ref2blk.upload(r2b);
  }
}

static int32_t find_block(const std::vector<int32_t>& rowptr, const std::vector<int32_t>& colidx, int32_t r,
                          int32_t c) {
  auto b = colidx.begin() + rowptr[r], e = colidx.begin() + rowptr[r + 1];
  auto it = std::lower_bound(b, e, c);
  if (it == e || *it != c) throw ConfigError("internal: block missing from the pattern");
  return static_cast<int32_t>(it - colidx.begin());
}

void Model::upload_geometry() {
  d_coords.upload(mesh.coords);
  d_cells.upload(mesh.cells);
  d_comp_vnode.clear();
  for (size_t c = 0; c < comp_names.size(); ++c) {
    d_comp_vnode.emplace_back();
    d_comp_vnode.back().upload(comp_vnode[c]);
  }
  std::vector<double> tx, ty;
  std::vector<int> off, len;
  for (const auto& t : ctx.interp) {
    off.push_back(static_cast<int>(tx.size()));
    len.push_back(static_cast<int>(t.x.size()));
    tx.insert(tx.end(), t.x.begin(), t.x.end());
    ty.insert(ty.end(), t.y.begin(), t.y.end());
  }
  d_tab_x.upload(tx);
  d_tab_y.upload(ty);
  d_tab_off.upload(off);
  d_tab_len.upload(len);
  tables.x = d_tab_x.get();
  tables.y = d_tab_y.get();
  tables.off = d_tab_off.get();
  tables.len = d_tab_len.get();
  // tabulated functions and images: descriptors + one packed value array each
  std::vector<FnTableDesc> fd;
  std::vector<double> fg;
  for (const auto& t : ctx.fn_table_data) {
    FnTableDesc d = t.desc;
    d.off = static_cast<int64_t>(fg.size());
    fd.push_back(d);
    fg.insert(fg.end(), t.g.begin(), t.g.end());
  }
  std::vector<ImageDesc> id;
  std::vector<double> ip;
  for (const auto& im : ctx.image_data) {
    ImageDesc d;
    d.off = static_cast<int64_t>(ip.size());
    d.rows = im.rows;
    d.cols = im.cols;
    d.x_res = im.x_res;
    d.y_res = im.y_res;
    d.x_off = im.x_off;
    d.y_off = im.y_off;
    id.push_back(d);
    ip.insert(ip.end(), im.px.begin(), im.px.end());
  }
  d_ftab_desc.upload(fd);
  d_ftab_val.upload(fg);
  d_img_desc.upload(id);
  d_img_px.upload(ip);
  tables.ft = d_ftab_desc.get();
  tables.ftg = d_ftab_val.get();
  tables.im = d_img_desc.get();
  tables.imp = d_img_px.get();
}

// greedy colouring: elements (or faces) sharing a vertex get different colours
static std::vector<int> greedy_colour(const std::vector<int32_t>& items_verts, int per_item, int64_t nv,
                                      int* ncolours) {
  const int64_t n = static_cast<int64_t>(items_verts.size()) / per_item;
  std::vector<uint64_t> vmask(nv, 0);
  std::vector<int> colour(n);
  int maxc = 0;
  for (int64_t i = 0; i < n; ++i) {
    uint64_t forb = 0;
    for (int a = 0; a < per_item; ++a) forb |= vmask[items_verts[i * per_item + a]];
    if (~forb == 0) throw ConfigError("colouring needs more than 64 colours");
    int c = __builtin_ctzll(~forb);
    colour[i] = c;
    maxc = std::max(maxc, c + 1);
    for (int a = 0; a < per_item; ++a) vmask[items_verts[i * per_item + a]] |= (uint64_t{1} << c);
  }
  *ncolours = maxc;
  return colour;
}

// ------------------------------------------------------------------ volume groups

void Model::build_volume_groups() {
  const int nl = dim + 1;
  const int nq = dim == 2 ? 3 : 4;
  Ini sf = cfg.sub("model").sub("scalar_field");
  vgroups.clear();
  for (size_t c = 0; c < comp_names.size(); ++c) {
    if (ns[c] == 0) continue;
    VolumeGroup g;
    g.comp = static_cast<int>(c);
    g.ns = ns[c];
    // elements of the compartment, coloured
    std::vector<int32_t> els;
    for (int64_t e = 0; e < mesh.ne; ++e)
      if (elem_comp[e] == static_cast<int>(c)) els.push_back(static_cast<int32_t>(e));
    g.ne = static_cast<int64_t>(els.size());
    if (g.ne == 0) continue;
    std::vector<int32_t> ev(els.size() * nl);
    for (size_t i = 0; i < els.size(); ++i)
      for (int a = 0; a < nl; ++a) ev[i * nl + a] = mesh.cells[static_cast<int64_t>(els[i]) * nl + a];
    int ncol = 0;
    auto col = greedy_colour(ev, nl, mesh.nv, &ncol);
    std::vector<int64_t> order(els.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return col[a] < col[b]; });
    g.color_offsets.assign(ncol + 1, 0);
    for (int64_t i : order) g.color_offsets[col[i] + 1]++;
    for (int k = 0; k < ncol; ++k) g.color_offsets[k + 1] += g.color_offsets[k];
    std::vector<int32_t> verts(els.size() * nl), nodes(els.size() * nl), bpos(els.size() * nl * nl);
    for (size_t j = 0; j < order.size(); ++j) {
      const int64_t i = order[j];
      for (int a = 0; a < nl; ++a) {
        verts[j * nl + a] = ev[i * nl + a];
        nodes[j * nl + a] = comp_vnode[c][ev[i * nl + a]];
      }
      for (int a = 0; a < nl; ++a)
        for (int b = 0; b < nl; ++b)
          bpos[(j * nl + a) * nl + b] = find_block(rowptr, colidx, nodes[j * nl + a], nodes[j * nl + b]);
    }
    g.verts.upload(verts);
    g.nodes.upload(nodes);
    g.bpos.upload(bpos);

    // gather lists of the two-phase assembly: for every node of the compartment its
    // (element, local vertex) pairs, for every block of the compartment's rows its
    // (element, local pair) triples, each in ascending element order
    if (g.ne * nl * nl > INT32_MAX) throw ConfigError("compartment too large for 32-bit gather lists");
    g.node_begin = comp_node_offset[c];
    g.nnodes = comp_node_offset[c + 1] - g.node_begin;
    g.block_begin = rowptr[g.node_begin];
    g.nblocks = rowptr[g.node_begin + g.nnodes] - g.block_begin;
    {
      std::vector<int64_t> rp(g.nnodes + 1, 0), bp(g.nblocks + 1, 0);
      for (int64_t j = 0; j < g.ne; ++j)
        for (int a = 0; a < nl; ++a) {
          rp[nodes[j * nl + a] - g.node_begin + 1]++;
          for (int b = 0; b < nl; ++b) bp[bpos[(j * nl + a) * nl + b] - g.block_begin + 1]++;
        }
      for (int64_t i = 0; i < g.nnodes; ++i) rp[i + 1] += rp[i];
      for (int64_t i = 0; i < g.nblocks; ++i) bp[i + 1] += bp[i];
      std::vector<int32_t> rl(g.ne * nl), bl(g.ne * nl * nl);
      std::vector<int64_t> rc(rp.begin(), rp.end() - 1), bc(bp.begin(), bp.end() - 1);
      for (int64_t j = 0; j < g.ne; ++j)
        for (int a = 0; a < nl; ++a) {
          rl[rc[nodes[j * nl + a] - g.node_begin]++] = static_cast<int32_t>(j * nl + a);
          for (int b = 0; b < nl; ++b)
            bl[bc[bpos[(j * nl + a) * nl + b] - g.block_begin]++] = static_cast<int32_t>((j * nl + a) * nl + b);
        }
      g.rlist_ptr.upload(rp);
      g.rlist.upload(rl);
      g.blist_ptr.upload(bp);
      g.blist.upload(bl);
    }

    // symbols of a volume program of compartment c
    Resolver res = [&](const std::string& nm) -> std::optional<Symbol> {
      Symbol s;
      for (const auto& sp : species) {
        if (nm == sp.name) {
          if (sp.comp == static_cast<int>(c)) { s.is_input = true; s.input = static_cast<uint16_t>(IN_SPECIES + sp.global); }
          return s;  // species of other compartments vanish on this element
        }
        for (int d = 0; d < 3; ++d)
          if (nm == "grad_" + sp.name + "_" + kAxes[d]) {
            if (sp.comp == static_cast<int>(c) && d < dim) {
              s.is_input = true;
              s.input = static_cast<uint16_t>(IN_GRAD + sp.global * 3 + d);
            }
            return s;
          }
      }
      for (int d = 0; d < 3; ++d)
        if (nm == std::string("position_") + kAxes[d]) {
          if (d < dim) { s.is_input = true; s.input = static_cast<uint16_t>(IN_POSITION + d); }
          return s;
        }
      if (nm == "time") { s.is_input = true; s.input = IN_TIME; return s; }
      if (nm == "entity_volume") { s.is_input = true; s.input = IN_ENTITY_VOLUME; return s; }
      if (nm == "in_volume") { s.value = 1.0; return s; }
      if (nm == "in_boundary" || nm == "in_skeleton" || nm == "integration_factor") return s;
      if (nm == "no_value") { s.value = DBL_MAX; return s; }
      return std::nullopt;
    };

    auto local_of = [&](const std::string& name) -> int {
      for (const auto& sp : species)
        if (sp.name == name) return sp.comp == static_cast<int>(c) ? sp.local : -1;
      return -1;
    };

    // A term is static when it is linear in the state with a coefficient that depends on
    // neither the state nor time (constant or position-only storage / scalar diffusion
    // without Jacobian entries).  Static terms are assembled once into the matrices Ms / Ks
    // (residual = matrix x state, exactly, since these terms are symmetric in test and trial);
    // the per-iteration kernels evaluate only the remaining, dynamic terms.
    auto is_static_text = [&](const std::string& text) {
      ProgramBuilder probe(ctx);
      int node = probe.compile_text(text, res);
      return !probe.depends_on(node, [](uint16_t id) { return id < IN_POSITION || id == IN_TIME; });
    };
    // three builders: static Jacobian program, dynamic residual-only, dynamic residual+Jacobian
    for (int pass = 0; pass < 3; ++pass) {
      const bool static_pass = pass == 0;
      const bool with_jac = pass != 1;
      ProgramBuilder pb(ctx);
      std::vector<Term> rterms, jterms;
      int coef = 0;
      auto out_of = [&](const std::string& text) { return pb.add_output(pb.compile_text(text, res)); };
      auto out_neg = [&](const std::string& text) {
        return pb.add_output(pb.unary(OP_NEG, pb.compile_text(text, res)));
      };
      auto outs_of = [&](const std::vector<std::string>& texts) {
        int first = -1;
        for (const auto& t : texts) {
          int o = pb.add_output(t.empty() ? pb.constant(0.0) : pb.compile_text(t, res));
          if (first < 0) first = o;
        }
        return first;
      };
      auto add_j = [&](uint8_t kind, int form, int test, int trial, int out) {
        Term T{};
        T.kind = kind;
        T.form = static_cast<uint8_t>(form);
        T.test = static_cast<uint8_t>(test);
        T.trial = static_cast<uint8_t>(trial);
        T.out = static_cast<uint16_t>(out);
        T.coef = static_cast<uint16_t>(coef);
        // mass-type terms: nq point weights + one slot for beta^2 (sum of the weights)
        int sz = (kind == J_MASS || kind == J_MASS_U || kind == J_STORAGE_SELF) ? nq + 1
               : (kind == J_DIFF_SCALAR) ? 1
               : (kind == J_DIFF_TENSOR) ? dim * dim : nl * dim;
        coef += sz;
        jterms.push_back(T);
      };
      auto add_r = [&](uint8_t kind, int form, int test, int trial, int out) {
        Term T{};
        T.kind = kind;
        T.form = static_cast<uint8_t>(form);
        T.test = static_cast<uint8_t>(test);
        T.trial = static_cast<uint8_t>(trial);
        T.out = static_cast<uint16_t>(out);
        rterms.push_back(T);
      };
      for (const auto& sp : species) {
        if (sp.comp != static_cast<int>(c)) continue;
        Ini scfg = sf.sub(sp.name);
        const int i = sp.local;
        // mass form: storage (local_equations.hh:340-353)
        if (scfg.has_sub("storage"))
          if (auto st = scalar_fn(scfg.sub("storage"), species)) {
            const bool stat = st->jac.empty() && is_static_text(st->value);
            if (static_pass) {
              if (stat) {
                g.static_mass = true;
                add_j(J_STORAGE_SELF, 0, i, i, out_of(st->value));
              }
            } else if (!stat) {
              g.has_mass = true;
              int o = out_of(st->value);
              add_r(R_STORAGE, 0, i, i, o);
              if (with_jac) {
                add_j(J_STORAGE_SELF, 0, i, i, o);
                for (const auto& [w, jt] : st->jac) {
                  int wl = local_of(w);
                  if (wl >= 0) add_j(J_MASS_U, 0, i, wl, out_of(jt));
                }
              }
            }
          }
        // stiffness form: reaction, velocity, diffusion (local_equations.hh:325-338)
        if (!static_pass && scfg.has_sub("reaction"))
          if (auto rf = scalar_fn(scfg.sub("reaction"), species)) {
            g.has_stiffness = true;
            add_r(R_REACTION, 1, i, i, out_of(rf->value));
            if (with_jac)
              for (const auto& [w, jt] : rf->jac) {
                int wl = local_of(w);
                if (wl >= 0) add_j(J_MASS, 1, i, wl, out_neg(jt));
              }
          }
        if (!static_pass && scfg.has_sub("velocity")) {
          Ini vc = scfg.sub("velocity");
          if (auto comps = vector_fn(vc, dim)) {
            g.has_stiffness = true;
            int o = outs_of(*comps);
            add_r(R_VELOCITY, 1, i, i, o);
            if (with_jac) {
              add_j(J_VELOCITY, 1, i, i, o);
              Ini jc = vc.sub("jacobian");
              for (const auto& sp2 : species)
                if (jc.has_sub(sp2.name))
                  if (auto jv = vector_fn(jc.sub(sp2.name), dim)) {
                    int wl = local_of(sp2.name);
                    if (wl >= 0) add_j(J_VELOCITY_JAC, 1, i, wl, outs_of(*jv));
                  }
            }
          }
        }
        if (scfg.has_sub("cross_diffusion")) {
          Ini cd = scfg.sub("cross_diffusion");
          for (const auto& sp2 : species) {
            if (!cd.has_sub(sp2.name)) continue;
            Ini dc = cd.sub(sp2.name);
            auto D = tensor_fn(dc, dim);
            if (!D) continue;
            const int wl = local_of(sp2.name);
            if (wl < 0) continue;  // gradient vanishes on this element
            std::vector<std::pair<int, TensorFn>> djac;
            Ini jc = dc.sub("jacobian");
            for (const auto& sp3 : species)
              if (jc.has_sub(sp3.name))
                if (auto JD = tensor_fn(jc.sub(sp3.name), dim)) {
                  int vl = local_of(sp3.name);
                  if (vl >= 0) djac.emplace_back(vl, *JD);
                }
            const bool stat = !D->tensor && djac.empty() && is_static_text(D->entries[0]);
            if (static_pass) {
              if (stat) {
                g.static_stiffness = true;
                add_j(J_DIFF_SCALAR, 1, i, wl, out_of(D->entries[0]));
              }
              continue;
            }
            if (stat) continue;
            g.has_stiffness = true;
            int o = outs_of(D->entries);
            add_r(D->tensor ? R_DIFF_TENSOR : R_DIFF_SCALAR, 1, i, wl, o);
            if (with_jac) {
              add_j(D->tensor ? J_DIFF_TENSOR : J_DIFF_SCALAR, 1, i, wl, o);
              for (const auto& [vl, JD] : djac)
                add_j(JD.tensor ? J_DIFFJAC_TENSOR : J_DIFFJAC_SCALAR, 1, i, vl, outs_of(JD.entries));
            }
          }
        }
      }
      if (coef > kMaxCoefficients) throw ConfigError("too many Jacobian terms in one compartment");
      // Jacobian slots: one per distinct (test, trial) pair, terms sorted by slot so the
      // volume kernel writes each slot of each local pair once
      auto assign_slots = [&](std::vector<Term>& terms, int& nslot, bool& all_mass, DeviceBuffer<int32_t>& pos,
                              std::vector<int32_t>* host_pos) {
        std::map<std::pair<int, int>, int> idx;
        std::vector<int32_t> p;
        all_mass = true;
        for (auto& T : terms) {
          const int te = T.test;
          const int tr = (T.kind == J_STORAGE_SELF || T.kind == J_VELOCITY) ? T.test : T.trial;
          auto it = idx.find({te, tr});
          if (it == idx.end()) {
            it = idx.emplace(std::make_pair(te, tr), static_cast<int>(p.size())).first;
            p.push_back(te * bs + tr);
          }
          T.slot = static_cast<uint8_t>(it->second);
          if (!(T.kind == J_MASS || T.kind == J_MASS_U || T.kind == J_STORAGE_SELF)) all_mass = false;
        }
        std::stable_sort(terms.begin(), terms.end(), [](const Term& a, const Term& b) { return a.slot < b.slot; });
        nslot = static_cast<int>(p.size());
        pos.upload(p);
        if (host_pos) *host_pos = p;
      };
      if (pass == 0) assign_slots(jterms, g.slots_static, g.static_all_mass, g.slot_pos_static, nullptr);
      if (pass == 2) assign_slots(jterms, g.slots_dyn, g.dyn_all_mass, g.slot_pos_dyn, &g.slot_pos_dyn_host);
      if (pass == 0) {
        g.prog_static.host = pb.finish();
        g.static_terms = jterms;
      } else if (pass == 1) {
        g.prog_res.host = pb.finish();
        g.res_terms_r = rterms;
      } else {
        g.prog_all.host = pb.finish();
        g.res_terms_a = rterms;
        g.jac_terms = jterms;
      }
    }
    g.prog_static.upload();
    g.prog_res.upload();
    g.prog_all.upload();
    g.d_static.upload(g.static_terms);
    g.d_res_r.upload(g.res_terms_r);
    g.d_res_a.upload(g.res_terms_a);
    g.d_jac.upload(g.jac_terms);
    vgroups.push_back(std::move(g));
  }
  int64_t er_max = 0, ej_max = 0;
  for (const auto& g : vgroups) {
    er_max = std::max<int64_t>(er_max, g.ne * nl * g.ns);
    ej_max = std::max<int64_t>(ej_max, g.ne * nl * nl * std::max(g.slots_dyn, g.slots_static));
  }
  d_er.resize(er_max);
  d_ej.resize(ej_max);
}

// ------------------------------------------------------------------ face groups

void Model::build_face_groups() {
  fgroups.clear();
  Ini sf = cfg.sub("model").sub("scalar_field");
  // outflow functions per species (local_equations.hh:677-697)
  std::vector<std::map<int, ScalarFn>> outflow(species.size());
  bool any = false;
  for (const auto& sp : species) {
    Ini sc = sf.sub(sp.name);
    if (!sc.has_sub("outflow")) continue;
    Ini oc = sc.sub("outflow");
    for (size_t k = 0; k < comp_names.size(); ++k)
      if (oc.has_sub(comp_names[k]))
        if (auto f = scalar_fn(oc.sub(comp_names[k]), species)) {
          outflow[sp.global][static_cast<int>(k)] = *f;
          any = true;
        }
  }
  if (!any) return;
  Faces F = compute_faces(mesh);
  const int nl = dim + 1;
  // group key: (c_in, c_out, boundary)
  std::map<std::tuple<int, int, int>, std::vector<int64_t>> groups;
  for (int64_t f = 0; f < F.nf; ++f) {
    const int ci = elem_comp[F.e0[f]];
    if (F.e1[f] < 0) {
      if (ci >= 0 && ns[ci] > 0) groups[{ci, -1, 1}].push_back(f);
      continue;
    }
    const int co = elem_comp[F.e1[f]];
    if (ci == co) continue;
    groups[{ci, co, 0}].push_back(f);
  }
  for (auto& [key, flist] : groups) {
    auto [ci, co, bnd] = key;
    FaceGroup g;
    g.comp[0] = ci;
    g.comp[1] = co;
    g.boundary = bnd != 0;
    bool has_terms = false;
    for (int side = 0; side < 2; ++side) {
      const int cs = g.comp[side], cother = g.comp[1 - side];
      if (cs < 0 || ns[cs] == 0) continue;
      if (side == 1 && g.boundary) continue;
      Resolver res = [&](const std::string& nm) -> std::optional<Symbol> {
        Symbol s;
        for (const auto& sp : species) {
          const bool here = sp.comp == cs || (cother >= 0 && sp.comp == cother);
          if (nm == sp.name) {
            if (here) { s.is_input = true; s.input = static_cast<uint16_t>(IN_SPECIES + sp.global); }
            return s;
          }
          for (int d = 0; d < 3; ++d)
            if (nm == "grad_" + sp.name + "_" + kAxes[d]) {
              if (here && d < dim) { s.is_input = true; s.input = static_cast<uint16_t>(IN_GRAD + sp.global * 3 + d); }
              return s;
            }
        }
        for (int d = 0; d < 3; ++d) {
          if (nm == std::string("position_") + kAxes[d]) {
            if (d < dim) { s.is_input = true; s.input = static_cast<uint16_t>(IN_POSITION + d); }
            return s;
          }
          if (nm == std::string("normal_") + kAxes[d]) {
            if (d < dim) { s.is_input = true; s.input = static_cast<uint16_t>(IN_NORMAL + d); }
            return s;
          }
        }
        if (nm == "time") { s.is_input = true; s.input = IN_TIME; return s; }
        if (nm == "entity_volume") { s.is_input = true; s.input = IN_ENTITY_VOLUME; return s; }
        if (nm == "in_boundary") { s.value = g.boundary ? 1.0 : 0.0; return s; }
        if (nm == "in_skeleton") { s.value = g.boundary ? 0.0 : 1.0; return s; }
        if (nm == "in_volume" || nm == "integration_factor") return s;
        if (nm == "no_value") { s.value = DBL_MAX; return s; }
        return std::nullopt;
      };
      ProgramBuilder pb(ctx);
      std::vector<Term> terms;
      int coef = 0;
      const int target = g.boundary ? cs : cother;
      if (target < 0) continue;
      for (const auto& sp : species) {
        if (sp.comp != cs) continue;
        auto it = outflow[sp.global].find(target);
        if (it == outflow[sp.global].end()) continue;
        // interior faces need a different compartment on the other side (local_operator.hh:836-853)
        if (!g.boundary && target == cs) continue;
        Term T{};
        T.kind = F_OUTFLOW;
        T.form = 1;
        T.test = static_cast<uint8_t>(sp.local);
        T.out = static_cast<uint16_t>(pb.add_output(pb.compile_text(it->second.value, res)));
        terms.push_back(T);
        for (const auto& [w, jt] : it->second.jac) {
          const SpeciesInfo* wsp = nullptr;
          for (const auto& s2 : species)
            if (s2.name == w) wsp = &s2;
          if (!wsp) continue;
          Term J{};
          J.kind = F_OUTFLOW_JAC;
          J.form = 1;
          J.test = static_cast<uint8_t>(sp.local);
          J.trial = static_cast<uint8_t>(wsp->local);
          if (wsp->comp == cs) J.side = 0;
          else if (!g.boundary && wsp->comp == cother) J.side = 1;
          else continue;
          J.out = static_cast<uint16_t>(pb.add_output(pb.compile_text(jt, res)));
          J.coef = static_cast<uint16_t>(coef);
          coef += dim == 2 ? 2 : 3;
          terms.push_back(J);
        }
      }
      if (coef > kMaxCoefficients) throw ConfigError("too many outflow Jacobian terms");
      if (terms.empty()) continue;
      has_terms = true;
      g.prog[side].host = pb.finish();
      g.prog[side].upload();
      g.terms[side] = terms;
      g.d_terms[side].upload(terms);
    }
    if (!has_terms) continue;
    // faces of the group, coloured by shared vertices
    std::vector<int32_t> fv(flist.size() * dim);
    for (size_t i = 0; i < flist.size(); ++i)
      for (int k = 0; k < dim; ++k) fv[i * dim + k] = F.verts[flist[i] * dim + k];
    int ncol = 0;
    auto col = greedy_colour(fv, dim, mesh.nv, &ncol);
    std::vector<int64_t> order(flist.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return col[a] < col[b]; });
    g.color_offsets.assign(ncol + 1, 0);
    for (int64_t i : order) g.color_offsets[col[i] + 1]++;
    for (int k = 0; k < ncol; ++k) g.color_offsets[k + 1] += g.color_offsets[k];
    g.nf = static_cast<int64_t>(flist.size());
    std::vector<int32_t> fverts(g.nf * dim), nin(g.nf * dim, -1), nout(g.nf * dim, -1), bpos(g.nf * 4 * dim * dim, -1);
    std::vector<int32_t> ein(g.nf), eout(g.nf);
    std::vector<double> normal(g.nf * dim), ielem(g.nf), fvol(g.nf);
    for (size_t j = 0; j < order.size(); ++j) {
      const int64_t f = flist[order[j]];
      ein[j] = F.e0[f];
      eout[j] = F.e1[f];
      double X[3][3] = {{0}};
      for (int k = 0; k < dim; ++k) {
        const int32_t v = F.verts[f * dim + k];
        fverts[j * dim + k] = v;
        if (ci >= 0) nin[j * dim + k] = comp_vnode[ci][v];
        if (co >= 0) nout[j * dim + k] = comp_vnode[co][v];
        for (int d = 0; d < dim; ++d) X[k][d] = mesh.coords[v * dim + d];
      }
      // opposite vertex of e0 for the orientation
      const int32_t vopp = mesh.cells[static_cast<int64_t>(F.e0[f]) * nl + F.l0[f]];
      double n[3] = {0, 0, 0}, meas;
      if (dim == 2) {
        const double tx = X[1][0] - X[0][0], ty = X[1][1] - X[0][1];
        meas = std::sqrt(tx * tx + ty * ty);
        n[0] = ty / meas;
        n[1] = -tx / meas;
        ielem[j] = meas;
        fvol[j] = meas;
      } else {
        const double a[3] = {X[1][0] - X[0][0], X[1][1] - X[0][1], X[1][2] - X[0][2]};
        const double b[3] = {X[2][0] - X[0][0], X[2][1] - X[0][1], X[2][2] - X[0][2]};
        n[0] = a[1] * b[2] - a[2] * b[1];
        n[1] = a[2] * b[0] - a[0] * b[2];
        n[2] = a[0] * b[1] - a[1] * b[0];
        meas = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int d = 0; d < 3; ++d) n[d] /= meas;
        ielem[j] = meas;
        fvol[j] = 0.5 * meas;
      }
      double dotp = 0.0;
      for (int d = 0; d < dim; ++d) dotp += n[d] * (X[0][d] - mesh.coords[vopp * dim + d]);
      if (dotp < 0)
        for (int d = 0; d < dim; ++d) n[d] = -n[d];
      for (int d = 0; d < dim; ++d) normal[j * dim + d] = n[d];
      for (int pr = 0; pr < 4; ++pr) {
        const int rs = pr / 2, cs2 = pr % 2;
        const std::vector<int32_t>& rn = rs == 0 ? nin : nout;
        const std::vector<int32_t>& cn = cs2 == 0 ? nin : nout;
        for (int k = 0; k < dim; ++k)
          for (int l = 0; l < dim; ++l) {
            const int32_t r = rn[j * dim + k], cc = cn[j * dim + l];
            if (r >= 0 && cc >= 0)
              bpos[((j * 4 + pr) * dim + k) * dim + l] = find_block(rowptr, colidx, r, cc);
          }
      }
    }
    g.fverts.upload(fverts);
    g.node_in.upload(nin);
    g.node_out.upload(nout);
    g.bpos.upload(bpos);
    g.elem_in.upload(ein);
    g.elem_out.upload(eout);
    g.normal.upload(normal);
    g.ielem.upload(ielem);
    g.fvolume.upload(fvol);
    fgroups.push_back(std::move(g));
  }
}

// ------------------------------------------------------------------ assembly driver

Bsr Model::bsr(double* val, float* val32) const {
  Bsr A;
  A.nrows = static_cast<int>(nnodes);
  A.bs = bs;
  A.nnzb = nnzb();
  A.rowptr = d_rowptr.get();
  A.colidx = d_colidx.get();
  A.val = val;
  A.val32 = val32;
  return A;
}

Sell Model::sell() const {
  Sell S;
  S.nrows = static_cast<int>(nnodes);
  S.bs = bs;
  S.nslices = (nnodes + 31) / 32;
  S.nslots = sell_slots;
  S.off = d_sell_off.get();
  S.cols = d_sell_cols.get();
  return S;
}

bool Model::assemble(const double* x, double t, double cm, double ca, double* r, double* J, int mode,
                     cudaStream_t s, float* jac_sell32) const {
  // static part: r += (cm Ms + ca Ks) x, J (+)= cm Ms + ca Ks
  const Bsr A0 = bsr(nullptr, nullptr);
  const int64_t nvals = nnzb() * bs * bs;
  const bool use_m = has_Ms && cm != 0.0, use_k = has_Ks && ca != 0.0;
  const double* C = nullptr;
  if ((use_m || use_k) && (mode & 2) && J) {
    if (!cs_valid || cs_cm != cm || cs_ca != ca) {
      if (d_Cs.size() != static_cast<size_t>(nvals)) d_Cs.resize(nvals);
      combine(nvals, cm, use_m ? d_Ms.get() : nullptr, ca, use_k ? d_Ks.get() : nullptr, d_Cs.get(), s);
      cs_cm = cm;
      cs_ca = ca;
      cs_valid = true;
    }
    C = d_Cs.get();
  } else if ((use_m || use_k) && cs_valid && cs_cm == cm && cs_ca == ca) {
    C = d_Cs.get();
  }
  // residual-only passes may take the static part alone or the state-dependent part alone
  const bool skip_static = (mode & kAssembleDynamicOnly) != 0, skip_dynamic = (mode & kAssembleStaticOnly) != 0;
  if ((skip_static || skip_dynamic) && (mode & 2))
    throw std::logic_error("assemble: static-only / dynamic-only passes are residual passes");
  if ((mode & 1) && r && !skip_static) {
    if (C) {
      spmv_acc(A0, C, x, r, 1.0, s);
    } else {
      if (use_m) spmv_acc(A0, d_Ms.get(), x, r, cm, s);
      if (use_k) spmv_acc(A0, d_Ks.get(), x, r, ca, s);
    }
  }
  // one compartment whose state-dependent gather covers every block of J: that gather takes
  // the static operator as its base (no copy of it into J first) and, with nothing added to J
  // after it, also writes the fp32 SELL-32 copy; when only some species pairs have dynamic
  // terms, a gather over every entry of every block (launch_gather_jacobian_full) does it
  const VolumeGroup* cover = nullptr;
  if ((mode & 2) && J && (mode & kAssembleOverwriteJacobian) && !numerical_jacobian && vgroups.size() == 1) {
    const VolumeGroup& g = vgroups[0];
    const bool active = (cm != 0.0 && g.has_mass) || (ca != 0.0 && g.has_stiffness);
    if (active && g.slots_dyn > 0 && g.block_begin == 0 && g.nblocks == nnzb()) cover = &g;
  }
  JacobianGatherOut gout;
  if (cover) {
    gout.overwrite = 1;
    gout.base = C;
    if (jac_sell32 && (fgroups.empty() || ca == 0.0) && !padded && n_constraints == 0) {
      gout.sell = jac_sell32;
      gout.sell_bpos = d_sell_bpos.get();
    }
  }
  if ((mode & 2) && J && !cover) {
    if (mode & kAssembleOverwriteJacobian) {
      if (C) cuda_check(cudaMemcpyAsync(J, C, nvals * sizeof(double), cudaMemcpyDeviceToDevice, s), "copy");
      else cuda_check(cudaMemsetAsync(J, 0, nvals * sizeof(double), s), "memset");
    } else if (C) {
      axpy(nvals, 1.0, C, J, s);
    }
  }
  const bool jac_f32 = (mode & kAssembleJacobianF32) != 0;
  mode &= 3;
  if (skip_dynamic) return false;
  for (const auto& g : vgroups) {
    if (!(cm != 0.0 && g.has_mass) && !(ca != 0.0 && g.has_stiffness)) continue;
    VolumeParams p{};
    p.coords = d_coords.get();
    p.verts = g.verts.get();
    p.nodes = g.nodes.get();
    p.bpos = g.bpos.get();
    const bool jac = (mode & 2) != 0;
    p.prog = jac ? g.prog_all.view() : g.prog_res.view();
    p.res_terms = jac ? g.d_res_a.get() : g.d_res_r.get();
    p.n_res_terms = static_cast<int>(jac ? g.res_terms_a.size() : g.res_terms_r.size());
    p.jac_terms = g.d_jac.get();
    p.n_jac_terms = static_cast<int>(g.jac_terms.size());
    p.tables = tables;
    p.x = x;
    p.r = r;
    p.J = J;
    p.bs = bs;
    p.species_offset = species_offset[g.comp];
    p.t = t;
    p.cm = cm;
    p.ca = ca;
    p.fd_eps = fd_eps;
    p.er = d_er.get();
    p.ej = d_ej.get();
    p.n_slots = g.slots_dyn;
    p.all_mass = g.dyn_all_mass ? 1 : 0;
    p.jac_f32 = jac_f32 ? 1 : 0;
    if (jac) set_volume_flags(p, g.prog_all.host, g.res_terms_a, g.jac_terms, dim);
    else set_volume_flags(p, g.prog_res.host, g.res_terms_r, {}, dim);
    const int ne = static_cast<int>(g.ne);
    if (numerical_jacobian && (mode & 2)) {
      // jacobian.type = numerical: residual pass (if asked) + finite-difference Jacobian pass
      // (coloured scatter), both with the residual program and terms
      p.prog = g.prog_res.view();
      p.res_terms = g.d_res_r.get();
      p.n_res_terms = static_cast<int>(g.res_terms_r.size());
      set_volume_flags(p, g.prog_res.host, g.res_terms_r, {}, dim);
      if ((mode & 1) && r) {
        launch_volume(dim, g.ns, p, 0, ne, 1, s);
        launch_gather_residual(r, bs, g.ns, g.node_begin, g.nnodes, g.rlist_ptr.get(), g.rlist.get(), d_er.get(), s);
      }
      if (J)
        for (size_t k = 0; k + 1 < g.color_offsets.size(); ++k)
          launch_volume(dim, g.ns, p, g.color_offsets[k], g.color_offsets[k + 1], kVolumeNumericalJacobian, s);
      continue;
    }
    // two-phase: element outputs for all cells of the compartment in one launch, then the
    // per-node / per-block gathers (fixed order, no atomics, no colouring)
    if (g.jit) launch_volume_jit(*g.jit, p, 0, ne, mode, s);
    else launch_volume(dim, g.ns, p, 0, ne, mode, s);
    if ((mode & 1) && r)
      launch_gather_residual(r, bs, g.ns, g.node_begin, g.nnodes, g.rlist_ptr.get(), g.rlist.get(), d_er.get(), s);
    if ((mode & 2) && J && g.slots_dyn > 0) {
      if (&g == cover)
        launch_gather_jacobian_full(J, bs, g.slots_dyn, g.slot_pos_dyn_host, g.block_begin, g.nblocks,
                                    g.blist_ptr.get(), g.blist.get(), d_ej.get(), jac_f32, s, gout);
      else
        launch_gather_jacobian(J, bs, g.slots_dyn, g.slot_pos_dyn.get(), g.block_begin, g.nblocks, g.blist_ptr.get(),
                               g.blist.get(), d_ej.get(), jac_f32, s, &g == cover ? gout : JacobianGatherOut{});
    }
  }
  if (ca != 0.0) {
    for (const auto& g : fgroups) {
      FaceParams p{};
      p.coords = d_coords.get();
      p.fverts = g.fverts.get();
      p.node_in = g.node_in.get();
      p.node_out = g.node_out.get();
      p.bpos = g.bpos.get();
      p.normal = g.normal.get();
      p.ielem = g.ielem.get();
      p.fvolume = g.fvolume.get();
      p.elem_in = g.elem_in.get();
      p.elem_out = g.elem_out.get();
      p.cells = d_cells.get();
      for (int side = 0; side < 2; ++side) {
        const int c = g.comp[side];
        p.vnode[side] = c >= 0 ? d_comp_vnode[c].get() : nullptr;
        p.terms[side] = g.d_terms[side].get();
        p.n_terms[side] = static_cast<int>(g.terms[side].size());
        p.prog[side] = g.prog[side].view();
        p.species_offset[side] = c >= 0 ? species_offset[c] : 0;
        p.ns[side] = c >= 0 ? ns[c] : 0;
      }
      p.tables = tables;
      p.x = x;
      p.r = r;
      p.J = J;
      p.bs = bs;
      p.t = t;
      p.ca = ca;
      for (size_t k = 0; k + 1 < g.color_offsets.size(); ++k) {
        if (numerical_jacobian && (mode & 2)) {
          // jacobian.type = numerical: the residual as usual, the Jacobian by forward differences
          if ((mode & 1) && r) launch_faces(dim, p, g.color_offsets[k], g.color_offsets[k + 1], 1, s);
          if (J) launch_faces_fd(dim, p, g.color_offsets[k], g.color_offsets[k + 1], fd_eps, s);
        } else {
          launch_faces(dim, p, g.color_offsets[k], g.color_offsets[k + 1], mode, s);
        }
      }
    }
  }
  return gout.sell != nullptr;
}

void Model::jacobian_apply(const double* x, double t, double cm, double ca, const double* v, double* y,
                           cudaStream_t s) const {
  cuda_check(cudaMemsetAsync(y, 0, static_cast<size_t>(nnodes) * bs * sizeof(double), s), "memset");
  const Bsr A0 = bsr(nullptr, nullptr);
  if (has_Ms && cm != 0.0) spmv_acc(A0, d_Ms.get(), v, y, cm, s);
  if (has_Ks && ca != 0.0) spmv_acc(A0, d_Ks.get(), v, y, ca, s);
  for (const auto& g : vgroups) {
    if (!(cm != 0.0 && g.has_mass) && !(ca != 0.0 && g.has_stiffness)) continue;
    if (g.slots_dyn == 0) continue;
    VolumeParams p{};
    p.coords = d_coords.get();
    p.verts = g.verts.get();
    p.nodes = g.nodes.get();
    p.bpos = g.bpos.get();
    p.prog = g.prog_all.view();
    p.res_terms = g.d_res_a.get();
    p.n_res_terms = static_cast<int>(g.res_terms_a.size());
    p.jac_terms = g.d_jac.get();
    p.n_jac_terms = static_cast<int>(g.jac_terms.size());
    p.tables = tables;
    p.x = x;
    p.bs = bs;
    p.species_offset = species_offset[g.comp];
    p.t = t;
    p.cm = cm;
    p.ca = ca;
    p.fd_eps = fd_eps;
    p.er = d_er.get();
    p.n_slots = g.slots_dyn;
    p.all_mass = g.dyn_all_mass ? 1 : 0;
    p.v = v;
    p.slot_pos = g.slot_pos_dyn.get();
    set_volume_flags(p, g.prog_all.host, g.res_terms_a, g.jac_terms, dim);
    launch_volume(dim, g.ns, p, 0, static_cast<int>(g.ne), 2 | kVolumeJacobianApply, s);
    launch_gather_residual(y, bs, g.ns, g.node_begin, g.nnodes, g.rlist_ptr.get(), g.rlist.get(), d_er.get(), s);
  }
  if (ca != 0.0) {
    for (const auto& g : fgroups) {
      FaceParams p{};
      p.coords = d_coords.get();
      p.fverts = g.fverts.get();
      p.node_in = g.node_in.get();
      p.node_out = g.node_out.get();
      p.bpos = g.bpos.get();
      p.normal = g.normal.get();
      p.ielem = g.ielem.get();
      p.fvolume = g.fvolume.get();
      p.elem_in = g.elem_in.get();
      p.elem_out = g.elem_out.get();
      p.cells = d_cells.get();
      for (int side = 0; side < 2; ++side) {
        const int c = g.comp[side];
        p.vnode[side] = c >= 0 ? d_comp_vnode[c].get() : nullptr;
        p.terms[side] = g.d_terms[side].get();
        p.n_terms[side] = static_cast<int>(g.terms[side].size());
        p.prog[side] = g.prog[side].view();
        p.species_offset[side] = c >= 0 ? species_offset[c] : 0;
        p.ns[side] = c >= 0 ? ns[c] : 0;
      }
      p.tables = tables;
      p.x = x;
      p.v = v;
      p.y = y;
      p.bs = bs;
      p.t = t;
      p.ca = ca;
      for (size_t k = 0; k + 1 < g.color_offsets.size(); ++k)
        launch_faces(dim, p, g.color_offsets[k], g.color_offsets[k + 1], kFaceJacobianApply, s);
    }
  }
  launch_unit_rows_apply(padded ? d_row_ns.get() : nullptr, nnodes, bs, d_cons_idx.get(), n_constraints, v, y, s);
}

}  // namespace dcgpu
