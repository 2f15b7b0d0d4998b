// Transform/reduce operators, dune/copasi/model/diffusion_reaction/reduce.hh:40-285.
//
// For every key of the reduce section: value = initial.value (default 0); then, over every
// cell in grid order and every point of the order-4 rule, value = reduction(evaluation,
// value) with reduction the user function "init, val: ..." (default +); the result is
// combined with initial.value once more, as reduce.hh:237-241 does for its single thread;
// "transformation" ("arg: ...") is applied; "error" / "warn" ("arg: ...") flag the key
// when they evaluate non-zero (reduce.hh:254-276).
//
// The evaluations of all keys run in one device pass (reduce.cu).  Sums, maxima and minima
// (reductions "a, b: a + b", "max(a, b)", "min(a, b)" in either argument order, and the
// default) fold on the device, the sum in block order rather than grid order; any other
// reduction function is folded on the host in grid order over the copied-back values.
// Species whose compartment does not contain a cell evaluate to 0 there.
#include <cfloat>
#include <cmath>
#include <map>

#include "model.hpp"
#include "reduce.cuh"

namespace dcgpu {

namespace {

const char* kRedAxes[3] = {"x", "y", "z"};

std::string strip_spaces(const std::string& s) {
  std::string o;
  for (char c : s)
    if (c != ' ' && c != '\t') o += c;
  return o;
}

// "a, b: body" compiled with its arguments as program inputs 0..n-1
struct HostFunction {
  Program p;
  std::vector<std::string> args;
  std::string body;
  double operator()(const ParserContext& ctx, const std::vector<double>& argv) const {
    std::vector<double> in(p.inputs.size());
    for (size_t i = 0; i < p.inputs.size(); ++i) in[i] = argv[p.inputs[i] - IN_SPECIES];
    return run_program_host(p, ctx, in.data());
  }
};

HostFunction compile_function(const ParserContext& ctx, const std::string& text, size_t nargs, const char* what) {
  HostFunction f;
  const auto colon = text.find(':');
  if (colon == std::string::npos) throw ConfigError(std::string(what) + " needs the form 'args: expression'");
  std::string head = text.substr(0, colon);
  size_t pos = 0;
  while (pos <= head.size()) {
    size_t c = head.find(',', pos);
    if (c == std::string::npos) c = head.size();
    std::string a = trim(head.substr(pos, c - pos));
    if (!a.empty()) f.args.push_back(a);
    pos = c + 1;
  }
  if (f.args.size() != nargs)
    throw ConfigError(std::string(what) + " must have exactly " + std::to_string(nargs) + " argument(s)");
  f.body = text.substr(colon + 1);
  ProgramBuilder pb(ctx);
  Resolver res = [&](const std::string& nm) -> std::optional<Symbol> {
    for (size_t i = 0; i < f.args.size(); ++i)
      if (nm == f.args[i]) {
        Symbol s;
        s.is_input = true;
        s.input = static_cast<uint16_t>(IN_SPECIES + i);
        return s;
      }
    return std::nullopt;
  };
  pb.add_output(pb.compile_text(f.body, res));
  f.p = pb.finish();
  return f;
}

}  // namespace

std::vector<ReduceResult> Model::reduce(const double* x, double t, const Ini& rcfg, cudaStream_t s) const {
  std::vector<ReduceResult> out;
  const auto keys = rcfg.sub_keys();
  if (keys.empty() || mesh.ne == 0) return out;
  const int nl = dim + 1;
  const int nq = reduce_points(dim);

  // cell tables in grid order (built on first use)
  if (d_red_cells.size() != static_cast<size_t>(mesh.ne) * nl) {
    std::vector<int32_t> cn(static_cast<size_t>(mesh.ne) * nl, -1), cc(mesh.ne, -1);
    for (int64_t e = 0; e < mesh.ne; ++e) {
      const int c = elem_comp[e];
      cc[e] = c;
      if (c < 0 || ns[c] == 0) continue;
      for (int a = 0; a < nl; ++a) cn[e * nl + a] = comp_vnode[c][mesh.cells[e * nl + a]];
    }
    std::vector<int8_t> spc(species.size()), spl(species.size());
    for (size_t g = 0; g < species.size(); ++g) {
      spc[g] = static_cast<int8_t>(species[g].comp);
      spl[g] = static_cast<int8_t>(species[g].local);
    }
    d_red_nodes.upload(cn);
    d_red_comp.upload(cc);
    d_red_spc.upload(spc);
    d_red_spl.upload(spl);
    d_red_cells.upload(mesh.cells);
  }

  // one program with an output per key
  ProgramBuilder pb(ctx);
  Resolver res = [&](const std::string& nm) -> std::optional<Symbol> {
    Symbol sym;
    for (const auto& sp : species) {
      if (nm == sp.name) {
        sym.is_input = true;
        sym.input = static_cast<uint16_t>(IN_SPECIES + sp.global);
        return sym;
      }
      for (int d = 0; d < 3; ++d)
        if (nm == "grad_" + sp.name + "_" + kRedAxes[d]) {
          if (d < dim) {
            sym.is_input = true;
            sym.input = static_cast<uint16_t>(IN_GRAD + sp.global * 3 + d);
          }
          return sym;
        }
    }
    for (int d = 0; d < 3; ++d)
      if (nm == std::string("position_") + kRedAxes[d]) {
        if (d < dim) {
          sym.is_input = true;
          sym.input = static_cast<uint16_t>(IN_POSITION + d);
        }
        return sym;
      }
    if (nm == "time") { sym.value = t; return sym; }
    if (nm == "integration_factor") { sym.is_input = true; sym.input = IN_INTEGRATION_FACTOR; return sym; }
    if (nm == "entity_volume") { sym.is_input = true; sym.input = IN_ENTITY_VOLUME; return sym; }
    if (nm == "in_volume") { sym.value = 1.0; return sym; }
    if (nm == "in_boundary" || nm == "in_skeleton") return sym;
    if (nm == "no_value") { sym.value = DBL_MAX; return sym; }
    return std::nullopt;
  };
  for (const auto& key : keys) {
    Ini sub = rcfg.sub(key);
    std::string ev = sub.has_key("evaluation.expression") ? trim(sub.get("evaluation.expression", "")) : "";
    pb.add_output(ev.empty() ? pb.constant(0.0) : pb.compile_text(ev, res));
  }
  ProgramBundle prog;
  prog.host = pb.finish();
  prog.upload();

  const int64_t npts = mesh.ne * nq;
  DeviceBuffer<double> vals(static_cast<size_t>(npts) * keys.size());
  ReduceParams p;
  p.ne = mesh.ne;
  p.coords = d_coords.get();
  p.cells = d_red_cells.get();
  p.cell_nodes = d_red_nodes.get();
  p.cell_comp = d_red_comp.get();
  p.sp_comp = d_red_spc.get();
  p.sp_local = d_red_spl.get();
  p.prog = prog.view();
  p.tables = tables;
  p.x = x;
  p.bs = bs;
  p.t = t;
  p.nkeys = static_cast<int>(keys.size());
  p.out = vals.get();
  launch_reduce_eval(dim, p, s);
  cuda_check(cudaGetLastError(), "reduce");

  constexpr int kBlocks = 304;
  DeviceBuffer<double> partial(kBlocks), result(keys.size());
  DeviceBuffer<unsigned> counter(1);
  cuda_check(cudaMemsetAsync(counter.get(), 0, sizeof(unsigned), s), "memset");
  std::vector<int> kind(keys.size(), -1);
  std::vector<HostFunction> red(keys.size());
  for (size_t k = 0; k < keys.size(); ++k) {
    Ini sub = rcfg.sub(keys[k]);
    if (!sub.has_key("reduction.expression")) {
      kind[k] = 0;
    } else {
      red[k] = compile_function(ctx, sub.get("reduction.expression", ""), 2, "Reduction");
      const std::string b = strip_spaces(red[k].body), a0 = red[k].args[0], a1 = red[k].args[1];
      if (b == a0 + "+" + a1 || b == a1 + "+" + a0) kind[k] = 0;
      else if (b == "max(" + a0 + "," + a1 + ")" || b == "max(" + a1 + "," + a0 + ")") kind[k] = 1;
      else if (b == "min(" + a0 + "," + a1 + ")" || b == "min(" + a1 + "," + a0 + ")") kind[k] = 2;
    }
    if (kind[k] >= 0)
      launch_fold(vals.get() + k * npts, npts, kind[k], partial.get(), kBlocks, counter.get(), result.get() + k, s);
  }
  std::vector<double> folded(keys.size(), 0.0);
  cuda_check(cudaMemcpyAsync(folded.data(), result.get(), keys.size() * sizeof(double), cudaMemcpyDeviceToHost, s),
             "reduce");
  cuda_check(cudaStreamSynchronize(s), "reduce");

  for (size_t k = 0; k < keys.size(); ++k) {
    Ini sub = rcfg.sub(keys[k]);
    const double init = sub.get_double("initial.value", 0.0);
    double v;
    if (kind[k] == 0) {
      v = (init + folded[k]) + init;
    } else if (kind[k] == 1) {
      v = std::fmax(std::fmax(init, folded[k]), init);
    } else if (kind[k] == 2) {
      v = std::fmin(std::fmin(init, folded[k]), init);
    } else {
      std::vector<double> h(npts);
      cuda_check(cudaMemcpy(h.data(), vals.get() + k * npts, npts * sizeof(double), cudaMemcpyDeviceToHost), "reduce");
      double acc = init;
      std::vector<double> argv(2);
      for (int64_t i = 0; i < npts; ++i) {
        argv[0] = h[i];
        argv[1] = acc;
        acc = red[k](ctx, argv);
      }
      argv[0] = acc;
      argv[1] = init;
      v = red[k](ctx, argv);
    }
    ReduceResult r;
    r.key = keys[k];
    if (sub.has_key("transformation.expression"))
      v = compile_function(ctx, sub.get("transformation.expression", ""), 1, "Transformation")(ctx, {v});
    r.value = v;
    if (sub.has_key("error.expression") &&
        compile_function(ctx, sub.get("error.expression", ""), 1, "Error function")(ctx, {v}) != 0.0)
      r.error = true;
    else if (sub.has_key("warn.expression") &&
             compile_function(ctx, sub.get("warn.expression", ""), 1, "Warning function")(ctx, {v}) != 0.0)
      r.warn = true;
    out.push_back(r);
  }
  return out;
}

}  // namespace dcgpu
