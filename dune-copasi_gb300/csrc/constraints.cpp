// Dirichlet (translation) constraints of the species.
//
// Replaces Dune::Copasi::Constraints (dune/copasi/model/constraints.hh:51-199) and the
// affine constraints container it fills.  "constrain.boundary" and "constrain.skeleton"
// expressions are evaluated once at set-up (time = NaN, constraints.hh:62-63) at the P1
// vertices of the faces of the species' compartment:
//   * a face with no neighbour cell in the compartment is a boundary face: in_boundary = 1,
//     the normal points out of the compartment cell;
//   * a face with the compartment on both sides is a skeleton face: in_skeleton = 1,
//     evaluated from both cells (normal out of each), and it constrains only vertices that
//     lie on no boundary face (the isBoundary check of constraints.hh:178);
//   * no_value (DBL_MAX) leaves the vertex free; when several faces give a vertex a value,
//     the first in (sorted face vertex ids, inside before outside) order is kept.
// P1 has no cell-interior DOFs, so "constrain.volume" never applies (constraints.hh:104).
//
// On the device a constrained entry takes its value before each stage solve, its
// residual row is zero and its Jacobian row a unit row, so every Newton correction leaves
// it unchanged.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <numeric>

#include "assemble.cuh"
#include "model.hpp"

namespace dcgpu {

namespace {
const char* kAxes[3] = {"x", "y", "z"};

// functor_factory_parser.impl.hh:121-124: an empty or all-zero expression is no functor
std::optional<std::string> expression_text(const Ini& sub) {
  std::string t = trim(sub.get("expression", ""));
  if (is_zero_expression(t)) return std::nullopt;
  return t;
}
}  // namespace

void Model::build_constraints() {
  Ini sf = cfg.sub("model").sub("scalar_field");
  struct Todo {
    const SpeciesInfo* sp;
    bool skeleton;
    Program p;
  };
  std::vector<Todo> todo;
  for (const auto& sp : species) {
    Ini c = sf.sub(sp.name);
    for (int kind = 0; kind < 2; ++kind) {
      const std::string key = kind == 0 ? "constrain.boundary" : "constrain.skeleton";
      if (!c.has_sub(key)) continue;
      auto txt = expression_text(c.sub(key));
      if (!txt) continue;
      ProgramBuilder pb(ctx);
      Resolver res = [&](const std::string& nm) -> std::optional<Symbol> {
        Symbol s;
        for (int d = 0; d < 3; ++d) {
          if (nm == std::string("position_") + kAxes[d] || nm == std::string("normal_") + kAxes[d]) {
            if (d < dim) {
              s.is_input = true;
              s.input = static_cast<uint16_t>((nm[0] == 'p' ? IN_POSITION : IN_NORMAL) + d);
            }
            return s;
          }
        }
        if (nm == "entity_volume") {
          s.is_input = true;
          s.input = IN_ENTITY_VOLUME;
          return s;
        }
        if (nm == "time") { s.value = std::nan(""); return s; }
        if (nm == "in_boundary") { s.value = kind == 0 ? 1.0 : 0.0; return s; }
        if (nm == "in_skeleton") { s.value = kind == 0 ? 0.0 : 1.0; return s; }
        if (nm == "in_volume" || nm == "integration_factor") return s;
        if (nm == "no_value") { s.value = DBL_MAX; return s; }
        return std::nullopt;
      };
      pb.add_output(pb.compile_text(*txt, res));
      todo.push_back({&sp, kind == 1, pb.finish()});
    }
  }
  if (todo.empty()) return;

  Faces F = compute_faces(mesh);
  std::vector<int64_t> ord(F.nf);
  std::iota(ord.begin(), ord.end(), 0);
  std::sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) {
    return std::lexicographical_compare(F.verts.begin() + a * dim, F.verts.begin() + (a + 1) * dim,
                                        F.verts.begin() + b * dim, F.verts.begin() + (b + 1) * dim);
  });
  const int nl = dim + 1;
  std::vector<int64_t> idx_all;
  std::vector<double> val_all;
  std::vector<char> taken(static_cast<size_t>(nnodes) * bs, 0);
  for (const auto& td : todo) {
    const int c = td.sp->comp;
    auto in_c = [&](int32_t e) { return e >= 0 && elem_comp[e] == c; };
    std::vector<char> bvert(mesh.nv, 0);
    for (int64_t f = 0; f < F.nf; ++f)
      if (in_c(F.e0[f]) != in_c(F.e1[f]))
        for (int j = 0; j < dim; ++j) bvert[F.verts[f * dim + j]] = 1;
    std::vector<char> done(mesh.nv, 0);
    std::vector<double> in(td.p.inputs.size());
    for (int64_t f : ord) {
      const bool i0 = in_c(F.e0[f]), i1 = in_c(F.e1[f]);
      int sides[2];
      int nsides = 0;
      if (!td.skeleton) {
        if (i0 == i1) continue;
        sides[nsides++] = i0 ? F.e0[f] : F.e1[f];
      } else {
        if (!(i0 && i1)) continue;
        sides[nsides++] = F.e0[f];
        sides[nsides++] = F.e1[f];
      }
      const int32_t* fv = &F.verts[f * dim];
      double p0[3] = {0, 0, 0}, t1[3] = {0, 0, 0}, t2[3] = {0, 0, 0};
      for (int d = 0; d < dim; ++d) {
        p0[d] = mesh.coords[static_cast<int64_t>(fv[0]) * dim + d];
        t1[d] = mesh.coords[static_cast<int64_t>(fv[1]) * dim + d] - p0[d];
        if (dim == 3) t2[d] = mesh.coords[static_cast<int64_t>(fv[2]) * dim + d] - p0[d];
      }
      double nrm0[3] = {0, 0, 0}, meas;
      if (dim == 2) {
        nrm0[0] = t1[1];
        nrm0[1] = -t1[0];
        meas = std::sqrt(t1[0] * t1[0] + t1[1] * t1[1]);
      } else {
        nrm0[0] = t1[1] * t2[2] - t1[2] * t2[1];
        nrm0[1] = t1[2] * t2[0] - t1[0] * t2[2];
        nrm0[2] = t1[0] * t2[1] - t1[1] * t2[0];
        meas = 0.5 * std::sqrt(nrm0[0] * nrm0[0] + nrm0[1] * nrm0[1] + nrm0[2] * nrm0[2]);
      }
      double len = 0.0;
      for (int d = 0; d < dim; ++d) len += nrm0[d] * nrm0[d];
      len = std::sqrt(len);
      for (int d = 0; d < dim; ++d) nrm0[d] /= len;
      for (int si = 0; si < nsides; ++si) {
        const int32_t e = sides[si];
        double ctr[3] = {0, 0, 0}, dot = 0.0;
        for (int d = 0; d < dim; ++d) {
          for (int a = 0; a < nl; ++a) ctr[d] += mesh.coords[static_cast<int64_t>(mesh.cells[e * nl + a]) * dim + d];
          ctr[d] /= nl;
          dot += nrm0[d] * (p0[d] - ctr[d]);
        }
        const double sgn = dot < 0 ? -1.0 : 1.0;
        for (int j = 0; j < dim; ++j) {
          const int32_t v = fv[j];
          if (done[v] || (td.skeleton && bvert[v])) continue;
          for (size_t i = 0; i < td.p.inputs.size(); ++i) {
            const uint16_t ik = td.p.inputs[i];
            if (ik >= IN_POSITION && ik < IN_POSITION + 3) in[i] = mesh.coords[static_cast<int64_t>(v) * dim + (ik - IN_POSITION)];
            else if (ik >= IN_NORMAL && ik < IN_NORMAL + 3) in[i] = sgn * nrm0[ik - IN_NORMAL];
            else in[i] = meas;  // IN_ENTITY_VOLUME
          }
          const double val = run_program_host(td.p, ctx, in.data());
          if (val == DBL_MAX) continue;
          done[v] = 1;
          const int64_t node = comp_vnode[c][v];
          const int64_t bi = node * bs + td.sp->local;
          if (taken[bi]) continue;
          taken[bi] = 1;
          idx_all.push_back(bi);
          val_all.push_back(val);
        }
      }
    }
  }
  std::vector<size_t> o(idx_all.size());
  std::iota(o.begin(), o.end(), 0);
  std::sort(o.begin(), o.end(), [&](size_t a, size_t b) { return idx_all[a] < idx_all[b]; });
  std::vector<int64_t> ci(o.size());
  std::vector<double> cv(o.size());
  for (size_t k = 0; k < o.size(); ++k) {
    ci[k] = idx_all[o[k]];
    cv[k] = val_all[o[k]];
  }
  cons_idx = ci;
  cons_val = cv;
  n_constraints = static_cast<int64_t>(ci.size());
  d_cons_idx.upload(ci);
  d_cons_val.upload(cv);
}

void Model::apply_constraints(double* x, cudaStream_t s) const {
  if (n_constraints) launch_constraints(x, d_cons_idx.get(), d_cons_val.get(), n_constraints, 0, s);
}
void Model::constrain_residual(double* r, cudaStream_t s) const {
  if (n_constraints) launch_constraints(r, d_cons_idx.get(), nullptr, n_constraints, 1, s);
}
void Model::constrain_jacobian(double* J, cudaStream_t s) const {
  if (n_constraints) {
    ConstraintRows cr{d_rowptr.get(), d_diag.get()};
    launch_constraint_rows(J, cr, d_cons_idx.get(), n_constraints, bs, s);
  }
}

}  // namespace dcgpu
