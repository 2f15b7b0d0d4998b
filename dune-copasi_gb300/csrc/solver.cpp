#include "solver.hpp"

#include "batch.hpp"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <limits>
#include <condition_variable>
#include <mutex>
#include <type_traits>

#include "assemble.cuh"
#include "gmres.cuh"
#include "linalg.cuh"

namespace dcgpu {

// ------------------------------------------------------------------ Runge-Kutta tables
// PDELab one-step parameter form: stage i (1-based) solves
//   sum_{j<=i} A[i-1][j] M(u_j, t + D[j] dt) + B[i-1][j] dt A(u_j, t + D[j] dt) = 0

RKTable RKTable::make(const std::string& name) {
  RKTable t;
  if (name == "ImplicitEuler") {
    t.A = {{-1.0, 1.0}};
    t.B = {{0.0, 1.0}};
    t.D = {0.0, 1.0};
  } else if (name == "ExplicitEuler") {
    t.A = {{-1.0, 1.0}};
    t.B = {{1.0, 0.0}};
    t.D = {0.0, 1.0};
  } else if (name == "Alexander2") {
    const double a = 1.0 - 0.5 * std::sqrt(2.0);
    t.A = {{-1.0, 1.0, 0.0}, {-1.0, 0.0, 1.0}};
    t.B = {{0.0, a, 0.0}, {0.0, 1.0 - a, a}};
    t.D = {0.0, a, 1.0};
  } else if (name == "Heun") {
    t.A = {{-1.0, 1.0, 0.0}, {-0.5, -0.5, 1.0}};
    t.B = {{1.0, 0.0, 0.0}, {0.0, 0.5, 0.0}};
    t.D = {0.0, 1.0, 1.0};
  } else if (name == "Shu3") {
    t.A = {{-1.0, 1.0, 0.0, 0.0}, {-0.75, -0.25, 1.0, 0.0}, {-1.0 / 3.0, 0.0, -2.0 / 3.0, 1.0}};
    t.B = {{1.0, 0.0, 0.0, 0.0}, {0.0, 0.25, 0.0, 0.0}, {0.0, 0.0, 2.0 / 3.0, 0.0}};
    t.D = {0.0, 1.0, 0.5, 1.0};
  } else if (name == "RungeKutta4") {
    t.A = {{-1.0, 1.0, 0.0, 0.0, 0.0}, {-1.0, 0.0, 1.0, 0.0, 0.0}, {-1.0, 0.0, 0.0, 1.0, 0.0},
           {-1.0, 0.0, 0.0, 0.0, 1.0}};
    t.B = {{0.5, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.5, 0.0, 0.0, 0.0}, {0.0, 0.0, 1.0, 0.0, 0.0},
           {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0, 0.0}};
    t.D = {0.0, 0.5, 0.5, 1.0, 1.0};
  } else if (name == "FractionalStepTheta") {
    const double th = 1.0 - 0.5 * std::sqrt(2.0), thp = 1.0 - 2.0 * th, al = 2.0 - std::sqrt(2.0),
                 be = 1.0 - al;
    t.A = {{-1.0, 1.0, 0.0, 0.0}, {0.0, -1.0, 1.0, 0.0}, {0.0, 0.0, -1.0, 1.0}};
    t.B = {{th * be, th * al, 0.0, 0.0}, {0.0, thp * al, thp * be, 0.0}, {0.0, 0.0, th * be, th * al}};
    t.D = {0.0, th, 1.0 - th, 1.0};
  } else if (name == "Alexander3") {
    const double al = 0.4358665215084590, tau2 = (1.0 + al) / 2.0;
    const double b1 = -(6.0 * al * al - 16.0 * al + 1.0) / 4.0, b2 = (6.0 * al * al - 20.0 * al + 5.0) / 4.0;
    t.A = {{-1.0, 1.0, 0.0, 0.0}, {-1.0, 0.0, 1.0, 0.0}, {-1.0, 0.0, 0.0, 1.0}};
    t.B = {{0.0, al, 0.0, 0.0}, {0.0, tau2 - al, al, 0.0}, {0.0, b1, b2, al}};
    t.D = {0.0, al, tau2, 1.0};
  } else {
    throw ConfigError("Not known time stepping type '" + name + "'");
  }
  return t;
}

// dune FloatCmp, relativeWeak with epsilon = 8 * DBL_EPSILON
static bool f_eq(double a, double b) { return std::fabs(a - b) <= 8.0 * DBL_EPSILON * std::max(std::fabs(a), std::fabs(b)); }
static bool f_le(double a, double b) { return a < b || f_eq(a, b); }
static bool f_lt(double a, double b) { return a < b && !f_eq(a, b); }
static bool f_gt(double a, double b) { return a > b && !f_eq(a, b); }

Solver::Solver(Model& m, cudaStream_t s) : model(m), stream(s) {
  n_ = m.nnodes * m.bs;
  x_.resize(n_);
  r_.resize(n_);
  stage_.resize(n_);
  const_.resize(n_);
  z_.resize(n_);
  J_.resize(static_cast<size_t>(m.nnzb()) * m.bs * m.bs);
  // model.assembly.split_residual = true (default) | false: the split stage residual of
  // one_step, for models whose mass form is static and that carry state-dependent
  // stiffness terms (Newton path, no constraints)
  {
    const std::string sr = m.cfg.get("model.assembly.split_residual", "true");
    if (sr != "true" && sr != "false") throw ConfigError("model.assembly.split_residual must be true or false");
    bool dyn_stiffness = !m.fgroups.empty();
    for (const auto& g : m.vgroups) dyn_stiffness = dyn_stiffness || g.has_stiffness;
    split_residual_ = sr == "true" && !m.dynamic_mass && dyn_stiffness && !m.is_linear && !m.numerical_jacobian &&
                      m.n_constraints == 0;
    if (split_residual_) dyn_.resize(n_);
  }
  kr_.resize(n_); krhat_.resize(n_); kp_.resize(n_); kv_.resize(n_); ks_.resize(n_); kt_.resize(n_);
  kphat_.resize(n_); kshat_.resize(n_); kx_.resize(n_);
  dinv_.resize(static_cast<size_t>(m.nnodes) * m.bs * m.bs);
  partial_.resize(kReduceBlocks * 4);
  // single-launch BiCGSTAB partial sums: room for two blocks on each of up to 256 SMs, so a
  // solve allocates nothing
  fpart_.resize(fused_bicgstab_partials(2 * 256));
  scal_.resize(32);
  counter_.resize(1);
  status_.resize(1);
  cuda_check(cudaMemsetAsync(counter_.get(), 0, sizeof(unsigned int), stream), "memset");
  cuda_check(cudaMemsetAsync(scal_.get(), 0, 32 * sizeof(double), stream), "memset");
  // 32 scalar slots + one for the deferred preconditioner status
  cuda_check(cudaMallocHost(&pinned_, 33 * sizeof(double)), "cudaMallocHost");
  rs_.partial = partial_.get();
  rs_.counter = counter_.get();
  rs_.result = scal_.get() + 16;

  Ini tso = m.cfg.sub("model").sub("time_step_operator");
  scheme_ = tso.get("type", "Alexander2");
  RKTable::make(scheme_);  // validate
  Ini ns = tso.sub("nonlinear_solver");
  newton_rel_ = ns.get_double("convergence_condition.relative_tolerance", 1e-4);
  auto range = ns.get_doubles("convergence_condition.iteration_range", {0.0, 40.0});
  if (range.size() != 2) throw ConfigError("convergence_condition.iteration_range needs two values");
  it_min_ = static_cast<int>(range[0]);
  it_max_ = static_cast<int>(range[1]);
  newton_abs_ = ns.get_double("convergence_condition.absolute_tolerance", 0.0);
  lin_threshold_ = ns.get_double("linearization_threshold", 0.0);
  dx_fixed_ = ns.get_bool("dx_inverse_fixed_tolerance", false);
  dx_min_rel_ = ns.get_double("dx_inverse_min_relative_tolerance", 0.1);
  norm_ = ns.get("norm", "l_2");
  if (norm_ != "l_2" && norm_ != "l_inf" && norm_ != "l_1") throw ConfigError("Not known nonlinear norm '" + norm_ + "'");
  Ini ls = tso.sub("linear_solver");
  std::string lt = ls.get("type", "UMFPack");
  // direct solvers of the reference (UMFPack default, SuperLU, DenseInverse) are replaced
  // by a BiCGSTAB solve converged to near machine precision
  lin_direct_ = (lt == "UMFPack" || lt == "SuperLU" || lt == "DenseInverse");
  // iterative registry of solver/istl/factory/iterative.hh:84-105: CG and the flexible /
  // generalized PCG variants (identical to CG for a fixed preconditioner) run as CG, the
  // GMRes variants as restarted GMRES (restart key as iterative.hh:63-64); Loop, Gradient
  // and MINRES converge to the same solution of the same correction equation and run as
  // BiCGSTAB
  if (!lin_direct_) {
    if (lt == "CG" || lt == "GeneralizedPCG" || lt == "RestartedFCG" || lt == "CompleteFCG") {
      krylov_cg_ = true;
    } else if (lt == "RestartedGMRes" || lt == "RestartedFlexibleGMRes") {
      // the flexible variant equals GMRES for a fixed preconditioner
      krylov_gmres_ = true;
      gmres_restart_ = static_cast<int>(ls.get_long("restart", 40));
      if (gmres_restart_ < 1 || gmres_restart_ > 500) throw ConfigError("linear_solver.restart must be in [1, 500]");
    } else if (lt != "BiCGSTAB" && lt != "Loop" && lt != "Gradient" && lt != "MINRES") {
      throw ConfigError("Not known linear solver type '" + lt + "'");
    }
  }
  lin_rel_ = ls.get_double("convergence_condition.relative_tolerance", 1e-4);
  lin_max_it_ = 500;
  if (ls.has_key("convergence_condition.iteration_range")) {
    auto r = ls.get_doubles("convergence_condition.iteration_range", {1.0, 500.0});
    lin_max_it_ = static_cast<int>(r.back());
  }
  if (lin_direct_) lin_max_it_ = std::max(lin_max_it_, 5000);
  // relative residual reduction that stands in for an exact direct solve inside Newton: a
  // correction off by 1e-10 (times the condition number) of its size is absorbed by the
  // next Newton iteration and leaves the converged stage solution within that fraction of
  // the last correction of the direct-solve one
  direct_tol_ = ls.get_double("direct_tolerance", 1e-10);
  if (!(direct_tol_ > 0.0 && direct_tol_ < 1.0)) throw ConfigError("linear_solver.direct_tolerance must be in (0, 1)");
  // linear_solver.matrix_free (make_step_operator.hh:201,289-293): the stage Jacobian is
  // never assembled; each Krylov product J v is evaluated element by element (and face by
  // face) at the Newton iterate, Model::jacobian_apply.  The reference then offers only its
  // iterative solvers (inverse.hh:31-58) and the matrix-free preconditioners Richardson and
  // InverseOperator (preconditioner.hh:94-95); the Krylov solve runs in fp64.
  matrix_free_ = ls.get_bool("matrix_free", false);
  if (matrix_free_) {
    if (lin_direct_)
      throw ConfigError("The key '" + lt + "' is not a known inverse operator type (linear_solver.matrix_free = true "
                        "takes an iterative solver)");
    if (m.numerical_jacobian)
      throw ConfigError("linear_solver.matrix_free = true with model.jacobian.type = numerical is not supported");
    mf_x_.resize(n_);
    J_.resize(0);
  }
  configure_preconditioner(ls);
  const bool want_mixed = ls.get("precision", "double") == "mixed";
  // mixed precision only: precision of the state-dependent Jacobian terms (single, default,
  // or double)
  const std::string jp = ls.get("jacobian_precision", "single");
  if (jp != "single" && jp != "double")
    throw ConfigError("linear_solver.jacobian_precision must be single or double, not '" + jp + "'");
  jac_f32_ = jp == "single";
  // mixed precision only: residual reduction of each fp32 correction solve inside the fp64
  // iterative refinement (fewer refinements against more fp32 iterations each)
  inner_set_ = ls.has_key("inner_reduction");
  mixed_inner_ = ls.get_double("inner_reduction", kMixedInnerReduction);
  if (!(mixed_inner_ >= 1e-7 && mixed_inner_ < 1.0))
    throw ConfigError("linear_solver.inner_reduction must be in [1e-7, 1)");
  const std::string fmt = ls.get("spmv", "auto");
  if (fmt == "auto") spmv_request_ = kSpmvAuto;
  else if (fmt == "bsr") spmv_request_ = kSpmvBsr;
  else if (fmt == "sell") spmv_request_ = kSpmvSell;
  else throw ConfigError("linear_solver.spmv must be auto, bsr or sell, not '" + fmt + "'");
  spmv_format = spmv_request_;
  // BiCGSTAB with block Jacobi: the whole solve in one cooperative launch (default), or one
  // launch per phase replayed from a CUDA graph (false)
  fused_ = ls.get_bool("single_launch", true);
  dec_ = tso.get_double("time_step_decrease_factor", 0.5);
  inc_ = tso.get_double("time_step_increase_factor", 1.1);
  has_min_ = tso.has_key("time_step_min");
  has_max_ = tso.has_key("time_step_max");
  dt_min_ = tso.get_double("time_step_min", 0.0);
  dt_max_ = tso.get_double("time_step_max", 0.0);
  if (f_gt(dec_, 1.0) || f_lt(dec_, 0.0)) throw ConfigError("Decrease factor must be in the range of (0,1]");
  if (f_lt(inc_, 1.0)) throw ConfigError("Increase factor must be in the range of (1,inf)");
  enable_mixed(want_mixed);
  std::vector<double> init = m.initial_state();
  set_state(init, tso.get_double("time_begin", 0.0));
}

// linear_solver.preconditioner (the reference's registry,
// dune/copasi/solver/istl/factory/preconditioner.hh:88-118; dune-istl parameter names):
//   Jacobi, BlockJacobi (default)  block Jacobi on the node blocks, fused into the Krylov
//                                  kernels; the reference's default SSOR is the key's
//                                  default only for its iterative solvers, whose
//                                  convergence (not their result) depends on it
//   SSOR, SOR, GaussSeidel         multicolour block SSOR / forward SOR (iterations,
//                                  relaxation; Gauss-Seidel: SOR with relaxation 1)
//   ILU (any fill level n), ILDL   multicolour block ILU(0) (relaxation)
//   DILU                           multicolour block DILU (relaxation)
//   Richardson                     z = relaxation * r
//   AMG                            the aggregation multigrid V-cycle (engine addition)
//   auto (the engine's default)    block Jacobi, until a solve does not converge within
//                                  preconditioner.auto_threshold (100) Krylov iterations:
//                                  that solve starts over with the multigrid, which stays
//                                  (stiff systems)
// InverseOperator (an inner solver as preconditioner) runs as block Jacobi: the outer
// solve converges to the same tolerance.
// the captured Krylov graphs hold the preconditioner's launches: drop them when it changes
void Solver::graphs_invalidate() {
  for (auto& g : graphs_) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
}

void Solver::build_multigrid() {
  const Model& m = model;
  std::vector<int32_t> group(m.nnodes, 0);
  for (size_t c = 0; c < m.comp_names.size(); ++c)
    for (int64_t k = m.comp_node_offset[c]; k < m.comp_node_offset[c + 1]; ++k) group[k] = static_cast<int32_t>(c);
  row_group_.upload(group);
  amg_->build(m.nnodes, m.bs, m.nnzb(), m.d_rowptr.get(), m.d_colidx.get(), m.d_diag.get(), row_group_.get(), stream);
  pc_ = amg_.get();
  graphs_invalidate();
}

void Solver::configure_preconditioner(const Ini& ls) {
  const Model& m = model;
  precond_ = ls.get("preconditioner.type", matrix_free_ ? "Richardson" : "auto");
  const std::string& p = precond_;
  if (matrix_free_) {
    // InverseOperator (an inner solve as preconditioner) runs as Richardson with relaxation 1
    if (p != "Richardson" && p != "InverseOperator")
      throw ConfigError("The key '" + p + "' is not a known preconditioner type (linear_solver.matrix_free = true: "
                        "Richardson, InverseOperator)");
    rich_.omega = p == "Richardson" ? ls.get_double("preconditioner.relaxation", 1.0) : 1.0;
    rich_.n = n_;
    pc_ = &rich_;
    return;
  }
  auto mc = [&](ColorPrecond::Kind kind, double omega_default) {
    mc_ = std::make_unique<ColorPrecond>();
    mc_->omega = ls.get_double("preconditioner.relaxation", omega_default);
    mc_->iterations = static_cast<int>(ls.get_long("preconditioner.iterations", 1));
    if (mc_->iterations < 1 || mc_->iterations > 100)
      throw ConfigError("linear_solver.preconditioner.iterations must be in [1, 100]");
    if (!(mc_->omega > 0.0 && mc_->omega < 2.0))
      throw ConfigError("linear_solver.preconditioner.relaxation must be in (0, 2)");
    mc_->build(kind, m.nnodes, m.bs, m.nnzb(), m.d_rowptr.get(), m.d_colidx.get(), m.d_diag.get(), stream);
    pc_ = mc_.get();
  };
  if (p == "Jacobi" || p == "BlockJacobi" || p == "InverseOperator") {
    pc_ = nullptr;
  } else if (p == "SSOR") {
    mc(ColorPrecond::Kind::Ssor, 1.0);
  } else if (p == "SOR") {
    mc(ColorPrecond::Kind::Sor, 1.0);
  } else if (p == "GaussSeidel") {
    mc(ColorPrecond::Kind::Sor, 1.0);
    mc_->omega = 1.0;
  } else if (p == "ILU" || p == "ILDL") {
    mc(ColorPrecond::Kind::Ilu0, 1.0);
  } else if (p == "DILU") {
    mc(ColorPrecond::Kind::Dilu, 1.0);
  } else if (p == "Richardson") {
    rich_.omega = ls.get_double("preconditioner.relaxation", 1.0);
    rich_.n = n_;
    pc_ = &rich_;
  } else if (p == "AMG" || p == "auto") {
    amg_ = std::make_unique<Amg>();
    const std::string sm = ls.get("preconditioner.smoother", "jacobi");
    if (sm == "jacobi") amg_->smoother = Amg::Smoother::Jacobi;
    else if (sm == "l1jacobi") amg_->smoother = Amg::Smoother::L1Jacobi;
    else if (sm == "gauss_seidel") amg_->smoother = Amg::Smoother::GaussSeidel;
    else if (sm == "ilu0") amg_->smoother = Amg::Smoother::Ilu0;
    else throw ConfigError("linear_solver.preconditioner.smoother must be jacobi, l1jacobi, gauss_seidel or ilu0, not '" +
                           sm + "'");
    amg_->omega = ls.get_double("preconditioner.relaxation", sm == "jacobi" ? 0.85 : 1.0);
    amg_->coarse_sweeps = static_cast<int>(ls.get_long("preconditioner.coarse_sweeps", 6));
    amg_->max_levels = static_cast<int>(ls.get_long("preconditioner.max_level", 10));
    amg_->coarsen_target = ls.get_long("preconditioner.coarsen_target", 0);
    amg_->mis_distance = static_cast<int>(ls.get_long("preconditioner.aggregation_distance", 2));
    amg_->correction = ls.get_double("preconditioner.coarse_correction", 1.0);
    amg_->finest_post_smoothing = ls.get_bool("preconditioner.finest_post_smoothing", true);
    amg_->w_levels = static_cast<int>(ls.get_long("preconditioner.w_levels", 0));
    if (amg_->w_levels < 0 || amg_->w_levels > 3)
      throw ConfigError("linear_solver.preconditioner.w_levels must be in [0, 3]");
    amg_->warp_rows_below = ls.get_long("preconditioner.warp_rows_below", Amg::kWarpRowsBelow);
    if (!(amg_->correction > 0.0 && amg_->correction < 4.0))
      throw ConfigError("linear_solver.preconditioner.coarse_correction must be in (0, 4)");
    if (amg_->mis_distance != 1 && amg_->mis_distance != 2)
      throw ConfigError("linear_solver.preconditioner.aggregation_distance must be 1 or 2");
    if (amg_->max_levels < 1) throw ConfigError("linear_solver.preconditioner.max_level must be >= 1");
    if (!(amg_->omega > 0.0 && amg_->omega < 2.0))
      throw ConfigError("linear_solver.preconditioner.relaxation must be in (0, 2)");
    auto_threshold_ = static_cast<int>(ls.get_long("preconditioner.auto_threshold", kAutoMultigridIterations));
    if (auto_threshold_ < 1) throw ConfigError("linear_solver.preconditioner.auto_threshold must be >= 1");
    auto_pc_ = p == "auto";
    if (!auto_pc_) build_multigrid();
  } else {
    throw ConfigError("The key '" + p + "' is not a known preconditioner type");
  }
}

std::string Solver::precond_info() const {
  if (auto_pc_)
    return std::string("{\"type\": \"auto\", \"active\": ") +
           (amg_->built() ? amg_->describe() : std::string("{\"type\": \"block_jacobi\"}")) + "}";
  if (amg_) return amg_->describe();
  if (mc_) return mc_->describe();
  if (pc_ == &rich_) return "{\"type\": \"Richardson\", \"relaxation\": " + std::to_string(rich_.omega) + "}";
  return "{\"type\": \"block_jacobi\", \"requested\": \"" + precond_ + "\"}";
}

void Solver::enable_mixed(bool on) {
  mixed_precision = on;
  if (matrix_free_) return;  // the matrix-free Krylov solve runs in fp64
  if (on && fr_.size() != static_cast<size_t>(n_)) {
    fr_.resize(n_); frhat_.resize(n_); fp_.resize(n_); fv_.resize(n_); fs_.resize(n_); ft_.resize(n_);
    fphat_.resize(n_); fshat_.resize(n_); fx_.resize(n_); fb_.resize(n_);
    fp2_.resize(n_); fv2_.resize(n_);
    fdinv_.resize(static_cast<size_t>(model.nnodes) * model.bs * model.bs);
    if (spmv_request_ != kSpmvSell) J32_.resize(static_cast<size_t>(model.nnzb()) * model.bs * model.bs);
    if (spmv_request_ != kSpmvBsr) {
      // the padding slots stay zero: the fused gather of Model::assemble writes real blocks only
      Js32_.resize(static_cast<size_t>(model.sell_slots) * 32 * model.bs * model.bs);
      cuda_check(cudaMemset(Js32_.get(), 0, Js32_.size() * sizeof(float)), "memset");
    }
  }
}

// Times the thread-per-row BSR SpMV and the warp-per-slice SELL-32 SpMV on the current fp32
// operator (both copies must be filled), five launches each after one warm-up, and keeps
// the faster layout for the rest of the run.
void Solver::tune_spmv() {
  const Bsr A = model.bsr(J_.get(), J32_.get());
  const Sell S = model.sell();
  cudaEvent_t e0, e1;
  cuda_check(cudaEventCreate(&e0), "cudaEventCreate");
  cuda_check(cudaEventCreate(&e1), "cudaEventCreate");
  constexpr int kReps = 5;
  for (int f = 0; f < 2; ++f) {
    auto run = [&] {
      if (f == 0) spmv32_vals(A, J32_.get(), fp_.get(), fv_.get(), stream);
      else spmv_sell32(S, Js32_.get(), fp_.get(), fv_.get(), stream);
    };
    run();
    cuda_check(cudaEventRecord(e0, stream), "cudaEventRecord");
    for (int k = 0; k < kReps; ++k) run();
    cuda_check(cudaEventRecord(e1, stream), "cudaEventRecord");
    cuda_check(cudaEventSynchronize(e1), "cudaEventSynchronize");
    float ms = 0.0f;
    cuda_check(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
    spmv_tune_us[f] = 1e3 * ms / kReps;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  spmv_format = spmv_tune_us[1] < spmv_tune_us[0] ? kSpmvSell : kSpmvBsr;
  if (spmv_format == kSpmvBsr) Js32_.resize(0);
  else J32_.resize(0);
}

Solver::~Solver() {
  if (pinned_) cudaFreeHost(pinned_);
  for (auto& p : pending_) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (cudaEvent_t e : event_pool_) cudaEventDestroy(e);
  for (auto& g : graphs_)
    if (g) cudaGraphExecDestroy(g);
  for (cudaEvent_t e : graph_events_) cudaEventDestroy(e);
  for (cudaEvent_t e : fused_ev_)
    if (e) cudaEventDestroy(e);
}

void Solver::set_state(const std::vector<double>& ref, double t) {
  set_state(ref.data(), static_cast<int64_t>(ref.size()), t);
}

// one copy of the caller's reference-layout vector to the device and a scatter kernel into
// the blocked layout (padded slots zero); no host-side reordering or temporary vectors
void Solver::set_state(const double* ref, int64_t n, double t) {
  if (n != model.ndof) throw std::invalid_argument("state size mismatch");
  if (ref_stage_.size() != static_cast<size_t>(n)) ref_stage_.resize(n);
  cuda_check(cudaMemcpyAsync(ref_stage_.get(), ref, n * sizeof(double), cudaMemcpyHostToDevice, stream), "set_state");
  if (model.padded) cuda_check(cudaMemsetAsync(x_.get(), 0, n_ * sizeof(double), stream), "set_state");
  scatter_idx(n, model.d_ref2blk.get(), ref_stage_.get(), x_.get(), stream);
  cuda_check(cudaStreamSynchronize(stream), "set_state");
  t_ = t;
  dyn_valid_ = false;
}

void Solver::get_state(double* out, int64_t n) const {
  if (n != model.ndof) throw std::invalid_argument("state size mismatch");
  if (ref_stage_.size() != static_cast<size_t>(n)) ref_stage_.resize(n);
  gather_idx(n, model.d_ref2blk.get(), x_.get(), ref_stage_.get(), stream);
  cuda_check(cudaMemcpyAsync(out, ref_stage_.get(), n * sizeof(double), cudaMemcpyDeviceToHost, stream), "get_state");
  cuda_check(cudaStreamSynchronize(stream), "get_state");
}

std::vector<double> Solver::get_state() const {
  std::vector<double> ref(model.ndof);
  get_state(ref.data(), model.ndof);
  return ref;
}

void Solver::check_setup_status() {
  if (!setup_status_pending_) return;
  setup_status_pending_ = false;
  cuda_check(cudaStreamSynchronize(stream), "status");  // normally already idle: the solve read its result
  if (*pinned_status()) throw StepFailure("singular diagonal block in the Jacobian");
}

double Solver::read_scalar(int slot) {
  double v;
  read_scalars(&v, slot, 1);
  return v;
}

void Solver::read_scalars(double* out, int first, int count) {
  cuda_check(cudaMemcpyAsync(pinned_, scal_.get() + first, count * sizeof(double), cudaMemcpyDeviceToHost, stream),
             "read scalars");
  cuda_check(cudaStreamSynchronize(stream), "read scalars");
  for (int i = 0; i < count; ++i) out[i] = pinned_[i];
  tflush();
}

void Solver::enable_profiling(bool on) {
  profiling_ = on;
  kernel_times = KernelTimes{};
}

void Solver::tbegin(int cat) {
  if (!profiling_) return;
  PendingTiming p{cat, nullptr, nullptr};
  for (cudaEvent_t* e : {&p.a, &p.b}) {
    if (!event_pool_.empty()) {
      *e = event_pool_.back();
      event_pool_.pop_back();
    } else {
      cuda_check(cudaEventCreate(e), "cudaEventCreate");
    }
  }
  cuda_check(cudaEventRecord(p.a, stream), "cudaEventRecord");
  pending_.push_back(p);
}

void Solver::tend() {
  if (!profiling_ || pending_.empty()) return;
  cuda_check(cudaEventRecord(pending_.back().b, stream), "cudaEventRecord");
}

void Solver::tflush() {
  if (pending_.empty()) return;
  for (auto& p : pending_) {
    float ms = 0.0f;
    cuda_check(cudaEventElapsedTime(&ms, p.a, p.b), "cudaEventElapsedTime");
    kernel_times.ms[p.cat] += ms;
    kernel_times.calls[p.cat] += 1;
    event_pool_.push_back(p.a);
    event_pool_.push_back(p.b);
  }
  pending_.clear();
}

double Solver::norm2(const double* v) {
  dot(v, v, n_, rs_, 0, stream);
  return read_scalar(16);
}

void Solver::setup_preconditioner() {
  cuda_check(cudaMemsetAsync(status_.get(), 0, sizeof(int), stream), "memset");
  Bsr A = model.bsr(J_.get(), nullptr);
  block_jacobi_setup(A, model.d_diag.get(), dinv_.get(), status_.get(), stream,
                     mixed_precision ? fdinv_.get() : nullptr);
  int st = 0;
  if (!pc_) {
    // read with the solve's own result instead of a stream synchronisation of its own
    // (check_setup_status); a singular block only makes that solve's values meaningless
    cuda_check(cudaMemcpyAsync(pinned_status(), status_.get(), sizeof(int), cudaMemcpyDeviceToHost, stream),
               "status");
    setup_status_pending_ = true;
  } else {
    cuda_check(cudaMemcpyAsync(&st, status_.get(), sizeof(int), cudaMemcpyDeviceToHost, stream), "status");
    cuda_check(cudaStreamSynchronize(stream), "status");
    if (st) throw StepFailure("singular diagonal block in the Jacobian");
  }
  if (mixed_precision) {
    // the BSR copy feeds the BSR SpMV and the tuner; the SELL-32 copy feeds the SELL SpMV
    // (the separately launched preconditioners keep their own copies)
    const bool need_bsr = spmv_format != kSpmvSell;
    const bool need_sell = spmv_format != kSpmvBsr;
    if (need_bsr) to_float(static_cast<int64_t>(model.nnzb()) * model.bs * model.bs, J_.get(), J32_.get(), stream);
    if (need_sell && !jac_sell_fresh_) bsr_to_sell(A, J_.get(), model.sell(), Js32_.get(), stream);
    if (spmv_format == kSpmvAuto) tune_spmv();
  }
  if ((amg_ && amg_->built()) || mc_) {
    // in the mixed path the fine level reads the Krylov solve's own SELL-32 operator copy
    const Sell S = model.sell();
    const bool share = mixed_precision && spmv_format == kSpmvSell && Js32_.size() > 0;
    const Sell* sp = share ? &S : nullptr;
    const float* sv = share ? Js32_.get() : nullptr;
    if (amg_) amg_->setup(J_.get(), dinv_.get(), fdinv_.get(), mixed_precision, status_.get(), stream, sp, sv);
    else mc_->setup(J_.get(), dinv_.get(), fdinv_.get(), mixed_precision, status_.get(), stream, sp, sv);
    cuda_check(cudaMemcpyAsync(&st, status_.get(), sizeof(int), cudaMemcpyDeviceToHost, stream), "status");
    cuda_check(cudaStreamSynchronize(stream), "status");
    if (st) throw StepFailure(amg_ ? "singular diagonal block in a coarse multigrid level"
                                   : "singular pivot block in the preconditioner factorisation");
  }
}

// Graph of kKrylovChunk BiCGSTAB iterations on this solver's fixed workspace (fp64 or
// fp32); with profiling on, event-record nodes bracket the two SpMV kernels of every
// iteration so their device time can be read after the replay.
cudaGraphExec_t Solver::krylov_graph(bool fp32) {
  const int slot = (fp32 ? 1 : 0) + (profiling_ ? 2 : 0);
  if (graphs_[slot]) return graphs_[slot];
  Bsr A = model.bsr(J_.get(), J32_.get());
  double* sc = scal_.get();
  cudaEvent_t* ev = nullptr;
  if (profiling_) {
    if (graph_events_.empty()) {
      graph_events_.resize(kKrylovChunk * 4);
      for (auto& e : graph_events_) cuda_check(cudaEventCreate(&e), "cudaEventCreate");
    }
    ev = graph_events_.data();
  }
  cudaGraph_t g = nullptr;
  const long long before = launch_count_this_thread();
  cuda_check(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
  for (int k = 0; k < kKrylovChunk; ++k) {
    cudaEvent_t* e = ev ? ev + 4 * k : nullptr;
    const Preconditioner* pc = pc_;
    if (fp32) {
      KrylovVectors<float> kv{fx_.get(), fr_.get(), frhat_.get(), fp_.get(), fv_.get(), fs_.get(), ft_.get(),
                              fphat_.get(), fshat_.get()};
      const bool sell = spmv_format == kSpmvSell;
      const Sell S = model.sell();
      const float* vals = sell ? Js32_.get() : J32_.get();
      if (krylov_cg_) cg_iteration<float, float>(A, vals, fdinv_.get(), kv, rs_, sc, stream, pc, sell ? &S : nullptr);
      else krylov_iteration<float, float>(A, vals, fdinv_.get(), kv, rs_, sc, stream, e, pc, sell ? &S : nullptr);
    } else {
      KrylovVectors<double> kv{kx_.get(), kr_.get(), krhat_.get(), kp_.get(), kv_.get(), ks_.get(), kt_.get(),
                               kphat_.get(), kshat_.get()};
      if (krylov_cg_) cg_iteration<double, double>(A, J_.get(), dinv_.get(), kv, rs_, sc, stream, pc);
      else krylov_iteration<double, double>(A, J_.get(), dinv_.get(), kv, rs_, sc, stream, e, pc);
    }
  }
  cuda_check(cudaStreamEndCapture(stream, &g), "cudaStreamEndCapture");
  cuda_check(cudaGraphInstantiate(&graphs_[slot], g, 0), "cudaGraphInstantiate");
  cudaGraphDestroy(g);
  // the capture launched nothing; replays are counted
  const long long captured = launch_count_this_thread() - before;
  launches_per_iter_ = static_cast<int>(captured / kKrylovChunk);
  count_launches(-captured);
  return graphs_[slot];
}

// Restarted GMRES with right preconditioning (dune-istl RestartedGMResSolver semantics:
// restart length m, relative reduction of the residual norm), classical Gram-Schmidt with
// one re-orthogonalisation pass, Givens rotations on the host (one synchronisation per
// iteration).  Right-hand side in kr_ / fr_, solution left in kx_ / fx_.
template <class T>
int Solver::gmres_t(double rel, int max_it, int* iters) {
  constexpr bool f32 = std::is_same_v<T, float>;
  const int64_t n = n_;
  const int m = gmres_restart_;
  DeviceBuffer<T>& Vbuf = [&]() -> DeviceBuffer<T>& {
    if constexpr (f32) return gV32_;
    else return gV_;
  }();
  if (Vbuf.size() != static_cast<size_t>(m + 1) * n) Vbuf.resize(static_cast<size_t>(m + 1) * n);
  if (gh_.size() < static_cast<size_t>(3 * (m + 2))) gh_.resize(3 * (m + 2));
  if (gpart_.size() < static_cast<size_t>(kGmresBlocks) * (m + 1)) gpart_.resize(static_cast<size_t>(kGmresBlocks) * (m + 1));
  T* V = Vbuf.get();
  T* b = f32 ? reinterpret_cast<T*>(fr_.get()) : reinterpret_cast<T*>(kr_.get());
  T* x = f32 ? reinterpret_cast<T*>(fx_.get()) : reinterpret_cast<T*>(kx_.get());
  T* r = f32 ? reinterpret_cast<T*>(frhat_.get()) : reinterpret_cast<T*>(krhat_.get());
  T* z = f32 ? reinterpret_cast<T*>(fphat_.get()) : reinterpret_cast<T*>(kphat_.get());
  T* u = f32 ? reinterpret_cast<T*>(fv_.get()) : reinterpret_cast<T*>(kv_.get());
  double* h1 = gh_.get();
  double* h2 = gh_.get() + (m + 2);
  double* hn = gh_.get() + 2 * (m + 2);
  const Bsr A = model.bsr(J_.get(), J32_.get());
  const Sell S = model.sell();
  // the preconditioner launches check a device "done" flag: keep it cleared
  cuda_check(cudaMemsetAsync(scal_.get(), 0, KS_COUNT * sizeof(double), stream), "memset");
  auto precond = [&](const T* in, T* out) {
    if (pc_) {
      pc_->apply(in, out, scal_.get(), KS_DONE, stream);
    } else if constexpr (f32) {
      block_jacobi_apply32(static_cast<int>(model.nnodes), model.bs, fdinv_.get(), in, out, stream);
    } else {
      block_jacobi_apply(static_cast<int>(model.nnodes), model.bs, dinv_.get(), in, out, stream);
    }
  };
  auto apply_A = [&](const T* in, T* out) {
    if constexpr (f32) {
      if (spmv_format == kSpmvSell) spmv_sell32(S, Js32_.get(), in, out, stream);
      else spmv32_vals(A, J32_.get(), in, out, stream);
    } else {
      if (matrix_free_) jacobian_apply_mf(in, out);
      else spmv(A, in, out, stream);
    }
  };
  auto norm = [&](const T* v) {
    gmres_mdot<T>(v, n, 1, v, hn, gpart_.get(), false, stream);
    double h = 0.0;
    cuda_check(cudaMemcpyAsync(&h, hn, sizeof(double), cudaMemcpyDeviceToHost, stream), "gmres");
    cuda_check(cudaStreamSynchronize(stream), "gmres");
    return std::sqrt(h);
  };
  cuda_check(cudaMemsetAsync(x, 0, n * sizeof(T), stream), "memset");
  cuda_check(cudaMemcpyAsync(r, b, n * sizeof(T), cudaMemcpyDeviceToDevice, stream), "copy");
  const double beta0 = norm(r);
  *iters = 0;
  if (beta0 == 0.0) return DC_OK;
  if (!std::isfinite(beta0)) return DC_ERR_DIVERGED;
  const double target = rel * beta0;
  double beta = beta0;
  std::vector<double> H(static_cast<size_t>(m + 1) * m), cs(m), sn(m), g(m + 1), hc1(m + 1), hc2(m + 1);
  int total = 0;
  while (true) {
    gmres_scale_value<T>(V, r, n, 1.0 / beta, stream);
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int k = 0;
    for (int j = 0; j < m && total < max_it; ++j) {
      T* vj1 = V + static_cast<int64_t>(j + 1) * n;
      precond(V + static_cast<int64_t>(j) * n, z);
      apply_A(z, vj1);
      gmres_mdot<T>(V, n, j + 1, vj1, h1, gpart_.get(), false, stream);
      gmres_maxpy<T>(vj1, V, n, j + 1, h1, -1.0, stream);
      gmres_mdot<T>(V, n, j + 1, vj1, h2, gpart_.get(), false, stream);
      gmres_maxpy<T>(vj1, V, n, j + 1, h2, -1.0, stream);
      gmres_mdot<T>(vj1, n, 1, vj1, hn, gpart_.get(), false, stream);
      cuda_check(cudaMemcpyAsync(hc1.data(), h1, (j + 1) * sizeof(double), cudaMemcpyDeviceToHost, stream), "gmres");
      cuda_check(cudaMemcpyAsync(hc2.data(), h2, (j + 1) * sizeof(double), cudaMemcpyDeviceToHost, stream), "gmres");
      double nn = 0.0;
      cuda_check(cudaMemcpyAsync(&nn, hn, sizeof(double), cudaMemcpyDeviceToHost, stream), "gmres");
      cuda_check(cudaStreamSynchronize(stream), "gmres");
      const double hj1 = std::sqrt(nn);
      if (!std::isfinite(hj1)) return DC_ERR_DIVERGED;
      double* col = &H[static_cast<size_t>(j) * (m + 1)];
      for (int i = 0; i <= j; ++i) col[i] = hc1[i] + hc2[i];
      col[j + 1] = hj1;
      if (hj1 > 0.0) gmres_scale_value<T>(vj1, vj1, n, 1.0 / hj1, stream);
      // previous rotations, then the one that zeroes col[j + 1]
      for (int i = 0; i < j; ++i) {
        const double t0 = cs[i] * col[i] + sn[i] * col[i + 1];
        col[i + 1] = -sn[i] * col[i] + cs[i] * col[i + 1];
        col[i] = t0;
      }
      const double den = std::hypot(col[j], col[j + 1]);
      cs[j] = den > 0.0 ? col[j] / den : 1.0;
      sn[j] = den > 0.0 ? col[j + 1] / den : 0.0;
      col[j] = den;
      col[j + 1] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      ++total;
      k = j + 1;
      if (std::fabs(g[j + 1]) <= target || hj1 == 0.0) break;
    }
    if (k == 0) break;
    // y = H^-1 g (upper triangular), x += M^-1 (V y)
    std::vector<double> y(k);
    for (int i = k - 1; i >= 0; --i) {
      double s = g[i];
      for (int l = i + 1; l < k; ++l) s -= H[static_cast<size_t>(l) * (m + 1) + i] * y[l];
      const double d = H[static_cast<size_t>(i) * (m + 1) + i];
      y[i] = d != 0.0 ? s / d : 0.0;
    }
    cuda_check(cudaMemcpyAsync(h1, y.data(), k * sizeof(double), cudaMemcpyHostToDevice, stream), "gmres");
    cuda_check(cudaMemsetAsync(u, 0, n * sizeof(T), stream), "memset");
    gmres_maxpy<T>(u, V, n, k, h1, 1.0, stream);
    precond(u, z);
    const double one = 1.0;
    cuda_check(cudaMemcpyAsync(h2, &one, sizeof(double), cudaMemcpyHostToDevice, stream), "gmres");
    gmres_maxpy<T>(x, z, n, 1, h2, 1.0, stream);
    // true residual of the restart
    apply_A(x, r);
    gmres_sub_from<T>(r, b, n, stream);
    beta = norm(r);
    if (!std::isfinite(beta)) return DC_ERR_DIVERGED;
    if (beta <= target) {
      *iters = total;
      return DC_OK;
    }
    if (total >= max_it) break;
  }
  *iters = total;
  return beta <= target ? DC_OK : DC_ERR_TIMEOUT;
}

namespace {
// Device share held by the single-launch solves in flight (all models of the process): a
// solve reserves its grid's slots before launching and returns them once its result has
// been read, waiting while they are taken.  Cooperative grids in flight together then
// always fit on the device at once, so no grid's barrier waits for blocks that cannot be
// scheduled; and every solve takes the single-launch path whatever else runs, so a
// simulation's results do not depend on the others.
class SlotBudget {
 public:
  void acquire(int slots, int capacity) {
    std::unique_lock<std::mutex> lk(m_);
    cv_.wait(lk, [&] { return used_ + slots <= capacity; });
    used_ += slots;
  }
  void release(int slots) {
    {
      std::lock_guard<std::mutex> lk(m_);
      used_ -= slots;
    }
    cv_.notify_all();
  }

 private:
  std::mutex m_;
  std::condition_variable cv_;
  long long used_ = 0;
};
SlotBudget g_slots;

struct SlotGuard {
  int slots;
  SlotGuard(int s, int capacity) : slots(s) { g_slots.acquire(s, capacity); }
  ~SlotGuard() { g_slots.release(slots); }
};
}  // namespace

// BiCGSTAB + block Jacobi as one cooperative launch (krylov_fused.cu).  Returns false, with
// nothing launched, when the device cannot run it; the caller then replays the graph of
// per-phase launches.
template <class T>
bool Solver::krylov_fused(double rel, int max_it, int* iters, int* status, const double* b64, double* z64) {
  constexpr bool f32 = std::is_same_v<T, float>;
  const bool sell = f32 && spmv_format == kSpmvSell;
  const Bsr A = model.bsr(J_.get(), J32_.get());
  int blocks = 0, slots = 0, capacity = 0;
  if (!fused_bicgstab_plan<T, T>(model.bs, sell, A.nrows, &blocks, &slots, &capacity)) return false;
  SlotGuard guard(slots, capacity);
  const int64_t np = fused_bicgstab_partials(blocks);
  if (static_cast<int64_t>(fpart_.size()) < np) fpart_.resize(np);
  FusedBicgArgs<T, T> a;
  a.nrows = A.nrows;
  a.rowptr = A.rowptr;
  a.colidx = A.colidx;
  if constexpr (f32) {
    a.vals = sell ? Js32_.get() : J32_.get();
    a.dinv = fdinv_.get();
    a.x = fx_.get(); a.r = fr_.get(); a.rhat = frhat_.get(); a.p = fp_.get(); a.v = fv_.get();
    a.s = fs_.get(); a.t = ft_.get(); a.phat = fphat_.get(); a.shat = fshat_.get();
    a.p2 = fp2_.get(); a.v2 = fv2_.get();
  } else {
    a.vals = J_.get();
    a.dinv = dinv_.get();
    a.x = kx_.get(); a.r = kr_.get(); a.rhat = krhat_.get(); a.p = kp_.get(); a.v = kv_.get();
    a.s = ks_.get(); a.t = kt_.get(); a.phat = kphat_.get(); a.shat = kshat_.get();
    a.p2 = nullptr; a.v2 = nullptr;  // the fp64 operator is BSR: five phases, one p and v
  }
  if (sell) a.S = model.sell();
  a.partial = fpart_.get();
  a.sc = scal_.get();
  a.rel = rel;
  a.max_it = max_it;
  if constexpr (f32) {
    if (b64) {
      // the fp64 iterative refinement of bicgstab_mixed, on the device
      a.b64 = b64;
      a.z64 = z64;
      a.r64 = kr_.get();
      a.vals64 = J_.get();
      a.inner = mixed_inner_;
      a.max_refinements = kMixedMaxRefinements;
    }
  }
  if (profiling_ && !fused_ev_[0])
    for (auto& e : fused_ev_) cuda_check(cudaEventCreate(&e), "cudaEventCreate");
  if (profiling_) cuda_check(cudaEventRecord(fused_ev_[0], stream), "cudaEventRecord");
  fused_bicgstab<T, T>(model.bs, sell, blocks, a, stream);
  if (profiling_) cuda_check(cudaEventRecord(fused_ev_[1], stream), "cudaEventRecord");
  double h[KS_COUNT];
  read_scalars(h, 0, KS_COUNT);
  if (h[KS_FAULT] != 0.0) throw std::runtime_error("single-launch BiCGSTAB: a grid-barrier wait timed out");
  *iters = static_cast<int>(h[KS_ITER]);
  if (b64) stats.refinements += static_cast<long long>(h[KS_REFINEMENTS]);
  if (profiling_) {
    float ms = 0.0f;
    cuda_check(cudaEventElapsedTime(&ms, fused_ev_[0], fused_ev_[1]), "cudaEventElapsedTime");
    kernel_times.ms[3] += ms;
    kernel_times.calls[3] += *iters;
  }
  *status = h[KS_DONE] == kDoneConverged ? DC_OK : (h[KS_DONE] == 0.0 ? DC_ERR_TIMEOUT : DC_ERR_DIVERGED);
  return true;
}

// Replays chunks of Krylov (BiCGSTAB or CG) iterations until the device flag reports
// convergence, breakdown or a non-finite value, or max_it iterations have run.  r (kr_ /
// fr_) holds the right-hand side on entry; the solution is left in the Krylov x vector.
int Solver::krylov_run(bool fp32, double rel, int max_it, int* iters) {
  if (krylov_gmres_) return fp32 ? gmres_t<float>(rel, max_it, iters) : gmres_t<double>(rel, max_it, iters);
  if (batch_) {
    int st = DC_OK;
    if (batch_solve(fp32, rel, max_it, iters, &st)) return st;
  }
  if (fused_ && !krylov_cg_ && !pc_) {
    int st = DC_OK;
    if (fp32 ? krylov_fused<float>(rel, max_it, iters, &st) : krylov_fused<double>(rel, max_it, iters, &st))
      return st;
  }
  double* sc = scal_.get();
  const int64_t n = n_;
  const Bsr A = model.bsr(J_.get(), J32_.get());
  const Preconditioner* pc = pc_;
  if (fp32) {
    KrylovVectors<float> kv{fx_.get(), fr_.get(), frhat_.get(), fp_.get(), fv_.get(), fs_.get(), ft_.get(),
                            fphat_.get(), fshat_.get()};
    if (krylov_cg_) cg_init<float, float>(A, fdinv_.get(), kv, rel, rs_, sc, stream, pc);
    else krylov_init<float>(kv, n, rel, rs_, sc, stream);
  } else {
    KrylovVectors<double> kv{kx_.get(), kr_.get(), krhat_.get(), kp_.get(), kv_.get(), ks_.get(), kt_.get(),
                             kphat_.get(), kshat_.get()};
    if (krylov_cg_) cg_init<double, double>(A, dinv_.get(), kv, rel, rs_, sc, stream, pc);
    else krylov_init<double>(kv, n, rel, rs_, sc, stream);
  }
  cudaGraphExec_t exec = krylov_graph(fp32);
  double h[KS_COUNT];
  read_scalars(h, 0, KS_COUNT);
  int it = 0;
  while (h[KS_DONE] == 0.0 && it < max_it) {
    cuda_check(cudaGraphLaunch(exec, stream), "cudaGraphLaunch");
    count_launches(static_cast<long long>(launches_per_iter_) * kKrylovChunk);
    read_scalars(h, 0, KS_COUNT);
    const int now = static_cast<int>(h[KS_ITER]);
    if (profiling_) {
      for (int k = 0; k < now - it && k < kKrylovChunk; ++k)
        for (int pair = 0; pair < 2; ++pair) {
          float ms = 0.0f;
          // profiling is best effort: an unreadable event pair is skipped
          if (cudaEventElapsedTime(&ms, graph_events_[4 * k + 2 * pair], graph_events_[4 * k + 2 * pair + 1]) ==
              cudaSuccess) {
            kernel_times.ms[1] += ms;
            kernel_times.calls[1] += 1;
          } else {
            cudaGetLastError();
          }
        }
    }
    it = now;
  }
  *iters = it;
  if (h[KS_DONE] == kDoneConverged) return DC_OK;
  if (h[KS_DONE] == 0.0) return DC_ERR_TIMEOUT;
  return DC_ERR_DIVERGED;
}

// BiCGSTAB + block Jacobi in the batch shared with the other simulations of a server: the
// right-hand side in kr_ / fr_, the solution left in kx_ / fx_, as krylov_run.  The fp64
// operator is copied into the SELL-32 layout first (the batch reads that layout only).
bool Solver::batch_solve(bool fp32, double rel, int max_it, int* iters, int* status) {
  if (krylov_cg_ || krylov_gmres_ || pc_ || model.bs > 8) return false;
  const Sell S = model.sell();
  if (fp32) {
    if (Js32_.size() == 0 || spmv_format != kSpmvSell) return false;
    BatchSystem<float> y;
    y.nrows = static_cast<int>(model.nnodes);
    y.bs = model.bs;
    y.S = S;
    y.vals = Js32_.get();
    y.dinv = fdinv_.get();
    y.x = fx_.get(); y.r = fr_.get(); y.rhat = frhat_.get(); y.p = fp_.get(); y.v = fv_.get();
    y.s = fs_.get(); y.t = ft_.get(); y.phat = fphat_.get(); y.shat = fshat_.get();
    *status = batch_->solve(y, stream, rel, max_it, iters);
  } else {
    const size_t nv = static_cast<size_t>(model.sell_slots) * 32 * model.bs * model.bs;
    if (Js64_.size() != nv) Js64_.resize(nv);
    bsr_to_sell64(model.bsr(J_.get(), nullptr), J_.get(), S, Js64_.get(), stream);
    BatchSystem<double> y;
    y.nrows = static_cast<int>(model.nnodes);
    y.bs = model.bs;
    y.S = S;
    y.vals = Js64_.get();
    y.dinv = dinv_.get();
    y.x = kx_.get(); y.r = kr_.get(); y.rhat = krhat_.get(); y.p = kp_.get(); y.v = kv_.get();
    y.s = ks_.get(); y.t = kt_.get(); y.phat = kphat_.get(); y.shat = kshat_.get();
    *status = batch_->solve(y, stream, rel, max_it, iters);
  }
  // the codes of the batch are those of the replayed solve: 0 converged, 1 breakdown / not
  // finite, 3 max_it
  *status = *status == 0 ? DC_OK : (*status == 3 ? DC_ERR_TIMEOUT : DC_ERR_DIVERGED);
  return true;
}

int Solver::bicgstab(const double* b, double* z, double rel_tol, int max_it, int* iters) {
  cuda_check(cudaMemcpyAsync(kr_.get(), b, n_ * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
  int st = krylov_run(false, rel_tol, max_it, iters);
  cuda_check(cudaMemcpyAsync(z, kx_.get(), n_ * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
  return st;
}

// fp32 BiCGSTAB on the correction equation inside fp64 iterative refinement:
//   r = b - J z (fp64);  solve J d = r in fp32 to a modest reduction;  z += d
int Solver::bicgstab_mixed(const double* b, double* z, double rel_tol, int max_it, int* iters) {
  // BiCGSTAB + block Jacobi: the whole refinement loop below in one cooperative launch
  // (batched solvers run the loop below, each correction solve in the batch)
  if (fused_ && !batch_ && !krylov_cg_ && !krylov_gmres_ && !pc_) {
    int st = DC_OK;
    if (krylov_fused<float>(rel_tol, max_it, iters, &st, b, z)) return st;
  }
  Bsr A = model.bsr(J_.get(), J32_.get());
  const int64_t n = n_;
  cuda_check(cudaMemsetAsync(z, 0, n * sizeof(double), stream), "memset");
  const double b0 = std::sqrt(norm2(b));
  *iters = 0;
  if (b0 == 0.0) return DC_OK;
  if (!std::isfinite(b0)) return DC_ERR_DIVERGED;
  const double target = rel_tol * b0;
  // with the multigrid, whose fp32 corrections converge in few iterations, coarser
  // corrections and more fp64 refinements take fewer iterations in all (measured on the
  // two-compartment system: 68-74 against 80-100 per step)
  const double inner_red =
      (!inner_set_ && amg_ && pc_ == amg_.get()) ? kMixedInnerReductionMultigrid : mixed_inner_;
  double rn = b0;
  int total = 0;
  for (int ref = 0; ref < kMixedMaxRefinements && total < max_it; ++ref) {
    // fp64 refinement residual r = b - J z (skip the SpMV for z = 0)
    if (ref == 0) {
      cuda_check(cudaMemcpyAsync(kr_.get(), b, n * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
    } else {
      residual(A, z, b, kr_.get(), stream);
      rn = std::sqrt(norm2(kr_.get()));
      if (!std::isfinite(rn)) return DC_ERR_DIVERGED;
      if (rn <= target) {
        *iters = total;
        return DC_OK;
      }
    }
    ++stats.refinements;
    // scale into fp32 range and solve the correction equation in fp32
    to_float_scaled(n, kr_.get(), 1.0 / rn, fr_.get(), stream);
    int it = 0;
    const int st = krylov_run(true, std::max(inner_red, 0.5 * target / rn), max_it - total, &it);
    total += it;
    if (st == DC_ERR_DIVERGED && it == 0) return DC_ERR_DIVERGED;
    add_float_scaled(n, fx_.get(), rn, z, stream);
  }
  residual(A, z, b, kr_.get(), stream);
  rn = std::sqrt(norm2(kr_.get()));
  *iters = total;
  return rn <= target ? DC_OK : DC_ERR_TIMEOUT;
}

// J v at the stored linearisation point, element by element (matrix-free mode)
void Solver::jacobian_apply_mf(const double* v, double* y) {
  tbegin(1);
  model.jacobian_apply(mf_x_.get(), mf_t_, mf_cm_, mf_ca_, v, y, stream);
  tend();
}

// Krylov solve without a matrix (linear_solver.matrix_free = true): every product is
// jacobian_apply_mf, the preconditioner is Richardson (the only matrix-free entries of the
// reference's registry are Richardson and InverseOperator, preconditioner.hh:94-95).  BiCGSTAB
// (and the aliases that run as it) or CG, in fp64, the scalars read back each iteration;
// GMRES runs gmres_t with the same product.  Right-hand side b, solution z.
int Solver::krylov_mf(const double* b, double* z, double rel, int max_it, int* iters) {
  const int64_t n = n_;
  *iters = 0;
  if (krylov_gmres_) {
    cuda_check(cudaMemcpyAsync(kr_.get(), b, n * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
    const int st = gmres_t<double>(rel, max_it, iters);
    cuda_check(cudaMemcpyAsync(z, kx_.get(), n * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
    return st;
  }
  if (gh_.size() < 8) gh_.resize(8);
  if (gpart_.size() < static_cast<size_t>(kGmresBlocks) * 2) gpart_.resize(static_cast<size_t>(kGmresBlocks) * 2);
  double* hd = gh_.get();
  auto dotp = [&](const double* a, const double* c) {
    gmres_mdot<double>(a, n, 1, c, hd, gpart_.get(), false, stream);
    double h = 0.0;
    cuda_check(cudaMemcpyAsync(&h, hd, sizeof(double), cudaMemcpyDeviceToHost, stream), "krylov");
    cuda_check(cudaStreamSynchronize(stream), "krylov");
    return h;
  };
  auto precond = [&](const double* in, double* out) { pc_->apply(in, out, nullptr, 0, stream); };
  double* x = z;
  double* r = kr_.get();
  double* rt = krhat_.get();
  double* p = kp_.get();
  double* v = kv_.get();
  double* y = kphat_.get();
  double* zz = kshat_.get();
  double* t = kt_.get();
  cuda_check(cudaMemsetAsync(x, 0, n * sizeof(double), stream), "memset");
  cuda_check(cudaMemcpyAsync(r, b, n * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
  const double r0 = std::sqrt(dotp(r, r));
  if (r0 == 0.0) return DC_OK;
  if (!std::isfinite(r0)) return DC_ERR_DIVERGED;
  const double target = rel * r0;
  if (krylov_cg_) {
    // preconditioned CG: p = y = M^-1 r, q = A p in v
    precond(r, y);
    cuda_check(cudaMemcpyAsync(p, y, n * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
    double rho = dotp(r, y);
    for (int it = 1; it <= max_it; ++it) {
      jacobian_apply_mf(p, v);
      const double pq = dotp(p, v);
      if (pq == 0.0 || !std::isfinite(pq)) return DC_ERR_DIVERGED;
      const double alpha = rho / pq;
      axpy(n, alpha, p, x, stream);
      axpy(n, -alpha, v, r, stream);
      *iters = it;
      const double rn = std::sqrt(dotp(r, r));
      if (!std::isfinite(rn)) return DC_ERR_DIVERGED;
      if (rn <= target) return DC_OK;
      precond(r, y);
      const double rho_new = dotp(r, y);
      axpby(n, 1.0, y, rho_new / rho, p, stream);
      rho = rho_new;
    }
    return DC_ERR_TIMEOUT;
  }
  // BiCGSTAB (dune-istl BiCGSTABSolver's recurrences)
  cuda_check(cudaMemcpyAsync(rt, r, n * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
  cuda_check(cudaMemsetAsync(p, 0, n * sizeof(double), stream), "memset");
  cuda_check(cudaMemsetAsync(v, 0, n * sizeof(double), stream), "memset");
  double rho = 1.0, alpha = 1.0, omega = 1.0;
  for (int it = 1; it <= max_it; ++it) {
    const double rho_new = dotp(rt, r);
    if (rho_new == 0.0 || !std::isfinite(rho_new)) return DC_ERR_DIVERGED;
    const double beta = (rho_new / rho) * (alpha / omega);
    // p = r + beta (p - omega v)
    axpy(n, -omega, v, p, stream);
    axpby(n, 1.0, r, beta, p, stream);
    precond(p, y);
    jacobian_apply_mf(y, v);
    const double rtv = dotp(rt, v);
    if (rtv == 0.0 || !std::isfinite(rtv)) return DC_ERR_DIVERGED;
    alpha = rho_new / rtv;
    axpy(n, -alpha, v, r, stream);  // r = s
    axpy(n, alpha, y, x, stream);
    *iters = it;
    double rn = std::sqrt(dotp(r, r));
    if (!std::isfinite(rn)) return DC_ERR_DIVERGED;
    if (rn <= target) return DC_OK;
    precond(r, zz);
    jacobian_apply_mf(zz, t);
    const double tt = dotp(t, t);
    if (tt == 0.0 || !std::isfinite(tt)) return DC_ERR_DIVERGED;
    omega = dotp(t, r) / tt;
    axpy(n, omega, zz, x, stream);
    axpy(n, -omega, t, r, stream);
    rn = std::sqrt(dotp(r, r));
    if (!std::isfinite(rn)) return DC_ERR_DIVERGED;
    if (rn <= target) return DC_OK;
    if (omega == 0.0) return DC_ERR_DIVERGED;
    rho = rho_new;
  }
  return DC_ERR_TIMEOUT;
}

int Solver::linear_solve(const double* b, double* z, double rel_tol, int* iters) {
  if (matrix_free_) {
    int it = 0;
    const int st = krylov_mf(b, z, rel_tol, lin_max_it_, &it);
    stats.linear_iterations += it;
    ++stats.linear_solves;
    if (iters) *iters = it;
    return st;
  }
  setup_preconditioner();
  int it = 0;
  // preconditioner "auto": block Jacobi gets auto_threshold iterations; a system that needs
  // more (stiff) switches this model to the multigrid and the solve starts over with it
  const bool trial = auto_pc_ && !amg_->built();
  const int max_it = trial ? std::min(lin_max_it_, auto_threshold_) : lin_max_it_;
  int st = mixed_precision ? bicgstab_mixed(b, z, rel_tol, max_it, &it) : bicgstab(b, z, rel_tol, max_it, &it);
  check_setup_status();
  stats.linear_iterations += it;
  ++stats.linear_solves;
  if (trial && st != DC_OK) {
    build_multigrid();
    int it2 = 0;
    st = linear_solve(b, z, rel_tol, &it2);
    it += it2;
  }
  if (iters) *iters = it;
  return st;
}

void Solver::linear_step(double* x, const ResFn& resjac) {
  // make_step_operator.hh:210-245: b = F(x); solve J z = b; x -= z
  resjac(x, r_.get());
  int it = 0;
  // a linear model's stage solution is this one solve, with no Newton iteration after it to
  // absorb the solve's error: direct-solve semantics here keep the near-machine-precision
  // reduction
  const double tol = lin_direct_ ? std::min(direct_tol_, 1e-13) : lin_rel_;
  int st = linear_solve(r_.get(), z_.get(), tol, &it);
  if (st != DC_OK) throw StepFailure("linear solver did not converge");
  axpy(n_, -1.0, z_.get(), x, stream);
}

void Solver::newton(double* x, const ResFn& res, const JacFn& jac, const ResFn& resjac) {
  auto norm = [&](const double* v) -> double {
    if (norm_ == "l_2") return norm2(v);  // two_norm2: the SQUARED norm (make_step_operator.hh:274-276)
    std::vector<double> h(n_);
    cuda_check(cudaMemcpyAsync(h.data(), v, n_ * sizeof(double), cudaMemcpyDeviceToHost, stream), "norm");
    cuda_check(cudaStreamSynchronize(stream), "norm");
    double acc = 0.0;
    for (double e : h) acc = (norm_ == "l_inf") ? std::max(acc, std::fabs(e)) : acc + std::fabs(e);
    return acc;
  };
  // the first iterate always needs its Jacobian (unless it already satisfies the test):
  // residual and Jacobian come from one assembly pass there
  resjac(x, r_.get());
  bool jac_at_x = true;
  double defect = norm(r_.get());
  const double first = defect;
  double prev = defect;
  int it = 0;
  bool have_jac = true;
  while (true) {
    if (!std::isfinite(defect)) throw StepFailure("Newton defect is not finite");
    if (it >= it_min_ && (defect <= newton_abs_ || defect < first * newton_rel_ || defect == 0.0)) break;
    if (it >= it_max_) throw StepFailure("Newton did not converge within the iteration range", DC_ERR_DIVERGED);
    if (!jac_at_x && (!have_jac || lin_threshold_ <= 0.0 || !(prev > 0.0 && defect / prev < lin_threshold_))) {
      jac(x);
      have_jac = true;
    }
    jac_at_x = false;
    double red;
    if (lin_direct_) {
      red = direct_tol_;
    } else if (dx_fixed_) {
      red = dx_min_rel_;
    } else {
      const double stop = std::max(first * newton_rel_, newton_abs_);
      const double q = (prev > 0.0) ? (defect * defect) / (prev * prev) : 1.0;
      if (stop / (10.0 * defect) > q) red = stop / (10.0 * defect);
      else red = std::min(dx_min_rel_, q);
    }
    int lit = 0;
    int st = linear_solve(r_.get(), z_.get(), red, &lit);
    if (st != DC_OK) throw StepFailure("linear solver did not converge");
    axpy(n_, -1.0, z_.get(), x, stream);
    prev = defect;
    res(x, r_.get());
    defect = norm(r_.get());
    ++it;
  }
  stats.newton_iterations += it;
  stats.last_newton = it;
  stats.step_stage_newton.push_back(it);
}

void Solver::one_step(double dt) {
  const RKTable tab = RKTable::make(scheme_);
  const int s = static_cast<int>(tab.A.size());
  if (static_cast<int>(us_.size()) < s + 1) {
    us_.resize(s + 1);
    for (auto& u : us_) if (u.size() != static_cast<size_t>(n_)) u.resize(n_);
  }
  const double t = t_;
  std::vector<double> ts(s + 1);
  for (int j = 0; j <= s; ++j) ts[j] = t + tab.D[j] * dt;
  cuda_check(cudaMemcpyAsync(us_[0].get(), x_.get(), n_ * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
  cuda_check(cudaMemcpyAsync(stage_.get(), x_.get(), n_ * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
  // Split residual: with a purely static mass form, the stage residual is
  // const + (a Ms + b dt Ks) y + b dt D(y), D the state-dependent stiffness terms.  D of the
  // last evaluated state is kept (dyn_): a stage's Newton ends with a residual at its
  // solution, so the next stage's explicit term and its first residual (the stage starts
  // from that solution) take D from there instead of another volume pass, and so does the
  // first residual of the next step.  D depends on the time only through programs that
  // read it; those models reuse it at the same time only.
  const bool split = split_residual_;
  auto dyn_reusable = [&](double at) { return dyn_valid_ && (!model.dynamic_time || dyn_t_ == at); };
  for (int i = 1; i <= s; ++i) {
    const auto& a = tab.A[i - 1];
    const auto& b = tab.B[i - 1];
    // explicit part of the stage residual, fixed during the Newton solve
    cuda_check(cudaMemsetAsync(const_.get(), 0, n_ * sizeof(double), stream), "memset");
    for (int j = 0; j < i; ++j) {
      if (a[j] == 0.0 && b[j] == 0.0) continue;
      if (split && j == i - 1 && dyn_reusable(ts[j])) {
        // the previous stage's solution: its D is the one kept from that stage's last residual
        model.assemble(us_[j].get(), ts[j], a[j], b[j] * dt, const_.get(), nullptr, 1 | Model::kAssembleStaticOnly,
                       stream);
        if (b[j] != 0.0) axpy(n_, b[j] * dt, dyn_.get(), const_.get(), stream);
        continue;
      }
      tbegin(0);
      model.assemble(us_[j].get(), ts[j], a[j], b[j] * dt, const_.get(), nullptr, 1, stream);
      tend();
      ++stats.assemblies;
    }
    const double ai = a[i], bi = b[i] * dt, ti = ts[i];
    // the stage starts from the previous stage's solution (or the step's start state), whose
    // D may be kept
    bool reuse_first = split && dyn_reusable(ti);
    auto res = [&](const double* y, double* r) {
      cuda_check(cudaMemcpyAsync(r, const_.get(), n_ * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
      if (split) {
        model.assemble(y, ti, ai, bi, r, nullptr, 1 | Model::kAssembleStaticOnly, stream);
        if (!reuse_first) {
          cuda_check(cudaMemsetAsync(dyn_.get(), 0, n_ * sizeof(double), stream), "memset");
          tbegin(0);
          model.assemble(y, ti, 0.0, 1.0, dyn_.get(), nullptr, 1 | Model::kAssembleDynamicOnly, stream);
          tend();
          ++stats.assemblies;
          dyn_t_ = ti;
        }
        reuse_first = false;
        dyn_valid_ = true;
        if (bi != 0.0) axpy(n_, bi, dyn_.get(), r, stream);
      } else {
        tbegin(0);
        model.assemble(y, ti, ai, bi, r, nullptr, 1, stream);
        tend();
        ++stats.assemblies;
      }
      model.constrain_residual(r, stream);
    };
    // mixed precision inside Newton: the state-dependent Jacobian terms in fp32 (the
    // Jacobian only steers the Newton correction; the residual, the static part and the
    // refinement stay fp64).  A linear model's single solve is its stage solution, so it
    // keeps the fp64 Jacobian.
    const int jmode = Model::kAssembleOverwriteJacobian |
                      ((mixed_precision && jac_f32_ && !model.is_linear) ? Model::kAssembleJacobianF32 : 0);
    auto finish_jac = [&]() {
      if (model.padded)
        launch_pad_identity(model.d_diag.get(), model.d_row_ns.get(), static_cast<int>(model.nnodes), model.bs,
                            J_.get(), 1.0, stream);
      model.constrain_jacobian(J_.get(), stream);
    };
    auto jac = [&](const double* y) {
      if (matrix_free_) {
        // linear_solver.matrix_free: no matrix; the Krylov solve's products J v are evaluated
        // element by element at this linearisation point
        cuda_check(cudaMemcpyAsync(mf_x_.get(), y, n_ * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
        mf_t_ = ti;
        mf_cm_ = ai;
        mf_ca_ = bi;
        return;
      }
      tbegin(4);
      jac_sell_fresh_ = model.assemble(y, ti, ai, bi, nullptr, J_.get(), 2 | jmode, stream, jac_sell_target());
      tend();
      finish_jac();
      ++stats.assemblies;
    };
    auto resjac = [&](const double* y, double* r) {
      if (split || matrix_free_) {
        // the residual (possibly from the kept D) and the Jacobian as separate passes
        res(y, r);
        jac(y);
        return;
      }
      cuda_check(cudaMemcpyAsync(r, const_.get(), n_ * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
      tbegin(5);
      jac_sell_fresh_ = model.assemble(y, ti, ai, bi, r, J_.get(), 3 | jmode, stream, jac_sell_target());
      tend();
      model.constrain_residual(r, stream);
      finish_jac();
      stats.assemblies += 2;
    };
    // constrained entries take their values before the stage solve; zero residual rows and
    // unit Jacobian rows keep them there
    model.apply_constraints(stage_.get(), stream);
    if (model.is_linear) linear_step(stage_.get(), resjac);
    else newton(stage_.get(), res, jac, resjac);
    cuda_check(cudaMemcpyAsync(us_[i].get(), stage_.get(), n_ * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
  }
  cuda_check(cudaMemcpyAsync(x_.get(), stage_.get(), n_ * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
  cuda_check(cudaStreamSynchronize(stream), "step");
  tflush();
}

int Solver::do_step(double& dt, double* dt_used) {
  auto check = [&](double d) {
    if (has_min_ && f_lt(std::fabs(d), std::fabs(dt_min_))) return false;
    if (has_max_ && f_gt(std::fabs(d), std::fabs(dt_max_))) return false;
    return true;
  };
  stats.step_stage_newton.clear();
  if (!check(dt)) return DC_ERR_DT_MIN;
  // Without time_step_min the reference keeps halving until dt underflows; here a step
  // gives up after kMaxRejections consecutive rejections (dt reduced by dec^60 ~ 1e-18).
  constexpr int kMaxRejections = 60;
  int rejections = 0;
  while (true) {
    try {
      one_step(dt);
      break;
    } catch (const StepFailure&) {
      // the kept state-dependent residual belongs to a state of the failed attempt
      dyn_valid_ = false;
      ++stats.failed_steps;
      // the state of the step's start is kept (x_ is only overwritten on success)
      dt = dt * dec_;
      if (!check(dt) || ++rejections >= kMaxRejections || dt == 0.0) return DC_ERR_DT_MIN;
    }
  }
  if (dt_used) *dt_used = dt;
  t_ = t_ + dt;
  ++stats.steps;
  double nd = dt * inc_;
  if (has_max_) nd = std::clamp(nd, -std::fabs(dt_max_), std::fabs(dt_max_));
  dt = nd;
  return DC_OK;
}

int Solver::evolve(double t_end, double& dt, const std::function<void(double)>& cb) {
  while (f_le(t_ + 2.0 * dt, t_end)) {
    int st = do_step(dt);
    if (st != DC_OK) return st;
    if (cb) cb(t_);
  }
  int snap = 0;
  while (f_lt(t_, t_end)) {
    const int k = static_cast<int>(std::ceil((t_end - t_) / dt));
    if (k <= 0) return DC_ERR_INTERNAL;
    dt = (t_end - t_) / k;
    int st = do_step(dt);
    if (st == DC_OK) {
      if (cb) cb(t_);
    } else {
      if (snap == 100) return st;
      ++snap;
      dt *= 0.5;
    }
  }
  return DC_OK;
}

}  // namespace dcgpu
