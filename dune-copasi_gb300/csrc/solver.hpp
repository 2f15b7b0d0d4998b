// Time stepping on the device: Runge-Kutta stages, Newton, preconditioned BiCGSTAB.
//
// Restates, for the GPU:
//   * the Runge-Kutta one-step operator of dune/copasi/model/make_step_operator.hh:408-443
//     (PDELab one-step parameter tables: ImplicitEuler, Alexander2 (default), ...);
//   * the Newton configuration of make_step_operator.hh:246-288 (relative tolerance on the
//     SQUARED l2 norm by default, iteration range {0,40}, linearization threshold, adaptive
//     linear tolerance) and the linear defect-correction branch :210-245;
//   * the LinearSolver of make_step_operator.hh:102-146, with the dune-istl Krylov solve
//     replaced by a device BiCGSTAB (block-Jacobi preconditioned; fp64, or fp32 inside
//     fp64 iterative refinement);
//   * SimpleAdaptiveStepper::do_step and TimeStepper::evolve / snap_to_time
//     (dune/copasi/common/stepper.hh:95-239, 337-368).
#pragma once

#include <functional>
#include <memory>
#include <string>
#include <vector>

#include "amg.hpp"
#include "mcolor.hpp"
#include "precond.hpp"
#include "krylov.cuh"
#include "model.hpp"

namespace dcgpu {

class KrylovBatcher;

enum Status : int {
  DC_OK = 0,
  DC_ERR_DIVERGED = 1,     // Newton / linear solve did not converge
  DC_ERR_DT_MIN = 2,       // time step reached its lower limit
  DC_ERR_TIMEOUT = 3,      // iteration cap hit
  DC_ERR_CONFIG = 4,
  DC_ERR_CUDA = 5,
  DC_ERR_ARGUMENT = 6,
  DC_ERR_INTERNAL = 7,
};

struct RKTable {
  std::vector<std::vector<double>> A, B;
  std::vector<double> D;
  static RKTable make(const std::string& name);
};

struct SolverStats {
  long newton_iterations = 0;
  long linear_iterations = 0;
  long linear_solves = 0;
  long assemblies = 0;
  long failed_steps = 0;
  long steps = 0;
  long refinements = 0;
  int last_newton = 0;
  // Newton iterations of every stage solve of the last do_step, in order (stages of
  // rejected attempts included; a stage whose Newton failed adds nothing)
  std::vector<int> step_stage_newton;
};

class StepFailure : public std::runtime_error {
 public:
  explicit StepFailure(const std::string& w, int code = DC_ERR_DIVERGED) : std::runtime_error(w), code(code) {}
  int code;
};

class Solver {
 public:
  explicit Solver(Model& m, cudaStream_t stream = nullptr);
  ~Solver();
  Solver(const Solver&) = delete;
  Solver& operator=(const Solver&) = delete;

  // state (reference DOF order on the host)
  void set_state(const std::vector<double>& ref, double t);
  void set_state(const double* ref, int64_t n, double t);  // reference DOF layout, host memory
  std::vector<double> get_state() const;
  void get_state(double* out, int64_t n) const;             // reference DOF layout, host memory
  double time() const { return t_; }
  const double* state_device() const { return x_.get(); }  // blocked state
  const double* device_state() const { return x_.get(); }
  double* device_state() { return x_.get(); }

  // one Runge-Kutta step from (x, t) with dt, result in x on success; throws StepFailure
  void one_step(double dt);
  // SimpleAdaptiveStepper::do_step; returns status, updates dt to the suggested next dt
  int do_step(double& dt, double* dt_used = nullptr);
  // TimeStepper::evolve (snap to end time); callback after each successful step
  int evolve(double t_end, double& dt, const std::function<void(double)>& cb);

  // linear algebra entry points for tests
  int linear_solve(const double* b, double* z, double rel_tol, int* iters);
  double* jacobian_values() { return J_.get(); }
  double* residual_buffer() { return r_.get(); }

  void enable_mixed(bool on);
  // Hands this solver's block-Jacobi BiCGSTAB solves (fp64, and the fp32 corrections of the
  // mixed path) to a batcher shared with other simulations (batch.hpp).  Solves with
  // another Krylov method or preconditioner, or with the fp32 operator in the BSR layout,
  // stay on this solver's own stream.  Call before the first step; b outlives the solver.
  void attach_batcher(KrylovBatcher* b) { batch_ = b; }

  // per-category device time of the hot launches, measured with CUDA events on the
  // solver's stream: 0 = assembly (all colour launches of one operator evaluation),
  // 1 = SpMV (fp64 and fp32), 2 = preconditioner apply,
  // 3 = single-launch BiCGSTAB solves, whose `calls` count the Krylov ITERATIONS they ran
  // 0 = residual-only assembly passes, 1 = SpMV, 2 = preconditioner, 3 = single-launch
  // BiCGSTAB iterations, 4 = Jacobian-only assembly passes, 5 = combined residual + Jacobian
  // assembly passes
  static constexpr int kTimerCategories = 6;
  struct KernelTimes {
    double ms[kTimerCategories] = {};
    long long calls[kTimerCategories] = {};
  };
  void enable_profiling(bool on);
  KernelTimes kernel_times;

  SolverStats stats;
  Model& model;
  bool mixed_precision = false;
  cudaStream_t stream;

 private:
  // res: residual at y; jac: Jacobian at y; resjac: both in one assembly pass
  using ResFn = std::function<void(const double*, double*)>;
  using JacFn = std::function<void(const double*)>;
  void newton(double* x, const ResFn& res, const JacFn& jac, const ResFn& resjac);
  void linear_step(double* x, const ResFn& resjac);
  bool jac_f32_ = true;  // mixed precision: state-dependent Jacobian terms in fp32
  void setup_preconditioner();
  static constexpr int kKrylovChunk = 8;   // BiCGSTAB iterations per graph replay
  cudaGraphExec_t graphs_[4] = {nullptr, nullptr, nullptr, nullptr};  // {fp64, fp32} x {plain, profiled}
  std::vector<cudaEvent_t> graph_events_;
  cudaGraphExec_t krylov_graph(bool fp32);
  int krylov_run(bool fp32, double rel, int max_it, int* iters);
  // the solve of krylov_run through the batcher; false (nothing done) when it does not apply
  bool batch_solve(bool fp32, double rel, int max_it, int* iters, int* status);
  KrylovBatcher* batch_ = nullptr;
  DeviceBuffer<double> Js64_;  // fp64 SELL-32 copy of J for the batched fp64 solve
  int bicgstab(const double* b, double* z, double rel_tol, int max_it, int* iters);
  int bicgstab_mixed(const double* b, double* z, double rel_tol, int max_it, int* iters);
  double norm2(const double* v);
  double read_scalar(int slot);
  void read_scalars(double* out, int first, int count);

  struct PendingTiming {
    int cat;
    cudaEvent_t a, b;
  };
  bool profiling_ = false;
  std::vector<cudaEvent_t> event_pool_;
  std::vector<PendingTiming> pending_;
  void tbegin(int cat);
  void tend();
  void tflush();  // call after the stream has been synchronised

  int64_t n_ = 0;          // padded vector length
  double t_ = 0.0;
  DeviceBuffer<double> x_, r_, J_, stage_, const_, z_;
  // split stage residual (see one_step): the state-dependent stiffness residual D of the
  // last evaluated state, the time it was evaluated at, and whether it belongs to stage_
  bool split_residual_ = false;
  DeviceBuffer<double> dyn_;
  bool dyn_valid_ = false;
  double dyn_t_ = 0.0;
  mutable DeviceBuffer<double> ref_stage_;  // reference-layout staging vector of set/get_state
  std::vector<DeviceBuffer<double>> us_;
  // Krylov workspace
  DeviceBuffer<double> kr_, krhat_, kp_, kv_, ks_, kt_, kphat_, kshat_, kx_, dinv_;
  DeviceBuffer<float> fr_, frhat_, fp_, fv_, fs_, ft_, fphat_, fshat_, fx_, fdinv_, fb_;
  DeviceBuffer<float> fp2_, fv2_;  // second p / v of the three-phase single-launch solve
  DeviceBuffer<float> J32_;
  DeviceBuffer<float> Js32_;  // fp32 operator in the SELL-32 layout
  bool jac_sell_fresh_ = false;  // the last Jacobian assembly also wrote Js32_
  float* jac_sell_target() {
    return mixed_precision && spmv_format != kSpmvBsr && Js32_.size() > 0 ? Js32_.get() : nullptr;
  }
  DeviceBuffer<double> partial_, scal_;
  DeviceBuffer<unsigned int> counter_;
  DeviceBuffer<int> status_;
  double* pinned_ = nullptr;
  int* pinned_status() { return reinterpret_cast<int*>(pinned_ + 32); }
  bool setup_status_pending_ = false;  // a block-Jacobi status copy awaits check_setup_status
  void check_setup_status();
  ReduceScratch rs_{};

  // configuration
  std::string scheme_;
  double newton_rel_ = 1e-4, newton_abs_ = 0.0, lin_threshold_ = 0.0, dx_min_rel_ = 0.1;
  bool dx_fixed_ = false;
  int it_min_ = 0, it_max_ = 40;
  std::string norm_ = "l_2";
  double lin_rel_ = 1e-4;
  bool lin_direct_ = true;
  bool krylov_cg_ = false;        // preconditioned CG instead of BiCGSTAB
  bool krylov_gmres_ = false;     // restarted GMRES (right-preconditioned) instead of BiCGSTAB
  int gmres_restart_ = 40;
  DeviceBuffer<double> gV_, gh_, gpart_;
  DeviceBuffer<float> gV32_;
  template <class T>
  int gmres_t(double rel, int max_it, int* iters);
  int launches_per_iter_ = 5;     // kernels of one captured Krylov iteration
  // single-launch BiCGSTAB (cooperative kernel) whenever the device supports it; the
  // graph-replayed per-phase iteration otherwise, or with linear_solver.single_launch = false
  bool fused_ = true;
  DeviceBuffer<double> fpart_;
  cudaEvent_t fused_ev_[2] = {nullptr, nullptr};
  // with b64 / z64 (fp32 only): the mixed-precision refinement loop solving J z = b64, in the
  // same launch
  template <class T>
  bool krylov_fused(double rel, int max_it, int* iters, int* status, const double* b64 = nullptr,
                    double* z64 = nullptr);
  // mixed precision: relative reduction asked of each fp32 correction, and the cap on
  // corrections per solve
  static constexpr double kMixedInnerReduction = 1e-4;
  static constexpr double kMixedInnerReductionMultigrid = 1e-2;  // default with the multigrid
  double mixed_inner_ = kMixedInnerReduction;  // linear_solver.inner_reduction
  bool inner_set_ = false;                     // the key was given
  static constexpr int kMixedMaxRefinements = 50;
  double direct_tol_ = 1e-10;
  int lin_max_it_ = 500;
  std::string precond_ = "Jacobi";
  // a preconditioner applied by its own launches (null: block Jacobi, fused into the
  // Krylov kernels); it reads the BSR operator, in fp32 as well with mixed precision
  const Preconditioner* pc_ = nullptr;
  std::unique_ptr<Amg> amg_;
  std::unique_ptr<ColorPrecond> mc_;
  RichardsonPrecond rich_;
  DeviceBuffer<int32_t> row_group_;  // compartment of every block row (multigrid)
  void configure_preconditioner(const Ini& ls);
  void build_multigrid();
  void graphs_invalidate();
  // matrix-free mode: linearisation point of the last Jacobian request (state, time, mass
  // and stiffness scales) and the products at it
  bool matrix_free_ = false;
  DeviceBuffer<double> mf_x_;
  double mf_t_ = 0.0, mf_cm_ = 0.0, mf_ca_ = 0.0;
  void jacobian_apply_mf(const double* v, double* y);
  int krylov_mf(const double* b, double* z, double rel, int max_it, int* iters);
  // preconditioner "auto": block Jacobi until a solve needs more than auto_threshold_
  // iterations, then the multigrid
  static constexpr int kAutoMultigridIterations = 100;
  bool auto_pc_ = false;
  int auto_threshold_ = kAutoMultigridIterations;

 public:
  // the preconditioner in use as a JSON object
  std::string precond_info() const;

 private:
  // fp32 SpMV layout: kSpmvAuto times both on the first fp32 operator and keeps the faster
  int spmv_request_ = kSpmvAuto;
  void tune_spmv();

 public:
  static constexpr int kSpmvAuto = -1, kSpmvBsr = 0, kSpmvSell = 1;
  int spmv_format = kSpmvAuto;     // the layout in use (auto until tuned)
  double spmv_tune_us[2] = {0.0, 0.0};  // BSR / SELL-32 SpMV time measured by the tuner

 private:
  double dec_ = 0.5, inc_ = 1.1;
  bool has_min_ = false, has_max_ = false;
  double dt_min_ = 0.0, dt_max_ = 0.0;
};

}  // namespace dcgpu
