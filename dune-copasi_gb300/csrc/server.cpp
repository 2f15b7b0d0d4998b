#include "server.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>

#include <cuda_runtime.h>

#include "model.hpp"
#include "solver.hpp"

namespace dcgpu {

Server::Server(int64_t budget_bytes, int max_active, bool batch_krylov) : budget_(budget_bytes) {
  if (budget_bytes <= 0) throw std::invalid_argument("memory budget must be positive");
  if (max_active <= 0 || max_active > 256) throw std::invalid_argument("max_active must be in [1, 256]");
  cuda_check(cudaGetDevice(&device_), "cudaGetDevice");
  if (batch_krylov) batcher_ = std::make_unique<KrylovBatcher>(device_, max_active);
  for (int i = 0; i < max_active; ++i) workers_.emplace_back([this] { worker(); });
}

Server::~Server() {
  {
    // finish every submitted request before the workers leave
    std::unique_lock<std::mutex> lk(mu_);
    cv_done_.wait(lk, [&] { return queue_.empty() && active_ == 0; });
    stop_ = true;
  }
  cv_work_.notify_all();
  for (auto& t : workers_) t.join();
}

double Server::now() const {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

int64_t Server::estimate_bytes(const std::string& ini, const std::string& overrides) {
  Ini cfg = Ini::parse(ini);
  if (!overrides.empty()) cfg.apply_overrides(overrides);
  Ini grid = cfg.sub("grid");
  int dim = 2;
  if (grid.has_key("dimension")) dim = static_cast<int>(grid.get_long("dimension", 2));
  else if (grid.has_key("extensions")) dim = static_cast<int>(grid.get_doubles("extensions", {}).size());
  if (dim != 2 && dim != 3) throw ConfigError("only grid.dimension 2 or 3 is supported");
  auto cells = grid.get_doubles("cells", std::vector<double>(dim, 1.0));
  const long level = grid.get_long("refinement_level", 0);
  double nv = 1.0, ncube = 1.0;
  for (int d = 0; d < dim && d < static_cast<int>(cells.size()); ++d) {
    const double c = cells[d] * std::pow(2.0, static_cast<double>(level));
    nv *= c + 1.0;
    ncube *= c;
  }
  double ne = ncube * (dim == 2 ? 2.0 : 6.0);
  if (grid.has_key("path")) {
    Mesh m = read_gmsh(grid.get("path", ""), dim);
    nv = static_cast<double>(m.nv);
    ne = static_cast<double>(m.ne);
  }
  const int nl = dim + 1;
  // species per compartment
  Ini sf = cfg.sub("model").sub("scalar_field");
  std::map<std::string, int> per;
  for (const auto& name : sf.sub_keys()) {
    std::string c = sf.sub(name).get("compartment", "");
    if (!c.empty()) ++per[c];
  }
  int bs = 1, ncomp = 0;
  for (const auto& kv : per) {
    bs = std::max(bs, kv.second);
    ++ncomp;
  }
  const double nnodes = nv * std::max(1, std::min(ncomp, 2));
  const double nnzb = nnodes * (dim == 2 ? 7.0 : 15.0);
  const double vals = nnzb * bs * bs * 8.0;
  const double n = nnodes * bs;
  double bytes = 4.5 * vals                      // J, static mass / stiffness / combination, fp32 copy
                 + 1.5 * nnodes * bs * bs * 8.0  // block-Jacobi inverses (fp64 + fp32)
                 + 25.0 * n * 8.0                // state, stages, Krylov vectors
                 + nnzb * 4.0 + nnodes * 8.0     // pattern
                 + ne * (2.0 * nl * 4.0 + nl * nl * 4.0) + nv * dim * 8.0   // cells, nodes, bpos, coords
                 + ne * nl * (nl * bs * bs + bs) * 8.0                      // element outputs (upper bound)
                 + ne * nl * (nl + 1) * 4.0 + (nnodes + nnzb) * 8.0;        // gather lists
  return static_cast<int64_t>(bytes * 1.2) + (int64_t{1} << 20);
}

int64_t Server::submit(const std::string& ini, const std::string& overrides, std::vector<double> init) {
  Request r;
  r.ini = ini;
  r.overrides = overrides;
  r.init = std::move(init);
  r.submit_t = now();
  r.bytes = estimate_bytes(ini, overrides);
  std::lock_guard<std::mutex> lk(mu_);
  r.id = next_id_++;
  if (r.bytes > budget_) {
    ServerResult res;
    res.id = r.id;
    res.status = DC_ERR_CONFIG;
    res.bytes_estimate = r.bytes;
    res.error = "request needs more device memory than the server's budget";
    done_.push_back(res);
    cv_done_.notify_all();
    return r.id;
  }
  queue_.push_back(std::move(r));
  cv_work_.notify_one();
  return queue_.back().id;
}

int Server::pending() {
  std::lock_guard<std::mutex> lk(mu_);
  return static_cast<int>(queue_.size()) + active_;
}

void Server::worker() {
  cudaSetDevice(device_);
  while (true) {
    Request req;
    {
      std::unique_lock<std::mutex> lk(mu_);
      auto admissible = [&]() {
        // first-come first-served, with later requests backfilling free memory
        return std::find_if(queue_.begin(), queue_.end(),
                            [&](const Request& r) { return in_use_ + r.bytes <= budget_; });
      };
      cv_work_.wait(lk, [&] { return stop_ || admissible() != queue_.end(); });
      // the device itself must have the room too (other processes, allocator slack):
      // admission waits, re-checking when a simulation finishes or shrinks its charge
      if (!stop_ && admissible() != queue_.end()) {
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess &&
            static_cast<int64_t>(free_b) < admissible()->bytes + kDeviceReserve && active_ > 0) {
          cv_work_.wait_for(lk, std::chrono::milliseconds(5));
          continue;
        }
      }
      auto it = admissible();
      if (it == queue_.end()) {
        if (stop_) return;
        continue;
      }
      req = std::move(*it);
      queue_.erase(it);
      in_use_ += req.bytes;
      ++active_;
    }
    ServerResult res;
    res.id = req.id;
    res.bytes_estimate = req.bytes;
    int64_t held = req.bytes;                          // bytes charged against the budget
    const int64_t base = device_bytes_this_thread();   // this worker's buffers before the request
    int64_t peak = 0;
    auto measure = [&]() {
      const int64_t m = device_bytes_this_thread() - base;
      if (m > peak) {
        peak = m;
        recharge(held, peak);
      }
    };
    const double t_admit = now();
    res.queue_s = t_admit - req.submit_t;
    std::vector<double> state;
    cudaStream_t stream = nullptr;
    try {
      cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
      Model model(req.ini, req.overrides);
      // Concurrent simulations solve with graph-replayed per-phase launches unless their
      // configuration asks otherwise: a single-launch solve holds whole SMs (its blocks use
      // the full register file) through its barrier waits, which starves the kernels of the
      // other simulations' streams (32-request serving mix: 21.3 M against 29.3 M
      // DOF·Newton-steps/s).  Every request of a server takes the same path, so results do
      // not depend on what else runs.
      const std::string sl_key = "model.time_step_operator.linear_solver.single_launch";
      if (!model.cfg.has_key(sl_key)) model.cfg.set(sl_key, "false");
      // the batch reads the fp32 operator in the SELL-32 layout: no per-model layout tuning
      const std::string spmv_key = "model.time_step_operator.linear_solver.spmv";
      if (batcher_ && !model.cfg.has_key(spmv_key)) model.cfg.set(spmv_key, "sell");
      Solver solver(model, stream);
      if (batcher_) solver.attach_batcher(batcher_.get());
      measure();
      res.setup_s = now() - t_admit;
      Ini tso = model.cfg.sub("model").sub("time_step_operator");
      const double t0 = tso.get_double("time_begin", 0.0);
      const double t1 = tso.get_double("time_end", 1.0);
      const double dt_max = tso.get_double("time_step_max", 0.1);
      double dt = tso.get_double("time_step_initial", tso.has_key("time_step_max") ? dt_max : 0.1);
      if (!req.init.empty()) solver.set_state(req.init, t0);
      // buffers made during the run (graphs' work vectors, a multigrid built on the way)
      res.status = solver.evolve(t1, dt, [&](double) { measure(); });
      res.ndof = model.ndof;
      res.newton_iterations = solver.stats.newton_iterations;
      res.linear_iterations = solver.stats.linear_iterations;
      res.steps = solver.stats.steps;
      state = solver.get_state();
      if (res.status != DC_OK) res.error = "time stepping failed";
    } catch (const ConfigError& e) {
      res.status = DC_ERR_CONFIG;
      res.error = e.what();
    } catch (const CudaError& e) {
      res.status = DC_ERR_CUDA;
      res.error = e.what();
    } catch (const StepFailure& e) {
      res.status = e.code;
      res.error = e.what();
    } catch (const std::exception& e) {
      res.status = DC_ERR_INTERNAL;
      res.error = e.what();
    }
    if (stream) cudaStreamDestroy(stream);
    const double t_end = now();
    res.run_s = t_end - t_admit;
    res.latency_s = t_end - req.submit_t;
    res.bytes_measured = peak;
    {
      std::lock_guard<std::mutex> lk(mu_);
      in_use_ -= held;
      --active_;
      states_[res.id] = std::move(state);
      done_.push_back(std::move(res));
    }
    cv_done_.notify_all();
    cv_work_.notify_all();
  }
}

BatchStats Server::batch_stats() const { return batcher_ ? batcher_->stats() : BatchStats{}; }
std::string Server::batch_tuning() const { return batcher_ ? batcher_->tuning() : std::string("{}"); }

void Server::recharge(int64_t& held, int64_t measured) {
  {
    std::lock_guard<std::mutex> lk(mu_);
    in_use_ += measured - held;
    held = measured;
  }
  // a smaller charge than the estimate may let a waiting request in
  cv_work_.notify_all();
}

std::vector<ServerResult> Server::poll(bool wait, int max) {
  std::unique_lock<std::mutex> lk(mu_);
  if (wait) cv_done_.wait(lk, [&] { return !done_.empty() || (queue_.empty() && active_ == 0); });
  std::vector<ServerResult> out;
  const int n = std::min<int>(max, static_cast<int>(done_.size()));
  out.assign(std::make_move_iterator(done_.begin()), std::make_move_iterator(done_.begin() + n));
  done_.erase(done_.begin(), done_.begin() + n);
  return out;
}

bool Server::take_state(int64_t id, std::vector<double>& out) {
  std::lock_guard<std::mutex> lk(mu_);
  auto it = states_.find(id);
  if (it == states_.end()) return false;
  out = std::move(it->second);
  states_.erase(it);
  return true;
}

}  // namespace dcgpu
