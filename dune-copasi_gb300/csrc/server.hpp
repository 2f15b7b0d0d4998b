// Request server: continuous admission of many independent simulations onto one GPU.
//
// No counterpart in the reference (it runs one simulation per process).  Requests (an INI
// text plus optional initial state) queue on the host; worker threads admit them as soon
// as their estimated device footprint fits into the memory budget and a slot is free, so
// requests that arrive while others run start without waiting for the running ones to
// finish.  Each admitted request owns a model on its own CUDA stream (graph-replayed
// Krylov iterations, deterministic reductions), so the work of concurrent requests
// overlaps on the device and every result is bitwise identical to the same request run
// alone.
#pragma once

#include <condition_variable>
#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "batch.hpp"

namespace dcgpu {

struct ServerResult {
  int64_t id = 0;
  int status = 0;
  double queue_s = 0.0;    // submit -> admission
  double run_s = 0.0;      // admission -> completion (model set-up + evolve)
  double latency_s = 0.0;  // submit -> completion
  int64_t ndof = 0;
  int64_t newton_iterations = 0;
  int64_t linear_iterations = 0;
  int64_t steps = 0;
  int64_t bytes_estimate = 0;
  int64_t bytes_measured = 0;  // peak device bytes the simulation's buffers held
  double setup_s = 0.0;        // model and solver set-up (part of run_s)
  std::string error;
};

class Server {
 public:
  // batch_krylov: the running simulations' block-Jacobi BiCGSTAB solves are packed into
  // one batch (KrylovBatcher, one slot per active simulation) instead of each replaying
  // its own graphs on its own stream
  Server(int64_t budget_bytes, int max_active, bool batch_krylov = false);
  ~Server();
  Server(const Server&) = delete;
  Server& operator=(const Server&) = delete;

  int64_t submit(const std::string& ini, const std::string& overrides, std::vector<double> init);
  // completed results (up to max); with wait, blocks until at least one is available or
  // nothing is pending / running
  std::vector<ServerResult> poll(bool wait, int max);
  // final state of a completed request (reference DOF order); erases it
  bool take_state(int64_t id, std::vector<double>& out);
  int pending() ;
  // counters of the Krylov batch (all zero without batch_krylov)
  BatchStats batch_stats() const;
  // the Krylov batch's tuned replay grids as JSON ("{}" without batch_krylov)
  std::string batch_tuning() const;

  static int64_t estimate_bytes(const std::string& ini, const std::string& overrides);
  // device memory kept free beyond an admitted request's estimate
  static constexpr int64_t kDeviceReserve = int64_t{256} << 20;

 private:
  struct Request {
    int64_t id;
    std::string ini, overrides;
    std::vector<double> init;
    double submit_t;
    int64_t bytes;
  };
  void worker();
  // charge a running simulation its measured footprint instead of what it was admitted
  // with (held: the bytes currently charged for it, updated)
  void recharge(int64_t& held, int64_t measured);
  double now() const;

  std::mutex mu_;
  std::condition_variable cv_work_, cv_done_;
  std::deque<Request> queue_;
  std::vector<ServerResult> done_;
  std::map<int64_t, std::vector<double>> states_;
  int64_t budget_, in_use_ = 0, next_id_ = 1;
  int active_ = 0;
  bool stop_ = false;
  std::unique_ptr<KrylovBatcher> batcher_;  // destroyed after the workers have joined
  std::vector<std::thread> workers_;
  int device_ = 0;
};

}  // namespace dcgpu
