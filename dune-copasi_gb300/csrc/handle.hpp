// The opaque model handle behind the C ABI (include/dcgpu.h).
#pragma once

#include <memory>

#include "model.hpp"
#include "server.hpp"
#include "solver.hpp"

struct dc_server {
  std::unique_ptr<dcgpu::Server> server;
};

struct dc_model {
  std::unique_ptr<dcgpu::Model> model;
  std::unique_ptr<dcgpu::Solver> solver;
  cudaStream_t stream = nullptr;
  dcgpu::DeviceBuffer<double> scratch_x, scratch_r, scratch_j;
};
