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
  int device = 0;  // the CUDA device that was current at creation (the model's buffers live there)
  dcgpu::DeviceBuffer<double> scratch_x, scratch_r, scratch_j;
};

// Looks up the allocation-free entry point's staging array on `device` (noalloc.cu); called
// at model creation so that the module holding the array is loaded there, not inside the
// first allocation-free call.  Returns false if the lookup failed (the entry point retries).
bool dc_noalloc_prepare(int device);
