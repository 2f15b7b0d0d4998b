// Transform/reduce operators on the device (see reduce.cu, reduce.cpp).
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "device.cuh"

namespace dcgpu {

struct ReduceParams {
  int64_t ne = 0;
  const double* coords = nullptr;     // nv * dim
  const int32_t* cells = nullptr;     // ne * (dim + 1) vertex ids
  const int32_t* cell_nodes = nullptr;  // ne * (dim + 1) block rows in the cell's compartment (-1: none)
  const int32_t* cell_comp = nullptr;   // ne (-1: no compartment)
  const int8_t* sp_comp = nullptr;    // compartment of each model-global species
  const int8_t* sp_local = nullptr;   // index inside its compartment
  DevProgram prog{};
  DevTables tables{};
  const double* x = nullptr;          // blocked state
  int bs = 1;
  double t = 0.0;
  int nkeys = 0;
  double* out = nullptr;              // nkeys * ne * nq, point (e, q) at e * nq + q
};

int reduce_points(int dim);  // points of the order-4 rule per cell
void launch_reduce_eval(int dim, const ReduceParams& p, cudaStream_t s);
// out = fold of v[0..n) with op 0 (+), 1 (max), 2 (min); partial holds nblocks doubles
void launch_fold(const double* v, int64_t n, int op, double* partial, int nblocks, unsigned* counter, double* out,
                 cudaStream_t s);

}  // namespace dcgpu
