// Graph set-up on the device for the preconditioners: prefix sums, Jones-Plassmann
// colouring of the block-row graph, stable ordering of rows by colour, MIS-k aggregation and
// the coarse pattern of an aggregation (with the fine-to-coarse block lists of the Galerkin
// product).
//
// Everything here is deterministic: priorities come from a fixed integer hash of the row
// index (ties broken by the index), decisions of one round read only the previous round's
// state, and every list is ordered by row or block index.  The host reads back scalar
// totals only (to size the next allocation).
#pragma once

#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "model.hpp"
#include "sell.cuh"

namespace dcgpu {

// CSR graph of block rows on the device (diagonal entries may be present: self-loops are
// ignored).  Rows of different `group` (null: one group) are treated as not adjacent.
struct DeviceGraph {
  int64_t n = 0;
  const int32_t* rowptr = nullptr;
  const int32_t* colidx = nullptr;
  const int32_t* group = nullptr;
};

// out[0..n] = exclusive prefix sums of in[0..n) (out[n] = the total, also returned, which
// synchronises s).  in and out may not alias.
int64_t exclusive_scan(const int32_t* in, int32_t* out, int64_t n, cudaStream_t s);

// Jones-Plassmann colouring (groups ignored: a colouring of the whole graph): colour[i] in
// [0, ncolours), adjacent rows never share a colour.  Each round colours the uncoloured rows
// whose hash priority beats every uncoloured neighbour's with the smallest colour that no
// coloured neighbour has.  Returns the number of colours.
int color_rows(const DeviceGraph& g, int32_t* colour, cudaStream_t s);

// perm[pos] = row, rows ordered by colour and by index within a colour; offsets (host,
// ncolours + 1 entries) delimit the colours in perm.
void order_by_color(int64_t n, const int32_t* colour, int ncolours, int32_t* perm, std::vector<int64_t>* offsets,
                    cudaStream_t s);

// Aggregation around a distance-k maximal independent set (k = 1 or 2) of the graph with
// edges inside a group only: roots are numbered in row order; every other row joins the
// highest-priority root adjacent to it, or else (k = 2) the aggregate of its highest-priority
// neighbour that joined one.  agg[i] receives the aggregate of row i; returns the number of
// aggregates.
int64_t aggregate_mis(const DeviceGraph& g, int k, int32_t* agg, cudaStream_t s);

// Structure of the coarse level of an aggregation (all device buffers, sized here).
struct CoarseStructure {
  int64_t n = 0, nnzb = 0;
  DeviceBuffer<int32_t> rowptr, colidx, diag, group;
  // members of every aggregate (ascending row)
  DeviceBuffer<int32_t> agg_ptr, agg_rows;
  // for every coarse block, the fine blocks that add into it (ascending fine block index)
  DeviceBuffer<int32_t> gal_ptr, gal_src;
};
void coarse_structure(const DeviceGraph& fine, const int32_t* agg, int64_t na, CoarseStructure* out,
                      cudaStream_t s);

// SELL-32 layout (sell.cuh) of a BSR pattern, built on the device: slot offsets per slice of
// 32 rows, the padded block columns, and for every slot the BSR block it holds (-1: padding).
struct SellStructure {
  int64_t nrows = 0, nslices = 0, nslots = 0;
  DeviceBuffer<int64_t> off;
  DeviceBuffer<int32_t> cols, bpos;
  Sell view(int bs) const {
    Sell S;
    S.nrows = static_cast<int>(nrows);
    S.bs = bs;
    S.nslices = nslices;
    S.nslots = nslots;
    S.off = off.get();
    S.cols = cols.get();
    return S;
  }
};
void sell_structure(int64_t nrows, const int32_t* rowptr, const int32_t* colidx, SellStructure* out, cudaStream_t s);
// out (nslots * 32 * bs * bs values) = the BSR blocks `bsr` in the layout S with the
// entries interleaved by lane (sellrow.cuh), padding zero
void sell_values(const SellStructure& S, int bs, const double* bsr, double* out, cudaStream_t s);
void sell_values(const SellStructure& S, int bs, const double* bsr, float* out, cudaStream_t s);

}  // namespace dcgpu
