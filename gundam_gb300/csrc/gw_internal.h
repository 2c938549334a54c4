// gw_internal.h -- what the host side of libgw hands to the kernel launchers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gw_layout.h"

namespace gw {

// Device-side status bits, OR-ed by kernels into DevView::status.
enum : uint32_t {
  kStatusCopyTimeout = 1u,   // a bounded wait on a bulk copy gave up
  kStatusBadTile = 2u        // a tile descriptor failed its in-kernel check
};

// Every device pointer and size a launch needs.  Plain data, passed by value.
struct DevView {
  int precision;        // 0 = FP64, 1 = FP32, 2 = double-float (GW_DF64)
  int plain_kind;       // K = 1 kernel: 0 = k_plain, 1 = k_plain_ws (warp-specialised)
  int n_params;
  int n_bins;
  int n_events;
  int n_tiles;
  int kpad;             // parameter points per row of the [param][kpad] arrays
  int llh_type;
  int has_prior;
  int has_cap;
  int n_tables;
  int n_table_fns;
  int tile_payload_bytes;  // shared-memory bytes reserved per payload stage
  int tile_hdr_bytes;      // shared-memory bytes for one tile's headers (16-byte multiple)
  int spline_knots;        // 1: Catmull-Rom payloads hold knot values only (slopes formed on the device)
  int spline_coefs;        // 1: monotonic, compact and uniform splines hold per-interval cubic coefficients
  int n_grids;             // knot grids of the grid form (0: none)
  double cap;

  const TileDesc* tiles;
  const uint64_t* hdr;
  const uint64_t* hdr_ev;     // the same headers, each tile's in slot (event-major) order (engines with k_max > 1)
  const unsigned char* payload;
  const uint16_t* evinfo;
  const uint16_t* evcost;     // [n_events] summed dial_cost + kEventCost through the event, from its tile's first
  const void* w0;             // T[n_events], bin-sorted
  const int32_t* bin_slot;    // [n_bins + 1]
  const void* pclamp;         // T2[n_params] = (lower, upper)
  const uint8_t* pflags;      // [n_params], bit 0 = truncate (no extrapolation)
  const double* mirror_lo;    // [n_params]
  const double* mirror_hi;    // [n_params]
  const double* prior_mean;   // [n_params]
  const double* prior_icov;   // [n_params * n_params]
  // eigen-decomposed parameter blocks: original[first + i] =
  // sum_j V[i][j] * given[first + j] (V row-major n x n, at eig_V + eig_off)
  int n_eigen;
  const int32_t* eig_first;
  const int32_t* eig_n;
  const int64_t* eig_off;
  const double* eig_V;
  const double* data;         // [n_bins]
  const TableDesc* tables;
  const TableFn* table_fns;
  const double* table_nodes;
  void* table_arena;          // T
  const int32_t* sorted_to_result;  // [n_events]
  const GridDesc* grids;      // [n_grids]
  const void* grid_clamp;     // T2[n_grids]: response clamp of the grid's dials, within [-1e20, 1e20]
  void* grid_pts;             // GridPoint<T>[n_grids * kpad], formed by k_params

  void* x;                    // T[n_params * kpad], mirrored parameter values
  double* penalty;            // [kpad]
  double2* partials;          // [n_slots * kpad]  (scratch)
  double* llh_blocks;         // [kpad * llh_nblk] (scratch)
  unsigned int* llh_counter;  // [kpad]           (scratch)
  int llh_nblk;
  double* event_weights;      // [n_events] in result order, or nullptr
  uint32_t* status;
};

// Launchers (gw_kernels.cu).  All are asynchronous on `stream`.
cudaError_t prepare_params(const DevView& v);  // once, before any launch or capture
cudaError_t launch_params(const DevView& v, const double* params, int K, cudaStream_t s);
cudaError_t launch_table_fns(const DevView& v, int K, int max_size, cudaStream_t s);
cudaError_t launch_plain(const DevView& v, int grid, cudaStream_t s);
// Shape of a batched (K > 1) launch.  kind 0 = k_batched: lanes over points,
// kc points per warp pass, kr points per lane.  kind 1 = k_multi: threads over
// dials, kc points per chunk, kr points per thread.  kind 3 = k_ws: the
// warp-specialised K = 1 kernel with kc = kr points per evaluator thread.
// threads per block and
// payload stages for both; minb = CTAs per SM the kernel's register
// allocation targets (its launch bounds; 0 = the compiler's choice).
struct BatchedShape {
  int kind, kc, kr, threads, stages, minb;
};
int batched_shape_count();
BatchedShape batched_shape(int i);

// One compiled batched kernel: its function (for occupancy queries) and its
// launcher, per precision [FP64, FP32, double-float] (indexed by the
// engine's precision value).
struct ShapeEntry {
  int kind, kc, kr, threads, stages, minb;
  const void* fn[3];
  void (*launch[3])(const DevView&, int, int, size_t, cudaStream_t);
};
int lane_shapes(const ShapeEntry** out);   // gw_lanes.cu
int multi_shapes(const ShapeEntry** out);  // gw_multi.cu
// kind 3 = k_ws (gw_ws.cu): the warp-specialised K = 1 kernel with kc points
// per evaluator thread (kr = kc).
int ws_shapes(const ShapeEntry** out);
size_t ws_smem_bytes(const DevView& v, int kc);
cudaError_t launch_batched(const DevView& v, int K, const BatchedShape& b, int grid, cudaStream_t s);
// True when every pass of the shape over K points stays inside the kpad
// columns of the parameter and partial-sum arrays.
bool batched_shape_covers(const DevView& v, const BatchedShape& b, int K);
cudaError_t launch_bins_llh(const DevView& v, int K, double* sums, double* sums2, double* llh,
                            double* llh_stat, cudaStream_t s);

// Shared memory a kernel shape needs, and how many CTAs fit on one SM.
size_t plain_smem_bytes(const DevView& v);
size_t batched_smem_bytes(const DevView& v, const BatchedShape& b);
int plain_blocks_per_sm(const DevView& v);
int batched_blocks_per_sm(const DevView& v, const BatchedShape& b);

constexpr int kPlainThreads = 256;

}  // namespace gw
