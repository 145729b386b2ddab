// Internal types shared by the host launchers and the kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gg.h"

namespace gg {

// device flag slots (context-owned int32[8]); see gg_read_flags
enum { FLAG_INDEX = 0, FLAG_TIMEOUT = 1, FLAG_UNSORTED = 2, FLAG_BOUNDS = 3 };

constexpr int kMaxPols = 8;
constexpr int kBinThreads = 256;

// One gridding job as the kernels see it.  For the binned methods `idx` and
// `vals` are the tile-sorted copies made by the binning pass: idx[k] is the
// packed (main*G+sub) pair of sorted visibility k and vals holds P planes of
// `vstride` complex values each.  Scatter reads the caller's uv/vals.
struct JobDesc {
  void *out;             // grid head (N*N*P complex of out type)
  const void *uv;        // caller's (u,v), scatter only
  const void *vals;      // values: sorted planes (binned) or caller's (scatter)
  const int2 *idx;       // sorted packed indices (binned)
  const void *gcf;       // un-offset table [G*G][S][S] (TABLE)
  const int *bookmarks;  // [ntiles+1] sorted offsets per uv tile (binned)
  float *lo;             // FP32 lo grid for compensated scatter (or null)
  int64_t npts;          // visibilities (scatter) / kept (binned)
  int64_t vstride;       // plane stride of sorted vals
  int N, S, G, log2G, P, T, log2T, ntx;
  int planar, out_f64, uv_f64;
  float sigma;
  // per-visibility GCF tables (1 = a single table); binned methods: the
  // binning key of a visibility is tile * n_gcf + its table index
  const int *gcf_index;  // scatter: the caller's per-visibility indices
  int n_gcf;
  // moving window, FP32 tables: real parts of the row-doubled tables and a
  // flag that is nonzero when any imaginary part is (null: not available)
  const float *gcf_real;
  const int *gcf_imag;
};

// A slice of one uv tile's sorted visibilities: the unit of the device work
// queue of the moving-window kernel (and of batched launches).  `slot` is the
// FP64 merge slot of the tile (see MergeSlots) when the tile is cut into
// several items and its partial sub-grids must be merged without FP32
// roundings; -1 otherwise.
struct __align__(16) WorkItem {
  int job;
  int bin;
  int start;
  int end;
  int slot;
  int pad_[3];
};

// FP64 merge slots of one support class of a compensated moving-window
// launch.  A tile cut into k > 1 work items would otherwise send k partial
// sub-grids to its FP32 output cells, each reduction rounding once (an error
// growing with k).  Instead every item of such a tile adds its partial
// sub-grid exactly (hi + lo in FP64) into the tile's slot: `cells` = P * R^2
// double2 values, R = T + S - 1 the sub-grid side; a finalize kernel then
// rounds every slot cell once into the grid.  Only for FP32 values with
// compensated accumulation into complex64 grids (complex128 grids take the
// FP64 reduction directly).
struct MergeSlots {
  double2 *base;  // [cap][cells], null: no slots in this class
  int2 *desc;     // [cap]: {job, bin} of the tile owning each slot
  int cap;        // slots available
  int cells;      // double2 values per slot
};

template <typename T> struct vec2_of;
template <> struct vec2_of<float> { using type = float2; };
template <> struct vec2_of<double> { using type = double2; };

}  // namespace gg
