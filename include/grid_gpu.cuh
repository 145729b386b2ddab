/*
 * grid_gpu.cuh -- drop-in replacement for the reference's gridGPU template
 * (grid_gpu.cuh:30-32 of NVIDIA/SKA-gpu-grid), implemented over the C ABI in
 * gg.h.  A caller that includes this header and links libgg.so keeps its
 * call unchanged:
 *
 *     gridGPU(out, in, in_vals, npts, IMG_SIZE, gcf, GCF_DIM);   // grid.cu:481
 *
 * The reference picks its method with compile-time macros; they are honoured
 * here the same way and turned into gg_options:
 *   __GATHER -> GG_MODE_GATHER, __MOVING_WINDOW -> GG_MODE_WINDOW,
 *   __COMPUTE_GCF -> GG_GCF_WPHASE (the reference scatter kernel's factor),
 *   POLARIZATIONS, GCF_GRID.
 * Differences from the reference (all deliberate): errors are returned by
 * gg_last_status() instead of only printed, nothing is allocated or pinned
 * per call, and the instantiation set is the same three type pairs
 * (grid_gpu.cu:820-825).
 */
#ifndef GG_GRID_GPU_CUH
#define GG_GRID_GPU_CUH

#include <cstddef>
#include <cstdio>

#include <vector_types.h> /* float2, double2 */

#include "gg.h"

namespace gg_dropin {

inline int &last_status() {
  static thread_local int s = GG_OK;
  return s;
}

inline gg_options options_from_macros() {
  gg_options o;
  gg_get_global_options(&o);
#if defined(__GATHER)
  o.mode = GG_MODE_GATHER;
#elif defined(__MOVING_WINDOW)
  o.mode = GG_MODE_WINDOW;
#endif
#if defined(__COMPUTE_GCF)
  o.gcf_kind = GG_GCF_WPHASE;
#endif
#if defined(POLARIZATIONS)
  o.polarizations = POLARIZATIONS;
#endif
#if defined(GCF_GRID)
  o.oversample = GCF_GRID;
#endif
  return o;
}

template <class O, class I> struct types;
template <> struct types<double2, double2> { enum { out = GG_C128, in = GG_C128 }; };
template <> struct types<double2, float2> { enum { out = GG_C128, in = GG_C64 }; };
template <> struct types<float2, float2> { enum { out = GG_C64, in = GG_C64 }; };

}  // namespace gg_dropin

/* status of the calling thread's last gridGPU call (GG_OK = 0) */
inline int gg_last_status() { return gg_dropin::last_status(); }

template <class CmplxOutType, class CmplxType>
void gridGPU(CmplxOutType *out, CmplxType *in, CmplxType *in_vals, size_t npts,
             size_t img_dim, CmplxType *gcf, size_t gcf_dim) {
  typedef gg_dropin::types<CmplxOutType, CmplxType> T;
  gg_options o = gg_dropin::options_from_macros();
  int st = gg_grid_host(&o, T::out, out, T::in, in, T::in, in_vals, npts,
                        img_dim, gcf, gcf_dim);
  gg_dropin::last_status() = st;
  if (st != GG_OK) std::fprintf(stderr, "gridGPU: %s\n", gg_last_error());
}

#endif /* GG_GRID_GPU_CUH */
