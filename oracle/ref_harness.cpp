/*
 * Build-recipe helper (TEST INFRASTRUCTURE ONLY): exposes the reference's own
 * CPU gridder to ctypes.  It #includes grid.cu from the reference checkout
 * given to the compiler with -I (see oracle/Makefile); no reference source is
 * copied into this repository.  The reference's main() is renamed so that
 * only its functions are used:
 *   gridCPU_pz  grid.cu:140-193     init_gcf  grid.cu:72-85
 *   w_comp_sub / w_comp_main / comp_grid   grid.cu:194-277 (host sorts)
 * Compile-time parameters (IMG_SIZE, GCF_DIM, POLARIZATIONS, PRECISION, ...)
 * come from -D flags with -D__DEFINES_H, which skips the body of Defines.h.
 */
#include <cstring>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cuda_runtime.h>
#define main reference_main
#include "grid.cu"
#undef main

extern "C" {

/* out_head points at the unpadded grid head, as at grid.cu:487 */
void ref_gridCPU_pz(void *out_head, void *in, void *in_vals, size_t npts,
                    size_t img_dim, void *gcf, size_t gcf_dim) {
  gridCPU_pz((OUTPRECISION2 *)out_head, (PRECISION2 *)in,
             (PRECISION2 *)in_vals, npts, img_dim, (PRECISION2 *)gcf, gcf_dim);
}

void ref_init_gcf(void *gcf, size_t size) { init_gcf((PRECISION2 *)gcf, size); }

void ref_sort_sub(void *in, size_t npts) {
  std::qsort(in, npts, sizeof(PRECISION2), w_comp_sub<PRECISION2, PRECISION>);
}
void ref_sort_main(void *in, size_t npts) {
  std::qsort(in, npts, sizeof(PRECISION2), w_comp_main<PRECISION2, PRECISION>);
}
void ref_sort_grid(void *in, size_t npts) {
  std::qsort(in, npts, sizeof(PRECISION2), comp_grid<PRECISION2, PRECISION>);
}

/* The input recipe of the reference harness (grid.cu:444-452): srand(1541617)
 * then, per visibility, u, v and POLARIZATIONS (re, im) pairs from rand(),
 * each computed in float.  Restated here (not called from grid.cu, whose
 * generator is inside main). */
void ref_harness_inputs(void *in_, void *in_vals_, size_t npts) {
  PRECISION2 *in = (PRECISION2 *)in_, *in_vals = (PRECISION2 *)in_vals_;
  srand(1541617);
  for (size_t n = 0; n < npts; n++) {
    in[n].x = ((float)rand()) / RAND_MAX * IMG_SIZE;
    in[n].y = ((float)rand()) / RAND_MAX * IMG_SIZE;
    for (int p = 0; p < POLARIZATIONS; p++) {
      in_vals[POLARIZATIONS * n + p].x = ((float)rand()) / RAND_MAX;
      in_vals[POLARIZATIONS * n + p].y = ((float)rand()) / RAND_MAX;
    }
  }
}

/* img, gcf, oversample, pols, sizeof in element, sizeof out element, debug1 */
void ref_params(int *p) {
  p[0] = IMG_SIZE; p[1] = GCF_DIM; p[2] = GCF_GRID; p[3] = POLARIZATIONS;
  p[4] = (int)sizeof(PRECISION2); p[5] = (int)sizeof(OUTPRECISION2);
#ifdef DEBUG1
  p[6] = 1;
#else
  p[6] = 0;
#endif
}
}
