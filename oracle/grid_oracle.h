/*
 * CPU oracle for the convolutional gridder -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's CPU gridder and of the integer
 * steps of its GPU driver.  Only tests, the smoke check and the CPU-baseline
 * leg of the benchmark may load this library, and only as the checker; the
 * product path (libgg.so) never links or calls it.
 *
 * Reference files cited below are paths within the NVIDIA/SKA-gpu-grid
 * project (grid.cu, grid_gpu.cu).
 */
#ifndef GRID_ORACLE_H
#define GRID_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Restates gridCPU_pz (grid.cu:140-193).
 *   out_planar : 2*pols*img_dim^2 doubles; real plane [p][y][x] followed by
 *                the imaginary plane (grid.cu:153-154).  ACCUMULATES (+=),
 *                exactly like the reference, which never zeroes its output.
 *   uv         : npts (u,v) pairs in grid-pixel units (CmplxType in[]).
 *   vals       : npts*pols complex values, interleaved (re,im).
 *   gcf        : the UN-offset table, gcf_grid^2 * gcf_dim^2 complex values,
 *                laid out [sub_y*gcf_grid+sub_x][b'][a'] (grid.cu:169-172
 *                after the centre offset of grid.cu:152).
 *   debug1     : nonzero = the reference's DEBUG1 footprint mode
 *                (grid.cu:180-182): adds (1, n) instead of val*gcf.
 */
void oracle_grid_pz(double *out_planar, const double *uv, const double *vals,
                    size_t npts, size_t img_dim, const double *gcf,
                    size_t gcf_dim, int gcf_grid, int pols, int debug1);

/* Same result, bit for bit: the img_dim rows are split into nthreads bands
 * and every band walks all visibilities in input order, so each cell sees
 * the same additions in the same order as oracle_grid_pz. */
void oracle_grid_pz_mt(double *out_planar, const double *uv,
                       const double *vals, size_t npts, size_t img_dim,
                       const double *gcf, size_t gcf_dim, int gcf_grid,
                       int pols, int debug1, int nthreads);

/* gridCPU_pz with a table per visibility: visibility n reads table
 * gcfinx[n] of n_gcf consecutive [G*G][S][S] tables -- the selection the
 * reference's vis.gcfinx (vis.h:17, set per baseline in hdf52struct.cpp:116)
 * stands for; its gridders themselves use one table.  A visibility whose
 * index is outside [0, n_gcf) is skipped.  gcfinx NULL = table 0 for all. */
void oracle_grid_pz_gcfinx(double *out_planar, const double *uv,
                           const double *vals, const int32_t *gcfinx,
                           size_t npts, size_t img_dim, const double *gcf,
                           int n_gcf, size_t gcf_dim, int gcf_grid, int pols,
                           int debug1, int nthreads);

/* gridCPU_pz with the reference GPU scatter kernel's COMPUTE_GCF factor in
 * place of the table (grid_gpu.cu:103-108, 137-147): every tap of a
 * visibility is multiplied by (sin phi, cos phi), phi computed in float from
 * (T, w) = the first entry of the centre-offset table gcf (gcf itself is
 * passed un-offset, as everywhere here) and the visibility's sub-pixel
 * position. */
void oracle_grid_pz_wphase(double *out_planar, const double *uv,
                           const double *vals, size_t npts, size_t img_dim,
                           const double *gcf, size_t gcf_dim, int gcf_grid,
                           int pols, int nthreads);

/* Per-cell magnitude sums for the forward-error metric of the tests and the
 * benchmark (no counterpart in the reference):
 *   mag[p][y][x] = sum of |val| * |w| over exactly the visibilities and taps
 * that gridCPU_pz adds into cell (x, y) of plane p (same index step, tap
 * window, table selection -- gcfinx NULL: table 0 -- and COMPUTE_GCF factor
 * when wphase is nonzero).  |grid - oracle| / mag at a cell is the forward
 * error of that cell's sum relative to the magnitudes summed there, the
 * quantity the rounding-error bound of a floating-point sum is stated in; it
 * stays meaningful at cells where the sum cancels.  mag holds
 * pols*img_dim^2 doubles, ACCUMULATED (+=). */
void oracle_grid_mag_pz(double *mag, const double *uv, const double *vals,
                        const int32_t *gcfinx, size_t npts, size_t img_dim,
                        const double *gcf, int n_gcf, size_t gcf_dim, int gcf_grid,
                        int pols, int wphase, int nthreads);

/* Degridding, the adjoint of oracle_grid_pz_gcfinx (the reference has no
 * degridder; this follows its gridder's conventions, grid.cu:157-191):
 *   vals_out[n][p] = sum over the taps (a, b) in (-S/2, S/2]^2 of visibility
 *                    n that fall on the grid of grid[p][y][x] * conj(w)
 * with the index step, tap window and table entry w of the gridder, so that
 * <grid_pz(v), g> = <v, degrid_pz(g)> for the complex inner product
 * <a, b> = sum conj(a) b.  grid_planar is laid out like out_planar above
 * (real planes, then imaginary planes); vals_out receives npts*pols complex
 * values (re, im), OVERWRITTEN.  A visibility whose oversample index falls
 * outside [0, gcf_grid) or whose table index (gcfinx, NULL: table 0) falls
 * outside [0, n_gcf) gets zero.  The products are summed in the tap order
 * b' (rows) then a' (columns), in double; nthreads split the visibilities,
 * so the result does not depend on nthreads. */
void oracle_degrid_pz(double *vals_out, const double *grid_planar,
                      const double *uv, const int32_t *gcfinx, size_t npts,
                      size_t img_dim, const double *gcf, int n_gcf,
                      size_t gcf_dim, int gcf_grid, int pols, int nthreads);

/* The index step of gridCPU_pz (grid.cu:159-163): main = floor(u),
 * sub = floorf(G*(u - floorf(u))) with the float conversions C applies.
 * Writes packed (main*G+sub) pairs like vis2ints (grid_gpu.cu:352-365). */
void oracle_vis2ints(const double *uv, size_t npts, int gcf_grid,
                     int32_t *packed_xy);

/* vis2ints as the GPU driver computes it, entirely in double
 * (grid_gpu.cu:357-363).  Agrees with oracle_vis2ints whenever u and v are
 * float-representable. */
void oracle_vis2ints_gpu_formula(const double *uv, size_t npts, int gcf_grid,
                                 int32_t *packed_xy);

/* Restates set_bookmarks (grid_gpu.cu:366-390) for packed ints sorted by
 * tile: bookmarks[z] = index of the first visibility whose tile id is >= z,
 * for z in [0, ntiles]; tile id = (main_y/blocksize)*blockgrid +
 * main_x/blocksize.  Entries past the last occupied tile are npts. */
void oracle_set_bookmarks(const int32_t *packed_xy, size_t npts, int gcf_grid,
                          int blocksize, int blockgrid, int32_t *bookmarks);

/* Separable Gaussian GCF table in the reference's layout (see
 * oracle_grid_pz): value(sx,sy,a',b') = g(a'-S/2+1 - sx/G) * g(b'-S/2+1 -
 * sy/G), g(x) = exp(-x^2/(2 sigma^2)), imaginary part 0.  g1 receives the
 * [G][S] one-dimensional factors (may be NULL). */
void oracle_gaussian_gcf(double *gcf, double *g1, int gcf_dim, int gcf_grid,
                         double sigma);

/* Builds the 2-D table from given 1-D factors g1[G][S]: an exact product,
 * identical on every IEEE-754 host. */
void oracle_gcf_from_1d(double *gcf, const double *g1, int gcf_dim,
                        int gcf_grid);

#ifdef __cplusplus
}
#endif
#endif
