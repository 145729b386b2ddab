/*
 * CPU oracle for the convolutional gridder -- TEST INFRASTRUCTURE ONLY.
 * See grid_oracle.h.  Compiled with -ffp-contract=off so that every
 * a*b-c*d is two rounded products and one rounded difference, as the
 * reference's x86 build computes it (an aarch64 compiler would otherwise
 * fuse them into FMAs).
 */
#include "grid_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* The index step of gridCPU_pz, grid.cu:159-163.  floorf() receives a double
 * argument there, so C converts it to float first; GCF_GRID*(...) is then
 * evaluated in double and converted to float again by the outer floorf. */
static inline void index_step(double u, int G, int *main_i, int *sub_i) {
  float uf = (float)u;
  double frac = (double)G * (u - (double)floorf(uf));
  *sub_i = (int)floorf((float)frac);
  *main_i = (int)floor(u);
}

typedef struct {
  double *out;
  const double *uv, *vals, *gcf;
  size_t npts, img_dim, gcf_dim;
  int G, P, debug1;
  long y0, y1; /* rows owned by this worker: [y0, y1) */
  const int32_t *gcfinx; /* per-visibility table index (NULL: table 0) */
  int n_gcf;
  int wphase; /* COMPUTE_GCF phase factor instead of the table */
  int mag;    /* magnitude sums |val|*|w| into out (one plane set) */
} band_job;

/* The reference GPU scatter kernel's COMPUTE_GCF factor (grid_gpu.cu:103-108,
 * 137-147): (T, w) = the first entry of the centre-offset table; every tap of
 * a visibility gets (sin phi, cos phi), phi = p1 - p2*sqrt(dx^2 + dy^2) with
 * dx = main_x - u + sub_x/G evaluated in double and stored as float, the
 * rest in float.  It has no CPU counterpart in the reference; this is its
 * restatement for the checker. */
static void wphase_factor(double u, double v, int main_x, int sub_x, int main_y,
                          int sub_y, int G, double T, double w, double *r2,
                          double *i2) {
  const float p1 = (float)(2 * 3.1415926 * w);
  const float p2 = (float)((double)p1 * T);
  float xs = (float)((double)main_x - u + sub_x * 1.0 / G);
  float ys = (float)((double)main_y - v + sub_y * 1.0 / G);
  xs = xs * xs;
  ys = ys * ys;
  const float ph = p1 - p2 * sqrtf(xs + ys);
  *r2 = (double)sinf(ph);
  *i2 = (double)cosf(ph);
}

/* Body of gridCPU_pz (grid.cu:157-191), restricted to rows [y0, y1).  The
 * tap loops run a (then b) from S/2 down to -S/2+1 (grid.cu:167-168); each
 * cell receives at most one addition per visibility, so the order of
 * additions into any one cell is the visibility order n. */
static void grid_band(const band_job *j) {
  const long S = (long)j->gcf_dim, N = (long)j->img_dim;
  const int G = j->G, P = j->P;
  /* gcf += GCF_DIM*(GCF_DIM-1)/2-1 (grid.cu:152), in complex elements */
  const double *gcf = j->gcf + 2 * (S * (S - 1) / 2 - 1);
  double *out1 = j->out;
  double *out2 = j->out + (size_t)P * N * N; /* grid.cu:154 */
  for (size_t n = 0; n < j->npts; n++) {
    int main_x, main_y, sub_x, sub_y;
    index_step(j->uv[2 * n], G, &main_x, &sub_x);
    index_step(j->uv[2 * n + 1], G, &main_y, &sub_y);
    if ((long)main_y + S / 2 < j->y0 || (long)main_y - S / 2 + 1 >= j->y1)
      continue; /* footprint misses this band entirely */
    long table = 0;
    if (j->gcfinx) {
      /* vis.gcfinx (vis.h:17): the visibility's own [G*G][S][S] table */
      if (j->gcfinx[n] < 0 || j->gcfinx[n] >= j->n_gcf) continue;
      table = (long)j->gcfinx[n] * G * G * S * S;
    }
    const double *g = gcf + 2 * (table + S * S * ((long)G * sub_y + sub_x));
    double wr = 0, wi = 0;
    if (j->wphase)
      wphase_factor(j->uv[2 * n], j->uv[2 * n + 1], main_x, sub_x, main_y, sub_y, G, gcf[0],
                    gcf[1], &wr, &wi);
    for (long a = S / 2; a > -S / 2; a--)
      for (long b = S / 2; b > -S / 2; b--) {
        long x = main_x + a, y = main_y + b;
        if (x < 0 || y < 0 || x >= N || y >= N) continue;
        if (y < j->y0 || y >= j->y1) continue;
        double r2 = j->wphase ? wr : g[2 * (S * b + a)];
        double i2 = j->wphase ? wi : g[2 * (S * b + a) + 1];
        for (int p = 0; p < P; p++) {
          size_t cell = (size_t)x + (size_t)N * y + (size_t)p * N * N;
          if (j->mag) {
            const double r1 = j->vals[2 * (P * n + p)], i1 = j->vals[2 * (P * n + p) + 1];
            out1[cell] += sqrt(r1 * r1 + i1 * i1) * sqrt(r2 * r2 + i2 * i2);
          } else if (j->debug1) {
            out1[cell] += 1;
            out2[cell] += (double)n;
          } else {
            double r1 = j->vals[2 * (P * n + p)];
            double i1 = j->vals[2 * (P * n + p) + 1];
            out1[cell] += r1 * r2 - i1 * i2;
            out2[cell] += r1 * i2 + r2 * i1;
          }
        }
      }
  }
}

void oracle_grid_pz(double *out_planar, const double *uv, const double *vals,
                    size_t npts, size_t img_dim, const double *gcf,
                    size_t gcf_dim, int gcf_grid, int pols, int debug1) {
  band_job j = {out_planar, uv, vals, gcf, npts, img_dim, gcf_dim,
                gcf_grid, pols, debug1, 0, (long)img_dim, NULL, 1, 0, 0};
  grid_band(&j);
}

static void *band_thread(void *arg) {
  grid_band((const band_job *)arg);
  return NULL;
}

void oracle_grid_pz_mt(double *out_planar, const double *uv,
                       const double *vals, size_t npts, size_t img_dim,
                       const double *gcf, size_t gcf_dim, int gcf_grid,
                       int pols, int debug1, int nthreads) {
  oracle_grid_pz_gcfinx(out_planar, uv, vals, NULL, npts, img_dim, gcf, 1,
                        gcf_dim, gcf_grid, pols, debug1, nthreads);
}

static void grid_mt(double *out_planar, const double *uv, const double *vals,
                    const int32_t *gcfinx, size_t npts, size_t img_dim,
                    const double *gcf, int n_gcf, size_t gcf_dim, int gcf_grid,
                    int pols, int debug1, int wphase, int nthreads);
static void grid_mt_mode(double *out_planar, const double *uv, const double *vals,
                         const int32_t *gcfinx, size_t npts, size_t img_dim,
                         const double *gcf, int n_gcf, size_t gcf_dim, int gcf_grid,
                         int pols, int debug1, int wphase, int mag, int nthreads);

void oracle_grid_mag_pz(double *mag, const double *uv, const double *vals,
                        const int32_t *gcfinx, size_t npts, size_t img_dim,
                        const double *gcf, int n_gcf, size_t gcf_dim, int gcf_grid,
                        int pols, int wphase, int nthreads) {
  grid_mt_mode(mag, uv, vals, gcfinx, npts, img_dim, gcf, n_gcf, gcf_dim, gcf_grid, pols, 0,
               wphase, 1, nthreads);
}

void oracle_grid_pz_gcfinx(double *out_planar, const double *uv,
                           const double *vals, const int32_t *gcfinx,
                           size_t npts, size_t img_dim, const double *gcf,
                           int n_gcf, size_t gcf_dim, int gcf_grid, int pols,
                           int debug1, int nthreads) {
  grid_mt(out_planar, uv, vals, gcfinx, npts, img_dim, gcf, n_gcf, gcf_dim, gcf_grid, pols,
          debug1, 0, nthreads);
}

void oracle_grid_pz_wphase(double *out_planar, const double *uv,
                           const double *vals, size_t npts, size_t img_dim,
                           const double *gcf, size_t gcf_dim, int gcf_grid,
                           int pols, int nthreads) {
  grid_mt(out_planar, uv, vals, NULL, npts, img_dim, gcf, 1, gcf_dim, gcf_grid, pols, 0, 1,
          nthreads);
}

static void grid_mt(double *out_planar, const double *uv, const double *vals,
                    const int32_t *gcfinx, size_t npts, size_t img_dim,
                    const double *gcf, int n_gcf, size_t gcf_dim, int gcf_grid,
                    int pols, int debug1, int wphase, int nthreads) {
  grid_mt_mode(out_planar, uv, vals, gcfinx, npts, img_dim, gcf, n_gcf, gcf_dim, gcf_grid, pols,
               debug1, wphase, 0, nthreads);
}

static void grid_mt_mode(double *out_planar, const double *uv, const double *vals,
                         const int32_t *gcfinx, size_t npts, size_t img_dim,
                         const double *gcf, int n_gcf, size_t gcf_dim, int gcf_grid,
                         int pols, int debug1, int wphase, int mag, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if ((size_t)nthreads > img_dim) nthreads = (int)img_dim;
  band_job *jobs = (band_job *)calloc((size_t)nthreads, sizeof(band_job));
  pthread_t *tid = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
  for (int t = 0; t < nthreads; t++) {
    band_job j = {out_planar, uv, vals, gcf, npts, img_dim, gcf_dim,
                  gcf_grid, pols, debug1,
                  (long)(img_dim * (size_t)t / (size_t)nthreads),
                  (long)(img_dim * (size_t)(t + 1) / (size_t)nthreads),
                  gcfinx, n_gcf, wphase, mag};
    jobs[t] = j;
  }
  char *joined = (char *)calloc((size_t)nthreads, 1);
  for (int t = 1; t < nthreads; t++)
    if (pthread_create(&tid[t], NULL, band_thread, &jobs[t]) == 0)
      joined[t] = 1;
    else
      grid_band(&jobs[t]); /* no thread: do the band here */
  grid_band(&jobs[0]);
  for (int t = 1; t < nthreads; t++)
    if (joined[t]) pthread_join(tid[t], NULL);
  free(joined);
  free(jobs);
  free(tid);
}

void oracle_vis2ints(const double *uv, size_t npts, int gcf_grid,
                     int32_t *packed_xy) {
  for (size_t n = 0; n < npts; n++) {
    int mx, sx, my, sy;
    index_step(uv[2 * n], gcf_grid, &mx, &sx);
    index_step(uv[2 * n + 1], gcf_grid, &my, &sy);
    packed_xy[2 * n] = mx * gcf_grid + sx;
    packed_xy[2 * n + 1] = my * gcf_grid + sy;
  }
}

void oracle_vis2ints_gpu_formula(const double *uv, size_t npts, int gcf_grid,
                                 int32_t *packed_xy) {
  for (size_t n = 0; n < npts; n++) {
    /* grid_gpu.cu:358-363: main = floor(v) (to int), sub = floor(G*(v-main))
     * with the int main promoted back to double */
    int my = (int)floor(uv[2 * n + 1]);
    int sy = (int)floor(gcf_grid * (uv[2 * n + 1] - my));
    int mx = (int)floor(uv[2 * n]);
    int sx = (int)floor(gcf_grid * (uv[2 * n] - mx));
    packed_xy[2 * n] = mx * gcf_grid + sx;
    packed_xy[2 * n + 1] = my * gcf_grid + sy;
  }
}

void oracle_set_bookmarks(const int32_t *packed_xy, size_t npts, int gcf_grid,
                          int blocksize, int blockgrid, int32_t *bookmarks) {
  /* grid_gpu.cu:369-389, run serially over q = 0..npts.  The reference's
   * final step fills up to blockgrid*blockgrid + blockgrid; the restatement
   * stops at the last meaningful entry, ntiles = blockgrid^2. */
  const long ntiles = (long)blockgrid * blockgrid;
  for (size_t q = 0; q <= npts; q++) {
    int mx, my, mxl, myl;
    if (q == 0) {
      myl = 0;
      mxl = -1;
    } else {
      /* C integer division, as in the reference (truncates toward zero) */
      mxl = packed_xy[2 * (q - 1)] / gcf_grid / blocksize;
      myl = packed_xy[2 * (q - 1) + 1] / gcf_grid / blocksize;
    }
    if (q == npts) {
      mx = my = blockgrid;
    } else {
      mx = packed_xy[2 * q] / gcf_grid / blocksize;
      my = packed_xy[2 * q + 1] / gcf_grid / blocksize;
    }
    if (mx != mxl || my != myl) {
      for (long z = (long)myl * blockgrid + mxl + 1;
           z <= (long)my * blockgrid + mx && z <= ntiles; z++)
        bookmarks[z] = (int32_t)q;
    }
  }
}

void oracle_gcf_from_1d(double *gcf, const double *g1, int S, int G) {
  for (int sy = 0; sy < G; sy++)
    for (int sx = 0; sx < G; sx++)
      for (int bp = 0; bp < S; bp++)
        for (int ap = 0; ap < S; ap++) {
          size_t k = (size_t)S * S * (sy * G + sx) + (size_t)S * bp + ap;
          gcf[2 * k] = g1[sx * S + ap] * g1[sy * S + bp];
          gcf[2 * k + 1] = 0.0;
        }
}

void oracle_gaussian_gcf(double *gcf, double *g1, int S, int G,
                         double sigma) {
  double *g = g1 ? g1 : (double *)malloc(sizeof(double) * S * G);
  for (int s = 0; s < G; s++)
    for (int ap = 0; ap < S; ap++) {
      /* tap a = a'-S/2+1 lands on cell main+a; the visibility sits at
       * main + s/G, so the sample distance is a - s/G */
      double x = (double)(ap - S / 2 + 1) - (double)s / G;
      g[s * S + ap] = exp(-x * x / (2.0 * sigma * sigma));
    }
  if (gcf) oracle_gcf_from_1d(gcf, g, S, G);
  if (!g1) free(g);
}

/* ---- degridding (adjoint of the gridder) --------------------------------- */

typedef struct {
  double *vals;
  const double *grid, *uv, *gcf;
  const int32_t *gcfinx;
  size_t n0, n1, img_dim, gcf_dim;
  int n_gcf, G, P;
} degrid_job;

static void degrid_range(const degrid_job *j) {
  const long S = (long)j->gcf_dim, N = (long)j->img_dim;
  const int G = j->G, P = j->P;
  const size_t NN = (size_t)N * N;
  const double *re = j->grid, *im = j->grid + (size_t)P * NN;
  for (size_t n = j->n0; n < j->n1; n++) {
    int main_x, main_y, sub_x, sub_y;
    index_step(j->uv[2 * n], G, &main_x, &sub_x);
    index_step(j->uv[2 * n + 1], G, &main_y, &sub_y);
    int ok = sub_x >= 0 && sub_x < G && sub_y >= 0 && sub_y < G;
    long table = 0;
    if (ok && j->gcfinx) {
      ok = j->gcfinx[n] >= 0 && j->gcfinx[n] < j->n_gcf;
      table = ok ? (long)j->gcfinx[n] * G * G * S * S : 0;
    }
    for (int p = 0; p < P; p++) {
      double sr = 0, si = 0;
      if (ok) {
        const double *w = j->gcf + 2 * (table + S * S * ((long)G * sub_y + sub_x));
        for (long bp = 0; bp < S; bp++)
          for (long ap = 0; ap < S; ap++) {
            const long x = main_x + ap - S / 2 + 1, y = main_y + bp - S / 2 + 1;
            if (x < 0 || y < 0 || x >= N || y >= N) continue;
            const double wr = w[2 * (S * bp + ap)], wi = w[2 * (S * bp + ap) + 1];
            const size_t c = (size_t)p * NN + (size_t)y * N + (size_t)x;
            /* grid * conj(w) */
            sr += re[c] * wr + im[c] * wi;
            si += im[c] * wr - re[c] * wi;
          }
      }
      j->vals[2 * (P * n + p)] = sr;
      j->vals[2 * (P * n + p) + 1] = si;
    }
  }
}

static void *degrid_thread(void *arg) {
  degrid_range((const degrid_job *)arg);
  return NULL;
}

void oracle_degrid_pz(double *vals_out, const double *grid_planar,
                      const double *uv, const int32_t *gcfinx, size_t npts,
                      size_t img_dim, const double *gcf, int n_gcf,
                      size_t gcf_dim, int gcf_grid, int pols, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if ((size_t)nthreads > npts) nthreads = npts > 0 ? (int)npts : 1;
  degrid_job *jobs = (degrid_job *)calloc((size_t)nthreads, sizeof(degrid_job));
  pthread_t *tid = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
  for (int t = 0; t < nthreads; t++) {
    degrid_job *j = &jobs[t];
    j->vals = vals_out;
    j->grid = grid_planar;
    j->uv = uv;
    j->gcf = gcf;
    j->gcfinx = gcfinx;
    j->n0 = npts * (size_t)t / (size_t)nthreads;
    j->n1 = npts * (size_t)(t + 1) / (size_t)nthreads;
    j->img_dim = img_dim;
    j->gcf_dim = gcf_dim;
    j->n_gcf = n_gcf < 1 ? 1 : n_gcf;
    j->G = gcf_grid;
    j->P = pols;
  }
  for (int t = 1; t < nthreads; t++) pthread_create(&tid[t], NULL, degrid_thread, &jobs[t]);
  degrid_range(&jobs[0]);
  for (int t = 1; t < nthreads; t++) pthread_join(tid[t], NULL);
  free(jobs);
  free(tid);
}
