// Grid -> dirty image: the centred inverse 2-D DFT of every polarisation
// plane of a gridded job, in place.  Not part of the reference (it stops at
// the grid); it is the step that follows gridding in an imaging pipeline.
//
// With the zero spatial frequency at cell (N/2, N/2) and the image centre at
// pixel (N/2, N/2), for even N
//
//   image[m][l] = sum_{v,u} grid[v][u] exp(+2 pi i ((u-N/2)(l-N/2) + (v-N/2)(m-N/2)) / N)
//               = (-1)^(l+m) * IDFT[(-1)^(u+v) grid][m][l]
//
// (the two (-1)^(N/2) factors of the shifts cancel in 2-D), so the shifts
// become a sign flip of every other cell before and after an unnormalised
// inverse FFT.  The FFT itself is cuFFT's, loaded when first used so that
// libgg.so does not depend on it.
#include <dlfcn.h>

#include <cufft.h>

#include <mutex>
#include <string>

#include "gg_kernels.cuh"

namespace gg {

namespace {

template <typename T2>
__global__ void __launch_bounds__(256) checker_kernel(T2 *g, int64_t N, int64_t total) {
  for (int64_t i = blockIdx.x * 256ll + threadIdx.x; i < total; i += (int64_t)gridDim.x * 256) {
    const int64_t x = i % N, y = (i / N) % N;
    if ((x + y) & 1) {
      T2 v = g[i];
      v.x = -v.x;
      v.y = -v.y;
      g[i] = v;
    }
  }
}

struct CufftApi {
  decltype(&cufftPlanMany) plan_many = nullptr;
  decltype(&cufftSetStream) set_stream = nullptr;
  decltype(&cufftExecC2C) exec_c2c = nullptr;
  decltype(&cufftExecZ2Z) exec_z2z = nullptr;
  decltype(&cufftDestroy) destroy = nullptr;
  bool ok = false;
};

const CufftApi &cufft_api() {
  static CufftApi api;
  static std::once_flag once;
  std::call_once(once, [] {
    void *h = nullptr;
    for (const char *name : {"libcufft.so.12", "libcufft.so.13", "libcufft.so"}) {
      h = dlopen(name, RTLD_NOW | RTLD_LOCAL);
      if (h) break;
    }
    if (!h) return;
    api.plan_many = reinterpret_cast<decltype(api.plan_many)>(dlsym(h, "cufftPlanMany"));
    api.set_stream = reinterpret_cast<decltype(api.set_stream)>(dlsym(h, "cufftSetStream"));
    api.exec_c2c = reinterpret_cast<decltype(api.exec_c2c)>(dlsym(h, "cufftExecC2C"));
    api.exec_z2z = reinterpret_cast<decltype(api.exec_z2z)>(dlsym(h, "cufftExecZ2Z"));
    api.destroy = reinterpret_cast<decltype(api.destroy)>(dlsym(h, "cufftDestroy"));
    api.ok = api.plan_many && api.set_stream && api.exec_c2c && api.exec_z2z && api.destroy;
  });
  return api;
}

template <typename T2>
cudaError_t checker(void *grid, int64_t N, int P, int sm_count, cudaStream_t s) {
  const int64_t total = (int64_t)P * N * N;
  const int64_t b = (total + 255) / 256;
  const int64_t cap = (int64_t)sm_count * 8;
  checker_kernel<T2><<<(unsigned)(b < cap ? b : cap), 256, 0, s>>>(reinterpret_cast<T2 *>(grid),
                                                                  N, total);
  count_launch();
  return cudaGetLastError();
}

}  // namespace

// 0 on success; otherwise a message in err
int image_inverse_fft(void *grid, int64_t N, int P, bool f64, int sm_count, cudaStream_t s,
                      std::string &err) {
  const CufftApi &api = cufft_api();
  if (!api.ok) {
    err = "cuFFT (libcufft.so) could not be loaded";
    return 1;
  }
  cudaError_t e = f64 ? checker<double2>(grid, N, P, sm_count, s)
                      : checker<float2>(grid, N, P, sm_count, s);
  if (e != cudaSuccess) {
    err = std::string("sign flip: ") + cudaGetErrorString(e);
    return 1;
  }
  cufftHandle plan = 0;
  int n[2] = {(int)N, (int)N};
  const int dist = (int)(N * N);
  cufftResult r = api.plan_many(&plan, 2, n, nullptr, 1, dist, nullptr, 1, dist,
                                f64 ? CUFFT_Z2Z : CUFFT_C2C, P);
  if (r != CUFFT_SUCCESS) {
    err = "cufftPlanMany failed (" + std::to_string((int)r) + ")";
    return 1;
  }
  r = api.set_stream(plan, s);
  if (r == CUFFT_SUCCESS) {
    if (f64) {
      cufftDoubleComplex *g = reinterpret_cast<cufftDoubleComplex *>(grid);
      r = api.exec_z2z(plan, g, g, CUFFT_INVERSE);
    } else {
      cufftComplex *g = reinterpret_cast<cufftComplex *>(grid);
      r = api.exec_c2c(plan, g, g, CUFFT_INVERSE);
    }
  }
  if (r == CUFFT_SUCCESS)
    e = f64 ? checker<double2>(grid, N, P, sm_count, s) : checker<float2>(grid, N, P, sm_count, s);
  // the plan (and its work area) outlives the transform it enqueued
  const cudaError_t es = cudaStreamSynchronize(s);
  api.destroy(plan);
  if (r != CUFFT_SUCCESS) {
    err = "cuFFT execution failed (" + std::to_string((int)r) + ")";
    return 1;
  }
  if (e != cudaSuccess || es != cudaSuccess) {
    err = std::string("sign flip: ") + cudaGetErrorString(e != cudaSuccess ? e : es);
    return 1;
  }
  return 0;
}

}  // namespace gg
