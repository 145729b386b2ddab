// Device-side building blocks shared by the gridding kernels (sm_103a).
//
//  * the index step, bit-exact with the reference CPU gridder
//    (grid.cu:159-163) and its packed form (vis2ints, grid_gpu.cu:352-365)
//  * error-free transformations for FP32 compensated (hi/lo) accumulation
//  * native vector reductions (red.global.add.v2.f32 / red.global.add.f64)
//    replacing the reference's CAS loops (atomicAddWrap, grid_gpu.cu:53-90)
//  * 1-D bulk (TMA) copies global -> shared with mbarrier completion and
//    bounded waits
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "gg_types.h"

namespace gg {

// ---------------------------------------------------------------------------
// index step
// ---------------------------------------------------------------------------

// main = floor(u); sub = floorf(G * (u - floorf(u))), where floorf() gets its
// double argument converted to float (grid.cu:159-163).  Evaluated with the
// same conversions so that main and sub are bit-exact with the CPU gridder
// for every finite u.  For float-representable u the result also equals the
// GPU driver's all-double formula (grid_gpu.cu:118-121, 358-363).
// The step for float coordinates with |u| < 2^23, entirely in FP32.
// floorf(u) is exact, and so is u - floorf(u) except for -1/2 < u < 0, where
// 1 + u rounds to float exactly as the CPU gridder's double difference does
// when its product with the power of two G is converted to float (the scale
// commutes with the rounding; 1 + u may even round to 1, an oversample index
// of G, which the binning drops and counts).  So this equals the double
// formula below on (double)u.  (floor(G*u) in one conversion gives the same
// integers outside (-1/2, 0) and measured no faster in the binning pass.)
__device__ __forceinline__ void index_step_f32(float u, int G, int &m, int &s) {
  float fl = floorf(u);
  s = (int)floorf(__fmul_rn((float)G, __fsub_rn(u, fl)));
  m = (int)fl;
}

// Returns false when u is not finite or |u| >= 2^24 (no grid is that large;
// the bound keeps the packed main*G+sub inside int32 for G <= 64).
// GB300's FP64 pipe is narrow, so a coordinate that is exactly representable
// as a normal float with |u| < 2^23 -- the convention of the reference
// harness and of float-precision callers -- is recognised from its bits and
// takes the exact FP32 form; every other value takes the FP64 expression.
__device__ __forceinline__ bool index_step(double u, int G, int &m, int &s) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(u);
  const unsigned hi = (unsigned)(bits >> 32), lo = (unsigned)bits;
  const unsigned E = (hi >> 20) & 0x7ffu;
  if ((lo & 0x1fffffffu) == 0u && E >= 897u && E <= 1045u) {
    // 2^-126 <= |u| < 2^23 and the low 29 mantissa bits are zero
    const float f = __int_as_float((int)((hi & 0x80000000u) | ((E - 896u) << 23) |
                                         ((hi & 0x000fffffu) << 3) | (lo >> 29)));
    index_step_f32(f, G, m, s);
    return true;
  }
  if (!(u > -16777216.0 && u < 16777216.0)) return false;
  float uf = __double2float_rn(u);
  double frac = __dmul_rn((double)G, __dsub_rn(u, (double)floorf(uf)));
  s = (int)floorf(__double2float_rn(frac));
  m = (int)floor(u);
  return true;
}

// The same step for float coordinates.
__device__ __forceinline__ bool index_step(float u, int G, int &m, int &s) {
  if (!(u > -8388608.0f && u < 8388608.0f)) return false;
  index_step_f32(u, G, m, s);
  return true;
}

// packed = main*G + sub (vis2ints); decoding with an arithmetic shift is a
// floor division, valid for negative mains too (G is a power of two).
__device__ __forceinline__ int unpack_main(int packed, int log2G) {
  return packed >> log2G;
}
__device__ __forceinline__ int unpack_sub(int packed, int log2G) {
  return packed & ((1 << log2G) - 1);
}

// floor division by a power of two
__device__ __forceinline__ int fdiv_pow2(int a, int log2d) { return a >> log2d; }

// ---------------------------------------------------------------------------
// error-free transformations (Knuth TAOCP vol.2 4.2.2 "TwoSum")
// ---------------------------------------------------------------------------

// s + e == a + b exactly, s = fl(a + b).  Explicit _rn intrinsics keep the
// compiler from contracting or reassociating the sequence.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// ---- packed FP32x2 helpers (PTX f32x2, sm_100+) ------------------------------
typedef unsigned long long u64;
__device__ __forceinline__ u64 pk2(float a, float b) {
  u64 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float2 upk2(u64 r) {
  float2 f;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(f.x), "=f"(f.y) : "l"(r));
  return f;
}
__device__ __forceinline__ u64 add2(u64 a, u64 b) {
  u64 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ u64 sub2(u64 a, u64 b) {
  u64 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ u64 mul2(u64 a, u64 b) {
  u64 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ u64 fma2(u64 a, u64 b, u64 c) {
  u64 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
// (s, e) = TwoSum(a, b) on both lanes: s = fl(a+b), a + b = s + e exactly
__device__ __forceinline__ u64 two_sum2(u64 a, u64 b, u64 &e) {
  const u64 s = add2(a, b);
  const u64 bb = sub2(s, a);
  e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
  return s;
}

// ---------------------------------------------------------------------------
// accumulators: one complex running sum per thread and cell
// ---------------------------------------------------------------------------

// plain FP32 sum
struct AccF32 {
  using VT = float;
  float re, im;
  __device__ __forceinline__ void zero() { re = im = 0.f; }
  __device__ __forceinline__ void add(float tr, float ti) {
    re = __fadd_rn(re, tr);
    im = __fadd_rn(im, ti);
  }
  __device__ __forceinline__ bool nonzero() const { return re != 0.f || im != 0.f; }
  __device__ __forceinline__ double dre() const { return (double)re; }
  __device__ __forceinline__ double dim() const { return (double)im; }
  __device__ __forceinline__ float fre() const { return re; }
  __device__ __forceinline__ float fim() const { return im; }
};

// FP32 compensated sum: hi carries the running sum, lo the exact rounding
// errors of every addition into hi (two_sum), itself summed in FP32.
struct AccComp {
  using VT = float;
  float hr, hi_, lr, li;
  __device__ __forceinline__ void zero() { hr = hi_ = lr = li = 0.f; }
  __device__ __forceinline__ void add(float tr, float ti) {
    float e;
    two_sum(hr, tr, hr, e);
    lr = __fadd_rn(lr, e);
    two_sum(hi_, ti, hi_, e);
    li = __fadd_rn(li, e);
  }
  __device__ __forceinline__ bool nonzero() const {
    return hr != 0.f || hi_ != 0.f || lr != 0.f || li != 0.f;
  }
  __device__ __forceinline__ double dre() const { return (double)hr + (double)lr; }
  __device__ __forceinline__ double dim() const { return (double)hi_ + (double)li; }
  __device__ __forceinline__ float fre() const { return __fadd_rn(hr, lr); }
  __device__ __forceinline__ float fim() const { return __fadd_rn(hi_, li); }
};

// FP64 sum: the reference's <double2,double2> arithmetic
struct AccF64 {
  using VT = double;
  double re, im;
  __device__ __forceinline__ void zero() { re = im = 0.0; }
  __device__ __forceinline__ void add(double tr, double ti) {
    re = __dadd_rn(re, tr);
    im = __dadd_rn(im, ti);
  }
  __device__ __forceinline__ bool nonzero() const { return re != 0.0 || im != 0.0; }
  __device__ __forceinline__ double dre() const { return re; }
  __device__ __forceinline__ double dim() const { return im; }
  __device__ __forceinline__ float fre() const { return (float)re; }
  __device__ __forceinline__ float fim() const { return (float)im; }
};

// complex product val * gcf, as the reference writes it (r1*r2 - i1*i2,
// r1*i2 + r2*i1; grid_gpu.cu:162-163)
template <typename T>
__device__ __forceinline__ void cmul(T vr, T vi, T gr, T gi, T &tr, T &ti) {
  tr = vr * gr - vi * gi;
  ti = vr * gi + gr * vi;
}

// ---------------------------------------------------------------------------
// global reductions (fire-and-forget; the L2 performs the add)
// ---------------------------------------------------------------------------

__device__ __forceinline__ void red_add_v2(float *addr, float a, float b) {
  asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(addr), "f"(a), "f"(b)
               : "memory");
}
__device__ __forceinline__ void red_add(float *addr, float a) {
  asm volatile("red.global.add.f32 [%0], %1;" ::"l"(addr), "f"(a) : "memory");
}
__device__ __forceinline__ void red_add(double *addr, double a) {
  asm volatile("red.global.add.f64 [%0], %1;" ::"l"(addr), "d"(a) : "memory");
}
// atomic add returning the previous pair (for hi/lo two-sum in global memory)
__device__ __forceinline__ float2 atom_add_v2(float *addr, float a, float b) {
  float2 r;
  asm volatile("atom.global.v2.f32.add {%0, %1}, [%2], {%3, %4};"
               : "=f"(r.x), "=f"(r.y)
               : "l"(addr), "f"(a), "f"(b)
               : "memory");
  return r;
}

// Adds one complex value into cell `cell` of polarisation plane `p` of an
// output grid of N*N cells, in the requested type and layout:
//   interleaved: plane p holds N*N (re,im) pairs at out + p*N*N pairs
//   planar:      re plane [P][N][N] then im plane [P][N][N]
template <typename OT>
__device__ __forceinline__ void grid_red(OT *out, size_t cell, int p, int P,
                                         size_t NN, bool planar, double re,
                                         double im);
template <>
__device__ __forceinline__ void grid_red<float>(float *out, size_t cell, int p,
                                                int P, size_t NN, bool planar,
                                                double re, double im) {
  size_t c = (size_t)p * NN + cell;
  if (planar) {
    red_add(out + c, (float)re);
    red_add(out + (size_t)P * NN + c, (float)im);
  } else {
    red_add_v2(out + 2 * c, (float)re, (float)im);
  }
}
template <>
__device__ __forceinline__ void grid_red<double>(double *out, size_t cell, int p,
                                                 int P, size_t NN, bool planar,
                                                 double re, double im) {
  size_t c = (size_t)p * NN + cell;
  if (planar) {
    red_add(out + c, re);
    red_add(out + (size_t)P * NN + c, im);
  } else {
    red_add(out + 2 * c, re);
    red_add(out + 2 * c + 1, im);
  }
}

// one finished cell added to the grid's present value (gather into a grid it
// accumulates into): the sum formed in FP64, rounded once to the grid's type
template <typename OT>
__device__ __forceinline__ void grid_add(OT *out, size_t cell, int p, int P, size_t NN,
                                         bool planar, double re, double im) {
  const size_t c = (size_t)p * NN + cell;
  OT *a = planar ? out + c : out + 2 * c;
  OT *b = planar ? out + (size_t)P * NN + c : out + 2 * c + 1;
  *a = (OT)((double)*a + re);
  *b = (OT)((double)*b + im);
}

// plain store of one finished cell (gather writes every cell exactly once)
template <typename OT>
__device__ __forceinline__ void grid_store(OT *out, size_t cell, int p, int P,
                                           size_t NN, bool planar, OT re, OT im) {
  size_t c = (size_t)p * NN + cell;
  if (planar) {
    out[c] = re;
    out[(size_t)P * NN + c] = im;
  } else {
    out[2 * c] = re;
    out[2 * c + 1] = im;
  }
}

// ---------------------------------------------------------------------------
// 1-D bulk copies (TMA engine) with mbarrier completion
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                   smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
// one arrival (no transaction bytes), e.g. a consumer releasing a buffer
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
// src, dst 16-byte aligned; bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src,
                                         uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], "
      "[%1], %2, [%3];" ::"r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{ .reg .pred P; mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2; "
      "selp.u32 %0, 1, 0, P; }"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: every waiter gives up once kWaitLimitNs of wall-clock time
// (the global timer) have passed without the phase completing -- or after
// kSpinLimit polls, should the timer not advance -- raises the context's
// timeout flag and reports failure, so a lost completion can never hang the
// GPU.  A bulk copy of valid global memory completes in microseconds; the
// limit only guards against a bug.
constexpr uint64_t kWaitLimitNs = 500000000ull;  // 0.5 s
constexpr uint32_t kSpinLimit = 1u << 26;
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity,
                                          int *flags) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (uint32_t i = 1; i < kSpinLimit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 63) == 0 && global_ns() - t0 > kWaitLimitNs) break;
  }
  if (flags) atomicOr(&flags[FLAG_TIMEOUT], 1);
  return false;
}

// Copy bytes [b0, b1) of a global array to smem.  The bulk engine needs a
// 16-byte aligned source and length: the copied span is widened to the
// enclosing 16-byte boundaries (allocations carry >= 16 bytes of tail
// padding), and the returned offset locates byte b0 inside the smem buffer.
__device__ __forceinline__ uint32_t stage_span(void *dst_smem, const char *base,
                                               size_t b0, size_t b1,
                                               uint64_t *bar) {
  size_t a0 = b0 & ~(size_t)15;
  size_t a1 = (b1 + 15) & ~(size_t)15;
  uint32_t n = (uint32_t)(a1 - a0);
  if (n) bulk_g2s(dst_smem, base + a0, n, bar);
  return (uint32_t)(b0 - a0);
}

}  // namespace gg
