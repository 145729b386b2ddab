/*
 * Build-recipe helper (TEST INFRASTRUCTURE ONLY).  The reference's main()
 * calls gridGPU (grid.cu:481); the oracle library never runs that main, but
 * the symbol must resolve.  An empty template definition with the three
 * explicit instantiations the reference provides (grid_gpu.cu:820-825).
 */
#include <cstddef>
#include <cuda_runtime.h>
template <class CmplxOutType, class CmplxType>
void gridGPU(CmplxOutType *, CmplxType *, CmplxType *, size_t, size_t,
             CmplxType *, size_t) {}
template void gridGPU<double2, double2>(double2 *, double2 *, double2 *,
                                        size_t, size_t, double2 *, size_t);
template void gridGPU<double2, float2>(double2 *, float2 *, float2 *, size_t,
                                       size_t, float2 *, size_t);
template void gridGPU<float2, float2>(float2 *, float2 *, float2 *, size_t,
                                      size_t, float2 *, size_t);
