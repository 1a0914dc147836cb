// animate.cu — device-side scene animation: mangle (src/kernel/mangler.cl:
// 12-32), the per-frame vertex update of the reference's wave demo
// (src/rt/rt-wave.cpp:141-167, height 0.2 set at :408-413), applied to the
// scene's float4 positions and normals in place.  The kernel has no fp64
// pragma, so its constants are single precision; sinf / cosf are CUDA's
// (within a few ulp of the host's, see the tests), the rest is exactly
// rounded.  One thread per vertex; 64 B read and written per vertex.
#include <cuda_runtime.h>
#include <stdint.h>

#include "lbvh.cuh"

namespace rt {

__global__ void __launch_bounds__(256) k_mangle(float4* __restrict__ pos, float4* __restrict__ nrm,
                                                uint32_t V, float arg, float height) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    float4 p = pos[i], q = nrm[i];
    const int index = (int)i;
    p.y = height * sinf(0.33f * arg + p.x) * cosf(0.57f * arg + p.z);
    const float xfactor = (0.33f + fmodf(0.01238431f * (float)index, 0.23467f)) * arg;
    const float zfactor = (0.57f + fmodf(0.02173f * (float)index, 0.3237247f)) * arg;
    q.x = cosf(xfactor + p.x);
    q.z = -sinf(zfactor + p.z);
    pos[i] = p;
    nrm[i] = q;
}

cudaError_t launch_mangle(float4* pos, float4* nrm, uint32_t V, float arg, float height,
                          cudaStream_t s) {
    if (V == 0) return cudaSuccess;
    k_mangle<<<(V + 255) / 256, 256, 0, s>>>(pos, nrm, V, arg, height);
    return cudaGetLastError();
}

}  // namespace rt
