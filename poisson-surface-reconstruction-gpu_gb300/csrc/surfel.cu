// DepthSurfel (base/CommonTypes.h:113-118) -> the SoA arrays of psr_points, on the device.
//
// The reference's surfel is 64 bytes: pixel (row, col), VertexAndConfidence (x y z, w),
// NormalAndRadius (nx ny nz, radius), ColorAndTime (r g b in [0, 1], time); its
// getCoordinateAndNormalKernel (mesh/BuildOctree.cu:135-143) reads position, normal and
// colour from it.  Colour becomes 8-bit here (round(255 c), clamped), the form psr_points
// takes.
#include <cuda_runtime.h>

#include "../../include/psr/psr.h"
#include "psr_common.cuh"

namespace psr {

struct SurfelRaw {
    unsigned row, col;
    float4 vc, nr, ct;
};
static_assert(sizeof(SurfelRaw) == 64, "DepthSurfel layout");

__global__ void __launch_bounds__(kBlock) k_surfels_to_points(const SurfelRaw* s, int n, float* xyz, float* nrm,
                                                              uint8_t* rgb) {
    PSR_GRID_STRIDE(i, n) {
        const float4 v = s[i].vc, q = s[i].nr;
        xyz[3 * (size_t)i] = v.x;
        xyz[3 * (size_t)i + 1] = v.y;
        xyz[3 * (size_t)i + 2] = v.z;
        nrm[3 * (size_t)i] = q.x;
        nrm[3 * (size_t)i + 1] = q.y;
        nrm[3 * (size_t)i + 2] = q.z;
        if (rgb) {
            const float4 c = s[i].ct;
            const float ch[3] = {c.x, c.y, c.z};
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                float u = rintf(ch[a] * 255.0f);
                u = fminf(fmaxf(u, 0.0f), 255.0f);   // NaN -> 0
                rgb[3 * (size_t)i + a] = (uint8_t)u;
            }
        }
    }
}

}  // namespace psr

extern "C" psr_status psr_surfels_to_points(const void* surfels, int count, float* xyz, float* normals, uint8_t* rgb,
                                            void* stream) {
    if (count < 0 || (count > 0 && (!surfels || !xyz || !normals))) return PSR_INVALID_INPUT;
    if (count == 0) return PSR_OK;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return PSR_CUDA_ERROR;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long blocks = ((long long)count + psr::kBlock - 1) / psr::kBlock;
    const long long cap = (long long)(sms > 0 ? sms : 148) * 8;
    if (blocks > cap) blocks = cap;
    psr::k_surfels_to_points<<<(int)blocks, psr::kBlock, 0, (cudaStream_t)stream>>>(
        (const psr::SurfelRaw*)surfels, count, xyz, normals, rgb);
    return cudaGetLastError() == cudaSuccess ? PSR_OK : PSR_CUDA_ERROR;
}
