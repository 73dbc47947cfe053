// Nearest-point queries against a fixed point set, for the Chamfer loss of
// the differentiable workload (fitting a grid's iso-surface to points).  No
// counterpart in the reference, which is not differentiable.
//
// Exhaustive and tiled: the queries of a block (one per thread) meet every
// point of one slice of the point set, staged tile by tile in shared memory;
// the slices of the set go to different blocks, so a few thousand queries
// still fill every SM.  Each thread keeps its best (distance, index) and
// merges it into the query's result with one 64-bit atomicMin on
// (float bits of the squared distance << 32 | index): squared distances are
// non-negative, whose float bits order like their values, so the minimum is
// the smallest distance and, among equal distances, the smallest index.  The
// distance is (dx*dx + dy*dy) + dz*dz in float, each operation rounded.
// The cost does not depend on where the queries lie (a tree or grid search
// degrades when many points are nearly equidistant from far queries, as
// points on a torus are from a sphere's vertices around its axis).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "mdmc.h"
#include "mdmc_kernels.h"

struct mdmc_point_index {
    int64_t count = 0;
    float4* points = nullptr;  // x, y, z, original index (int bits)
};

namespace mdmc {
namespace {

constexpr int kNearestThreads = 256;
constexpr int kNearestTile = 256;  // points staged per round

__global__ void kPackPoints(const float* __restrict__ p, int n, float4* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = make_float4(p[3 * (int64_t)i], p[3 * (int64_t)i + 1], p[3 * (int64_t)i + 2], __int_as_float(i));
}

__global__ void kNearestInit(unsigned long long* best, int64_t count) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) best[i] = ~0ull;
}

// blockIdx.x: a group of kNearestThreads queries; blockIdx.y: a slice of the points
__global__ void __launch_bounds__(kNearestThreads) kNearestSlice(const float4* __restrict__ pts, int n, int sliceLen,
                                                                 const float* __restrict__ q, int64_t count,
                                                                 unsigned long long* __restrict__ best) {
    __shared__ float4 tile[kNearestTile];
    const int64_t i = (int64_t)blockIdx.x * kNearestThreads + threadIdx.x;
    const bool active = i < count;
    const float qx = active ? q[3 * i] : 0.f, qy = active ? q[3 * i + 1] : 0.f, qz = active ? q[3 * i + 2] : 0.f;
    const int p0 = blockIdx.y * sliceLen, p1 = min(n, p0 + sliceLen);
    float bd = INFINITY;
    int bi = 0x7FFFFFFF;
    for (int t0 = p0; t0 < p1; t0 += kNearestTile) {
        const int len = min(kNearestTile, p1 - t0);
        __syncthreads();
        if ((int)threadIdx.x < len) tile[threadIdx.x] = pts[t0 + threadIdx.x];
        __syncthreads();
#pragma unroll 8
        for (int k = 0; k < len; ++k) {
            const float4 p = tile[k];
            const float dx = qx - p.x, dy = qy - p.y, dz = qz - p.z;
            const float d = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            // points are visited in increasing index: a strictly smaller distance wins
            if (d < bd) {
                bd = d;
                bi = t0 + k;
            }
        }
    }
    if (active && bi != 0x7FFFFFFF)
        atomicMin(best + i, ((unsigned long long)__float_as_uint(bd) << 32) | (unsigned)bi);
}

__global__ void kNearestFinish(const unsigned long long* __restrict__ best, int64_t count, int32_t* __restrict__ nearest,
                               float* __restrict__ d2) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const unsigned long long b = best[i];
    nearest[i] = (int32_t)(uint32_t)(b & 0xFFFFFFFFull);
    if (d2) d2[i] = __uint_as_float((uint32_t)(b >> 32));
}

}  // namespace
}  // namespace mdmc

using namespace mdmc;

extern "C" MDMC_API mdmc_status mdmc_point_index_create(mdmc_point_index** out, const float* points, int64_t count,
                                                        void* stream) {
    if (!out) return MDMC_ERROR_INVALID_ARGUMENT;
    *out = nullptr;
    if (!points || count < 1 || count > 0x7FFFFFFF) return MDMC_ERROR_INVALID_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    mdmc_point_index* ix = new mdmc_point_index();
    ix->count = count;
    cudaError_t e = cudaMalloc(&ix->points, sizeof(float4) * (size_t)count);
    if (e == cudaSuccess) {
        countLaunch();
        kPackPoints<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(points, (int)count, ix->points);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        mdmc_point_index_destroy(ix);
        return e == cudaErrorMemoryAllocation ? MDMC_ERROR_OUT_OF_MEMORY : MDMC_ERROR_CUDA;
    }
    *out = ix;
    return MDMC_OK;
}

extern "C" MDMC_API void mdmc_point_index_destroy(mdmc_point_index* ix) {
    if (!ix) return;
    cudaFree(ix->points);
    delete ix;
}

extern "C" MDMC_API mdmc_status mdmc_point_index_nearest(const mdmc_point_index* ix, const float* queries,
                                                         int64_t count, int32_t* nearest, float* dist2,
                                                         uint64_t* scratch, void* stream) {
    if (!ix || (count > 0 && (!queries || !nearest || !scratch)) || count < 0 || count > 0x7FFFFFFF)
        return MDMC_ERROR_INVALID_ARGUMENT;
    if (count == 0) return MDMC_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const int n = (int)ix->count;
    // enough slices of the points for about four blocks per SM
    const int64_t groups = (count + kNearestThreads - 1) / kNearestThreads;
    int slices = (int)std::max<int64_t>(1, std::min<int64_t>((152 * 4 + groups - 1) / groups,
                                                             ((int64_t)n + kNearestTile - 1) / kNearestTile));
    slices = std::min(slices, 65535);
    const int sliceLen = (int)(((int64_t)n + slices - 1) / slices);
    countLaunch(3);
    unsigned long long* best = reinterpret_cast<unsigned long long*>(scratch);
    kNearestInit<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(best, count);
    kNearestSlice<<<dim3((unsigned)groups, (unsigned)slices), kNearestThreads, 0, s>>>(ix->points, n, sliceLen, queries,
                                                                                        count, best);
    kNearestFinish<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(best, count, nearest, dist2);
    return cudaGetLastError() == cudaSuccess ? MDMC_OK : MDMC_ERROR_CUDA;
}

extern "C" MDMC_API int64_t mdmc_point_index_count(const mdmc_point_index* ix) { return ix ? ix->count : 0; }
