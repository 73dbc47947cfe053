// Nearest-point queries against a fixed point set, for the Chamfer loss of
// the differentiable workload (fitting a grid's iso-surface to points).  No
// counterpart in the reference, which is not differentiable.
//
// Tiled, exact, with pruning that cannot change the answer.  The index keeps
// the points sorted along a Morton curve in tiles of 128 (nearby points share
// a tile) with each tile's bounding box.  The queries are grouped by a coarse
// Morton key, so that a block's queries lie close together.  A query first
// takes the nearest of the tiles' first points as an upper bound; then the
// queries of a block (one per thread) go through one slice of the tiles,
// staging in shared memory only the tiles some query of the block still
// needs: a tile whose box is farther from every query than that query's bound
// cannot hold its nearest point.  Each thread keeps its best (distance, index) and merges it into the
// query's result with one 64-bit atomicMin on (float bits of the squared
// distance << 32 | index): squared distances are non-negative, whose float
// bits order like their values, so the minimum is the smallest distance and,
// among equal distances, the smallest index.  The distance is
// (dx*dx + dy*dy) + dz*dz in float, each operation rounded.
//
// Why the pruning is exact: for the point c of a box nearest to q (q clamped
// to the box), |q - c| <= |q - p| per axis for every p in the box, and every
// float operation of the distance is monotonic, so the box's float distance is
// at most the float distance of each of its points.  A tile is skipped only
// when that bound exceeds the query's current best distance strictly, so no
// point at the best distance (a tie included) is ever skipped.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

#include "mdmc.h"
#include "mdmc_kernels.h"

namespace mdmc {
constexpr int kPointTile = 128;  // points per tile (and staged per round)
}

struct mdmc_point_index {
    int64_t count = 0;
    int tiles = 0;
    float4* points = nullptr;   // x, y, z, original index (int bits); Morton order
    float4* boxes = nullptr;    // per tile: min x, y, z, -, max x, y, z, - (two float4)
    float lo[3] = {0, 0, 0}, scale[3] = {0, 0, 0};  // the points' box, for the queries' bucket keys
};

namespace mdmc {
namespace {

constexpr int kNearestThreads = 128;  // queries per block (128 and 128: 2.17 -> 1.90 ms per fit step against 256 and 256)

__device__ __forceinline__ float dist2(float qx, float qy, float qz, float px, float py, float pz) {
    const float dx = qx - px, dy = qy - py, dz = qz - pz;
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// (distance, index) packed for atomicMin; ~0 (no candidate) for a distance
// that is not finite (a NaN coordinate, or an overflow): such a point never
// wins, as no strictly smaller distance than the initial infinity is found
__device__ __forceinline__ unsigned long long packBest(float d, int index) {
    return d < INFINITY ? ((unsigned long long)__float_as_uint(d) << 32) | (uint32_t)index : ~0ull;
}

// Queries go to blocks in the order of a 12-bit Morton key (4 bits per axis
// of their place in the points' box), so that a block's queries lie close
// together and need fewer tiles; a counting sort (the order inside a bucket
// does not matter: every query's result is exact wherever it is computed).
constexpr int kQueryBuckets = 4096;
struct QueryKey {
    float lo[3], scale[3];  // scale maps the box to [0, 16)
    __device__ __forceinline__ int operator()(float x, float y, float z) const {
        const float v[3] = {x, y, z};
        int code = 0;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            float f = (v[a] - lo[a]) * scale[a];
            f = f >= 0.f ? (f < 15.f ? f : 15.f) : 0.f;  // (NaN lands at 0)
            const int u = (int)f;
#pragma unroll
            for (int b = 0; b < 4; ++b) code |= ((u >> b) & 1) << (3 * b + a);
        }
        return code;
    }
};
__global__ void kQueryHistogram(const float* __restrict__ q, int64_t count, QueryKey key, int* __restrict__ hist) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) atomicAdd(hist + key(q[3 * i], q[3 * i + 1], q[3 * i + 2]), 1);
}
// one block of 1024 threads: exclusive prefix of the 4096 bucket counts, in place
__global__ void __launch_bounds__(1024) kQueryBucketScan(int* __restrict__ hist) {
    __shared__ int part[1024];
    const int t = threadIdx.x;
    const int4 v = reinterpret_cast<int4*>(hist)[t];
    const int sum = v.x + v.y + v.z + v.w;
    part[t] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {  // inclusive Hillis-Steele scan
        const int add = t >= o ? part[t - o] : 0;
        __syncthreads();
        part[t] += add;
        __syncthreads();
    }
    const int base = part[t] - sum;
    reinterpret_cast<int4*>(hist)[t] = make_int4(base, base + v.x, base + v.x + v.y, base + v.x + v.y + v.z);
}
__global__ void kQueryScatter(const float* __restrict__ q, int64_t count, QueryKey key, int* __restrict__ offsets,
                              int* __restrict__ perm) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) perm[atomicAdd(offsets + key(q[3 * i], q[3 * i + 1], q[3 * i + 2]), 1)] = (int)i;
}

// the upper bound: the nearest of the tiles' first points (a real candidate)
__global__ void __launch_bounds__(kNearestThreads) kNearestSeed(const float4* __restrict__ pts, int tiles,
                                                                const float* __restrict__ q, const int* __restrict__ perm,
                                                                int64_t count, unsigned long long* __restrict__ best) {
    __shared__ float4 rep[kNearestThreads];
    const int64_t j = (int64_t)blockIdx.x * kNearestThreads + threadIdx.x;
    const bool active = j < count;
    const int64_t i = active ? (perm ? perm[j] : j) : 0;
    const float qx = active ? q[3 * i] : 0.f, qy = active ? q[3 * i + 1] : 0.f, qz = active ? q[3 * i + 2] : 0.f;
    unsigned long long b = ~0ull;
    for (int t0 = 0; t0 < tiles; t0 += kNearestThreads) {
        const int len = min(kNearestThreads, tiles - t0);
        __syncthreads();
        if ((int)threadIdx.x < len) rep[threadIdx.x] = pts[(int64_t)(t0 + threadIdx.x) * kPointTile];
        __syncthreads();
        for (int k = 0; k < len; ++k) {
            const float4 p = rep[k];
            const unsigned long long c = packBest(dist2(qx, qy, qz, p.x, p.y, p.z), __float_as_int(p.w));
            b = c < b ? c : b;
        }
    }
    if (active) best[i] = b;
}

// blockIdx.x: a group of kNearestThreads queries; blockIdx.y: a slice of the tiles
__global__ void __launch_bounds__(kNearestThreads) kNearestSlice(const float4* __restrict__ pts, int n,
                                                                 const float4* __restrict__ boxes, int tiles,
                                                                 int tilesPerSlice, const float* __restrict__ q,
                                                                 const int* __restrict__ perm, int64_t count,
                                                                 unsigned long long* __restrict__ best) {
    __shared__ float4 tile[kPointTile];
    const int64_t j = (int64_t)blockIdx.x * kNearestThreads + threadIdx.x;
    const bool active = j < count;
    const int64_t i = active ? (perm ? perm[j] : j) : 0;
    const float qx = active ? q[3 * i] : 0.f, qy = active ? q[3 * i + 1] : 0.f, qz = active ? q[3 * i + 2] : 0.f;
    unsigned long long bk = active ? best[i] : ~0ull;  // the seed: (distance, index) of a real point
    const int s0 = blockIdx.y * tilesPerSlice, s1 = min(tiles, s0 + tilesPerSlice);
    for (int t = s0; t < s1; ++t) {
        const float4 lo = boxes[2 * t], hi = boxes[2 * t + 1];
        const float cx = fminf(fmaxf(qx, lo.x), hi.x), cy = fminf(fmaxf(qy, lo.y), hi.y),
                    cz = fminf(fmaxf(qz, lo.z), hi.z);
        const float bound = dist2(qx, qy, qz, cx, cy, cz);
        // (no candidate yet: no bound to prune with)
        const bool need = active && (bk == ~0ull || !(bound > __uint_as_float((uint32_t)(bk >> 32))));
        if (!__syncthreads_or(need)) continue;  // (the barrier also ends the last tile's reads)
        const int base = t * kPointTile, len = min(kPointTile, n - base);
        if ((int)threadIdx.x < len) tile[threadIdx.x] = pts[base + threadIdx.x];
        __syncthreads();
        if (need) {
#pragma unroll 8
            for (int k = 0; k < len; ++k) {
                const float4 p = tile[k];
                const unsigned long long c = packBest(dist2(qx, qy, qz, p.x, p.y, p.z), __float_as_int(p.w));
                bk = c < bk ? c : bk;
            }
        }
    }
    if (active) atomicMin(best + i, bk);
}

__global__ void kNearestFinish(const unsigned long long* __restrict__ best, int64_t count, int32_t* __restrict__ nearest,
                               float* __restrict__ d2) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const unsigned long long b = best[i];
    nearest[i] = (int32_t)(uint32_t)(b & 0xFFFFFFFFull);
    if (d2) d2[i] = __uint_as_float((uint32_t)(b >> 32));
}

// 10 bits per axis of the point's place in the set's bounding box, interleaved
uint32_t morton30(float x, float y, float z, const float lo[3], const float scale[3]) {
    const float v[3] = {x, y, z};
    uint32_t code = 0;
    for (int a = 0; a < 3; ++a) {
        float f = (v[a] - lo[a]) * scale[a];
        f = f < 0.f ? 0.f : (f > 1023.f ? 1023.f : f);  // (NaN coordinates land at 0)
        const uint32_t u = (uint32_t)f;
        for (int b = 0; b < 10; ++b) code |= ((u >> b) & 1u) << (3 * b + a);
    }
    return code;
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
    // the points on the host: Morton order, tiles and their boxes (a one-time build)
    std::vector<float> host(3 * (size_t)count);
    cudaError_t e = cudaMemcpyAsync(host.data(), points, sizeof(float) * host.size(), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return MDMC_ERROR_CUDA;
    }
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY}, scale[3];
    for (int64_t i = 0; i < count; ++i)
        for (int a = 0; a < 3; ++a) {
            const float v = host[3 * i + a];
            if (v < lo[a]) lo[a] = v;
            if (v > hi[a]) hi[a] = v;
        }
    for (int a = 0; a < 3; ++a) {
        if (!(hi[a] >= lo[a])) lo[a] = hi[a] = 0.f;  // no finite coordinate
        scale[a] = hi[a] > lo[a] ? 1023.f / (hi[a] - lo[a]) : 0.f;
    }
    std::vector<uint32_t> code((size_t)count);
    for (int64_t i = 0; i < count; ++i) code[i] = morton30(host[3 * i], host[3 * i + 1], host[3 * i + 2], lo, scale);
    std::vector<int> order((size_t)count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return code[a] < code[b]; });
    const int tiles = (int)((count + kPointTile - 1) / kPointTile);
    std::vector<float4> sorted((size_t)count), boxes(2 * (size_t)tiles);
    for (int64_t k = 0; k < count; ++k) {
        const int i = order[k];
        float4 p;
        p.x = host[3 * (size_t)i];
        p.y = host[3 * (size_t)i + 1];
        p.z = host[3 * (size_t)i + 2];
        int iw = i;
        std::memcpy(&p.w, &iw, sizeof(int));
        sorted[k] = p;
    }
    for (int t = 0; t < tiles; ++t) {
        float4 bl, bh;
        bl.x = bl.y = bl.z = INFINITY;
        bh.x = bh.y = bh.z = -INFINITY;
        bl.w = bh.w = 0.f;
        bool nan = false;
        for (int64_t k = (int64_t)t * kPointTile; k < std::min<int64_t>(count, (int64_t)(t + 1) * kPointTile); ++k) {
            const float4 p = sorted[k];
            nan = nan || p.x != p.x || p.y != p.y || p.z != p.z;
            bl.x = std::min(bl.x, p.x); bl.y = std::min(bl.y, p.y); bl.z = std::min(bl.z, p.z);
            bh.x = std::max(bh.x, p.x); bh.y = std::max(bh.y, p.y); bh.z = std::max(bh.z, p.z);
        }
        if (nan) {  // a NaN point: a box no query can rule out
            bl.x = bl.y = bl.z = -INFINITY;
            bh.x = bh.y = bh.z = INFINITY;
        }
        boxes[2 * (size_t)t] = bl;
        boxes[2 * (size_t)t + 1] = bh;
    }
    mdmc_point_index* ix = new mdmc_point_index();
    ix->count = count;
    ix->tiles = tiles;
    for (int a = 0; a < 3; ++a) {
        ix->lo[a] = lo[a];
        ix->scale[a] = hi[a] > lo[a] ? 16.f / (hi[a] - lo[a]) : 0.f;
    }
    e = cudaMalloc(&ix->points, sizeof(float4) * (size_t)count);
    if (e == cudaSuccess) e = cudaMalloc(&ix->boxes, sizeof(float4) * boxes.size());
    if (e == cudaSuccess) e = cudaMemcpy(ix->points, sorted.data(), sizeof(float4) * sorted.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(ix->boxes, boxes.data(), sizeof(float4) * boxes.size(), cudaMemcpyHostToDevice);
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
    cudaFree(ix->boxes);
    delete ix;
}

extern "C" MDMC_API mdmc_status mdmc_point_index_nearest(const mdmc_point_index* ix, const float* queries,
                                                         int64_t count, int32_t* nearest, float* dist2,
                                                         uint64_t* scratch, void* stream) {
    if (!ix || (count > 0 && (!queries || !nearest || !scratch)) || count < 0 || count > 0x7FFFFFFF)
        return MDMC_ERROR_INVALID_ARGUMENT;
    if (count == 0) return MDMC_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const int n = (int)ix->count, tiles = ix->tiles;
    // enough slices of the tiles for about four blocks per SM
    const int64_t groups = (count + kNearestThreads - 1) / kNearestThreads;
    int slices = (int)std::max<int64_t>(1, std::min<int64_t>((152 * 4 + groups - 1) / groups, tiles));
    slices = std::min(slices, 65535);
    const int tilesPerSlice = (tiles + slices - 1) / slices;
    slices = (tiles + tilesPerSlice - 1) / tilesPerSlice;
    unsigned long long* best = reinterpret_cast<unsigned long long*>(scratch);
    // scratch: best (count words), the permutation (count ints), the bucket
    // counts (4096 ints, from a 16-byte boundary)
    int* perm = reinterpret_cast<int*>(scratch + count);
    int* hist = reinterpret_cast<int*>(scratch + count + (count + 1) / 2 + 1);
    hist = reinterpret_cast<int*>((reinterpret_cast<uintptr_t>(hist) + 15) & ~(uintptr_t)15);
    QueryKey key;
    for (int a = 0; a < 3; ++a) {
        key.lo[a] = ix->lo[a];
        key.scale[a] = ix->scale[a];
    }
    if (cudaMemsetAsync(hist, 0, sizeof(int) * kQueryBuckets, s) != cudaSuccess) return MDMC_ERROR_CUDA;
    countLaunch(6);
    const unsigned qb = (unsigned)((count + 255) / 256);
    kQueryHistogram<<<qb, 256, 0, s>>>(queries, count, key, hist);
    kQueryBucketScan<<<1, 1024, 0, s>>>(hist);
    kQueryScatter<<<qb, 256, 0, s>>>(queries, count, key, hist, perm);
    kNearestSeed<<<(unsigned)groups, kNearestThreads, 0, s>>>(ix->points, tiles, queries, perm, count, best);
    kNearestSlice<<<dim3((unsigned)groups, (unsigned)slices), kNearestThreads, 0, s>>>(
        ix->points, n, ix->boxes, tiles, tilesPerSlice, queries, perm, count, best);
    kNearestFinish<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(best, count, nearest, dist2);
    return cudaGetLastError() == cudaSuccess ? MDMC_OK : MDMC_ERROR_CUDA;
}

extern "C" MDMC_API int64_t mdmc_point_index_count(const mdmc_point_index* ix) { return ix ? ix->count : 0; }
