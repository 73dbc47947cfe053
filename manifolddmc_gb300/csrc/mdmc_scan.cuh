// Exclusive prefix sums over int, int2 and int4 arrays, in three phases: per-tile
// reduction, one-block scan of the tile sums, per-tile scan with the tile's
// offset.  out has n+1 entries; out[n] is the total.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "mdmc_kernels.h"

namespace mdmc {

constexpr int kScanThreads = 512;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr int kScanMaxTiles = 1 << 20;  // largest tile-sum array the one-block pass scans (2^31 elements)

template <typename T>
struct ScanOps;
template <>
struct ScanOps<int> {
    __device__ static int zero() { return 0; }
    __device__ static int add(int a, int b) { return a + b; }
};
template <>
struct ScanOps<int2> {
    __device__ static int2 zero() { return make_int2(0, 0); }
    __device__ static int2 add(int2 a, int2 b) { return make_int2(a.x + b.x, a.y + b.y); }
};
template <>
struct ScanOps<int4> {
    __device__ static int4 zero() { return make_int4(0, 0, 0, 0); }
    __device__ static int4 add(int4 a, int4 b) { return make_int4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
};

__device__ __forceinline__ int shflUp(int v, int o) { return __shfl_up_sync(0xffffffffu, v, o); }
__device__ __forceinline__ int2 shflUp(int2 v, int o) {
    return make_int2(__shfl_up_sync(0xffffffffu, v.x, o), __shfl_up_sync(0xffffffffu, v.y, o));
}
__device__ __forceinline__ int4 shflUp(int4 v, int o) {
    return make_int4(__shfl_up_sync(0xffffffffu, v.x, o), __shfl_up_sync(0xffffffffu, v.y, o),
                     __shfl_up_sync(0xffffffffu, v.z, o), __shfl_up_sync(0xffffffffu, v.w, o));
}
__device__ __forceinline__ int minus(int a, int b) { return a - b; }
__device__ __forceinline__ int2 minus(int2 a, int2 b) { return make_int2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ int4 minus(int4 a, int4 b) { return make_int4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }

template <typename T>
__device__ T warpInclusive(T v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T u = shflUp(v, o);
        if (lane >= o) v = ScanOps<T>::add(v, u);
    }
    return v;
}

// block-wide exclusive scan of one value per thread; returns the block total
template <typename T>
__device__ T blockExclusive(T v, T& total) {
    __shared__ T warpSums[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    T inc = warpInclusive(v);
    if (lane == 31) warpSums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        T w = lane < nw ? warpSums[lane] : ScanOps<T>::zero();
        T wi = warpInclusive(w);
        warpSums[lane] = wi;
    }
    __syncthreads();
    T before = warp > 0 ? warpSums[warp - 1] : ScanOps<T>::zero();
    total = warpSums[nw - 1];
    __syncthreads();
    // exclusive = inclusive - own value
    return ScanOps<T>::add(before, minus(inc, v));
}

// element readers: an array, or the popcounts of a bit-mask's words (the
// per-word counts are then never stored).  A reader of 4-byte elements may
// also read four at once (four(i, v): elements i..i+3, i a multiple of 4,
// one 16-byte load per array); vectorOk() says on the host whether its
// arrays are 16-byte aligned, which that needs.
template <typename T>
struct ArrayRead {
    static constexpr bool kFour = sizeof(T) == 4;
    const T* __restrict__ p;
    __device__ __forceinline__ T operator[](int64_t i) const { return p[i]; }
    __device__ __forceinline__ void four(int64_t i, T v[4]) const {
        const int4 q = *reinterpret_cast<const int4*>(p + i);
        v[0] = (T)q.x;
        v[1] = (T)q.y;
        v[2] = (T)q.z;
        v[3] = (T)q.w;
    }
    bool vectorOk() const { return kFour && (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }
};
struct PopcRead {
    static constexpr bool kFour = true;
    const uint32_t* __restrict__ p;
    __device__ __forceinline__ int operator[](int64_t i) const { return __popc(p[i]); }
    __device__ __forceinline__ void four(int64_t i, int v[4]) const {
        const uint4 q = *reinterpret_cast<const uint4*>(p + i);
        v[0] = __popc(q.x);
        v[1] = __popc(q.y);
        v[2] = __popc(q.z);
        v[3] = __popc(q.w);
    }
    bool vectorOk() const { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }
};

// elements i..i+3 (i a multiple of 4) into v, zero past n: one vector load
// per array when the reader has one and all four lie below n
template <typename T, class In>
__device__ __forceinline__ void loadFour(const In& in, bool vec, int64_t i, int64_t n, T v[4]) {
    if constexpr (In::kFour) {
        if (vec && i + 3 < n) {
            in.four(i, v);
            return;
        }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = i + k < n ? in[i + k] : ScanOps<T>::zero();
}

// called by the apply pass with every element's exclusive prefix and value,
// and once with the element count and the total; kPrefixes false: the apply
// pass writes only out[n], the total
struct NoPost {
    static constexpr bool kStaged = false;
    static constexpr bool kPrefixes = true;
    template <typename T>
    __device__ __forceinline__ void operator()(int64_t, T, T) const {}
    template <typename T>
    __device__ __forceinline__ void total(int64_t, T) const {}
};

// the element count: known on the host (dev == nullptr), or read on the
// device from *dev and capped at max (the launch covers max elements)
struct ScanCount {
    int64_t max;
    const int* dev;
    __device__ __forceinline__ int64_t get() const {
        if (!dev) return max;
        const int64_t n = *dev;
        return n < 0 ? 0 : (n < max ? n : max);
    }
};

__device__ __forceinline__ int64_t scanTiles(int64_t n) { return (n + kScanTile - 1) / kScanTile; }

template <typename T, class In>
__global__ void __launch_bounds__(kScanThreads) kScanReduce(In in, ScanCount cnt, T* __restrict__ tileSums, bool vec) {
    const int64_t n = cnt.get();
    if (blockIdx.x > 0 && blockIdx.x >= scanTiles(n)) return;
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    T acc = ScanOps<T>::zero();
    if (vec) {  // each thread its four consecutive elements (kScanItems == 4)
        T v[4];
        loadFour<T>(in, vec, base + (int64_t)threadIdx.x * kScanItems, n, v);
#pragma unroll
        for (int k = 0; k < 4; ++k) acc = ScanOps<T>::add(acc, v[k]);
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            int64_t i = base + (int64_t)k * kScanThreads + threadIdx.x;
            if (i < n) acc = ScanOps<T>::add(acc, in[i]);
        }
    }
    T total;
    blockExclusive(acc, total);
    if (threadIdx.x == 0) tileSums[blockIdx.x] = total;
}

// one block: exclusive scan of the tile sums in place, total -> tileSums[numTiles].
// Chunks of 1024 sums are scanned one after the other with a running carry,
// one value per thread and chunk (the block launches with 1024 threads, so a
// thread may hold at most 64 registers).
template <typename T>
__global__ void __launch_bounds__(1024) kScanTiles(T* tileSums, ScanCount cnt) {
    const int numTiles = (int)scanTiles(cnt.get());
    __shared__ T carryShared;
    if (threadIdx.x == 0) carryShared = ScanOps<T>::zero();
    __syncthreads();
    for (int base = 0; base < numTiles; base += 1024) {
        const int i = base + threadIdx.x;
        const T v = i < numTiles ? tileSums[i] : ScanOps<T>::zero();
        T total;
        const T exc = blockExclusive(v, total);
        const T carry = carryShared;
        if (i < numTiles) tileSums[i] = ScanOps<T>::add(carry, exc);
        __syncthreads();
        if (threadIdx.x == 0) carryShared = ScanOps<T>::add(carry, total);
        __syncthreads();
    }
    if (threadIdx.x == 0) tileSums[numTiles] = carryShared;
}

// Each thread scans kScanItems consecutive elements straight from memory.
template <typename T, class In, class Post>
__global__ void __launch_bounds__(kScanThreads) kScanApply(In in, ScanCount cnt, const T* __restrict__ tileSums,
                           T* __restrict__ out, Post post, bool vec) {
    const int64_t n = cnt.get();
    const int nTiles = (int)scanTiles(n);
    const int lastBlock = nTiles > 0 ? nTiles - 1 : 0;
    if ((int)blockIdx.x > lastBlock) return;
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    // each thread owns kScanItems (= 4) consecutive elements
    static_assert(kScanItems == 4, "loadFour reads four elements");
    T vals[kScanItems];
    loadFour<T>(in, vec, base + (int64_t)threadIdx.x * kScanItems, n, vals);
    T acc = ScanOps<T>::zero();
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) acc = ScanOps<T>::add(acc, vals[k]);
    T total;
    T run = ScanOps<T>::add(tileSums[blockIdx.x], blockExclusive(acc, total));
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + (int64_t)threadIdx.x * kScanItems + k;
        if (i < n) {
            if constexpr (Post::kPrefixes) out[i] = run;
            post(i, run, vals[k]);
        }
        run = ScanOps<T>::add(run, vals[k]);
    }
    if ((int)blockIdx.x == lastBlock && threadIdx.x == 0) {
        out[n] = tileSums[nTiles];
        post.total(n, tileSums[nTiles]);
    }
}

// The same with the tile going through shared memory twice: loaded and
// stored by consecutive threads (coalesced), scanned by each thread over
// kScanItems consecutive elements; post gets each element's value as the
// difference of consecutive prefixes.  For posts that write per-element
// records (Post::kStaged), whose stores the direct kernel would stride.
template <typename T, class In, class Post>
__global__ void __launch_bounds__(kScanThreads) kScanApplyStaged(In in, ScanCount cnt, const T* __restrict__ tileSums,
                                 T* __restrict__ out, Post post) {
    __shared__ T stage[kScanTile];
    const int64_t n = cnt.get();
    const int nTiles = (int)scanTiles(n);
    const int lastBlock = nTiles > 0 ? nTiles - 1 : 0;
    if ((int)blockIdx.x > lastBlock) return;
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + (int64_t)k * kScanThreads + threadIdx.x;
        stage[k * kScanThreads + threadIdx.x] = i < n ? in[i] : ScanOps<T>::zero();
    }
    __syncthreads();
    T vals[kScanItems];
    T acc = ScanOps<T>::zero();
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        vals[k] = stage[threadIdx.x * kScanItems + k];
        acc = ScanOps<T>::add(acc, vals[k]);
    }
    T total;
    const T tileBase = tileSums[blockIdx.x];
    T run = ScanOps<T>::add(tileBase, blockExclusive(acc, total));  // (ends with a barrier: stage is read)
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        stage[threadIdx.x * kScanItems + k] = run;
        run = ScanOps<T>::add(run, vals[k]);
    }
    __syncthreads();
    const T tileEnd = ScanOps<T>::add(tileBase, total);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int idx = k * kScanThreads + threadIdx.x;
        const int64_t i = base + idx;
        if (i < n) {
            const T r = stage[idx];
            if constexpr (Post::kPrefixes) out[i] = r;
            post(i, r, minus(idx + 1 < kScanTile ? stage[idx + 1] : tileEnd, r));
        }
    }
    if ((int)blockIdx.x == lastBlock && threadIdx.x == 0) {
        out[n] = tileSums[nTiles];
        post.total(n, tileSums[nTiles]);
    }
}

// in and out may alias only if the caller accepts in being overwritten after
// the reduction (kScanApply reads in[i] before writing out[i] of the same i).
// scratch needs numTiles + 1 elements.  Returns false if n is too large.
// nDev != nullptr: the element count is read on the device from *nDev,
// at most n (the capacity the launches cover).
template <typename T, class In, class Post = NoPost>
bool exclusiveScanOf(In in, T* out, int64_t n, T* scratch, cudaStream_t s, Post post = Post(),
                     const int* nDev = nullptr) {
    const int64_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles > kScanMaxTiles) return false;
    const int nt = tiles > 0 ? (int)tiles : 1;
    const ScanCount cnt{n, nDev};
    // (four elements per load only from 16-byte aligned arrays)
    bool vec = false;
    if constexpr (In::kFour) vec = in.vectorOk();
    if (n > 0 || nDev) {
        countLaunch();
        kScanReduce<T, In><<<nt, kScanThreads, 0, s>>>(in, cnt, scratch, vec);
    } else {
        cudaMemsetAsync(scratch, 0, sizeof(T), s);
    }
    countLaunch();
    kScanTiles<T><<<1, 1024, 0, s>>>(scratch, cnt);
    if (n > 0 || nDev) {
        countLaunch();
        if constexpr (Post::kStaged)
            kScanApplyStaged<T, In, Post><<<nt, kScanThreads, 0, s>>>(in, cnt, scratch, out, post);
        else
            kScanApply<T, In, Post><<<nt, kScanThreads, 0, s>>>(in, cnt, scratch, out, post, vec);
    } else {
        cudaMemcpyAsync(out, scratch, sizeof(T), cudaMemcpyDeviceToDevice, s);
    }
    return true;
}

template <typename T>
bool exclusiveScan(const T* in, T* out, int64_t n, T* scratch, cudaStream_t s) {
    return exclusiveScanOf<T>(ArrayRead<T>{in}, out, n, scratch, s);
}

// exclusive scan of the popcounts of n mask words: out[i] = set bits in
// words 0..i-1, out[n] = all set bits
inline bool exclusiveScanPopc(const uint32_t* mask, int* out, int64_t n, int* scratch, cudaStream_t s) {
    return exclusiveScanOf<int>(PopcRead{mask}, out, n, scratch, s);
}

inline int64_t scanScratchElems(int64_t n) { return (n + kScanTile - 1) / kScanTile + 2; }

}  // namespace mdmc
