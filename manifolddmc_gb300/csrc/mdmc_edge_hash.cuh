// Open-addressed edge table of the halfedge mesh: key = (min vertex, max
// vertex), value = number of faces on the edge and up to four halfedge ids
// (HalfedgeDeviceHashTable, D/Halfedges/HalfedgeHashTables.h:22-158).
// 32-byte buckets (one sector per probe), a 64-bit mixing hash mapped onto the
// capacity by a multiply-high, linear probing with a bounded probe count.
#pragma once

#include "mdmc_types.h"

namespace mdmc {

constexpr int kMaxProbes = 1024;

// concatenateKeys, D/Utils/Utilities.h:15-22
__host__ __device__ __forceinline__ unsigned long long edgeKey(int a, int b) {
    unsigned lo = (unsigned)(a < b ? a : b), hi = (unsigned)(a < b ? b : a);
    return ((unsigned long long)lo << 32) | hi;
}

__device__ __forceinline__ unsigned long long mixKey(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
}

__device__ __forceinline__ unsigned long long bucketOf(unsigned long long key, unsigned long long cap) {
    return __umul64hi(mixKey(key), cap);
}

// Inserts halfedge h on edge (a, b).
__device__ __forceinline__ void edgeInsert(Bucket* t, unsigned long long cap, int a, int b, int h,
                                           uint32_t* status) {
    const unsigned long long key = edgeKey(a, b);
    unsigned long long i = bucketOf(key, cap);
    for (int p = 0; p < kMaxProbes; ++p) {
        Bucket* bk = t + i;
        unsigned long long k = *(volatile unsigned long long*)&bk->key;
        if (k == kEmptyKey) k = atomicCAS(&bk->key, kEmptyKey, key);
        if (k == kEmptyKey || k == key) {
            int slot = atomicAdd(&bk->cnt, 1) + 1;
            if (slot < 4) bk->ids[slot] = h;
            else atomicOr(status, kStatusBucketOverflow);
            return;
        }
        if (++i == cap) i = 0;
    }
    atomicOr(status, kStatusProbeLimit);
}

// Number of faces on edge (a, b), -1 if the edge is absent
// (HalfedgeDeviceHashTable::getNumFaces, HalfedgeHashTables.h:296-311).
__device__ __forceinline__ int edgeValence(const Bucket* t, unsigned long long cap, int a, int b) {
    const unsigned long long key = edgeKey(a, b);
    unsigned long long i = bucketOf(key, cap);
    for (int p = 0; p < kMaxProbes; ++p) {
        unsigned long long k = t[i].key;
        if (k == key) return t[i].cnt + 1;
        if (k == kEmptyKey) return -1;
        if (++i == cap) i = 0;
    }
    return -1;
}

}  // namespace mdmc
