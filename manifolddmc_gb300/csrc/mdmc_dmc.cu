// Grid preparation and the Dual Marching Cubes stage.
//
// Reference: performDualMarchingCubes + mapQuadrilaterals
// (D/DualMarchingCubes.cu:38-85), CellIntersection::sliceP
// (D/CellIntersection.inl:368-439), collectHalfedgeElements
// (D/Halfedges/HalfedgeMesh.cu:14-60), refineGrid (D/UniformGrid.inl:279-319).
//
// GB300 design: one warp per x-row of cells.  Two lean streaming passes over
// the grid (count, emit) replace the reference's single global atomic vertex
// counter and its 20M-bucket quad hash table: the count pass gives per-row
// (active cells, owned quads), an exclusive scan turns them into row offsets,
// and the emit pass writes the active cells' records at deterministic offsets
// using warp ballots and shuffles.  The vertices are then computed by a dense
// kernel over the active-cell list (no lane idles behind a neighbour's
// surface iteration), at offsets from a scan of the cells' contour counts.
// Each quad is built by the cell that owns its grid edge (the cell at the
// edge's origin), which looks up the three other cells' records by row, so no
// quad hash is needed; the same thread writes the quad's four halfedges and
// inserts its edges into the edge table.
#include <cuda_runtime.h>

#include "mdmc_device.cuh"
#include "mdmc_kernels.h"
#include "mdmc_scan.cuh"

namespace mdmc {

// ---------------------------------------------------------------------------
// refineGrid, D/UniformGrid.inl:279-319.  One block row per output row
// (blockIdx.y, blockIdx.z = y, z), so no per-sample index division.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) kRefine(const float* __restrict__ in, int3 din, float* __restrict__ out,
                                               int3 dout, int r, int pad) {
    const int x0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (x0 >= dout.x) return;
    int x = x0, y = blockIdx.y, z = blockIdx.z;
    if (pad) {
        x = min(max(x, 1), dout.x - 2) - 1;
        y = min(max(y, 1), dout.y - 2) - 1;
        z = min(max(z, 1), dout.z - 2) - 1;
    }
    const float f = (float)(r + 1);
    const float qx = (float)x / f, qy = (float)y / f, qz = (float)z / f;
    const int mx = (int)floorf(qx), my = (int)floorf(qy), mz = (int)floorf(qz);
    const F3 diff = f3(qx - (float)mx, qy - (float)my, qz - (float)mz);
    float s[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int cx = min(max(mx + (c & 1), 0), din.x - 1);
        const int cy = min(max(my + ((c >> 1) & 1), 0), din.y - 1);
        const int cz = min(max(mz + ((c >> 2) & 1), 0), din.z - 1);
        s[c] = __ldg(in + ((int64_t)cz * din.y + cy) * din.x + cx);
    }
    out[((int64_t)blockIdx.z * dout.y + blockIdx.y) * dout.x + x0] = trilinear(s, diff);
}

void launchRefine(const float* in, int3 din, float* out, int3 dout, int r, int pad, cudaStream_t s) {
    dim3 grid((dout.x + 127) / 128, dout.y, dout.z);
    countLaunch();
    kRefine<<<grid, 128, 0, s>>>(in, din, out, dout, r, pad);
}

// ---------------------------------------------------------------------------
// coarse-cell pre-pass for refined grids.  A refined cell lies inside one
// coarse cell and its samples are trilinear interpolations of that cell's
// eight corners: in exact arithmetic they stay within [min, max] of the
// corners, and the rounding of refineGrid's expression (three lerp levels,
// at most ~15 unit roundings of m = max|corner|) stays below 15u*m (u = 2^-24).
// With D = 64u*m (exact: a power-of-two multiple), a coarse cell whose corners
// all satisfy max < fl(iso - D), or min >= fl(iso + D), holds only case-0 /
// case-255 refined cells.  The float rounding of iso -+ D is at most u/2 of
// |iso - D|; while |iso| <= 97m that is below the 49u*m of slack, and when
// |iso| > 97m no refined sample can reach iso at all, so the test never skips
// a crossing cell.  D is at least 2^-120, which covers the absolute rounding
// of subnormal values.  NaN corners keep the cell.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) kCoarseMayCross(const float* __restrict__ c, int cX, int cY, int cZ, float iso,
                                                       uint32_t* __restrict__ bits, int64_t numCells,
                                                       uint32_t* __restrict__ list, unsigned long long* listCount,
                                                       FastDiv divCX1, FastDiv divCY1) {
    __shared__ unsigned warpCount[8];
    __shared__ unsigned long long blockBase;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool may = false;
    if (i < numCells) {
        // fewer than 2^32 coarse cells: 32-bit division
        const uint32_t iu = (uint32_t)i, ncx = (uint32_t)(cX - 1), ncy = (uint32_t)(cY - 1);
        const uint32_t row = divCX1.div(iu), layer = divCY1.div(row);
        const int x = (int)(iu - row * ncx);
        const int y = (int)(row - layer * ncy);
        const int z = (int)layer;
        float lo = INFINITY, hi = -INFINITY, mag = 0.f;
        bool nan = false;
        // (coarse grids have fewer than 2^32 samples: 32-bit offsets)
        const uint32_t sy = (uint32_t)cX, sz = (uint32_t)cX * (uint32_t)cY;
        const uint32_t base = (uint32_t)z * sz + (uint32_t)y * sy + (uint32_t)x;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float v = __ldg(c + (base + ((k >> 2) & 1) * sz + ((k >> 1) & 1) * sy + (k & 1)));
            nan = nan || (v != v);
            lo = fminf(lo, v);
            hi = fmaxf(hi, v);
            mag = fmaxf(mag, fabsf(v));
        }
        // 64 * 2^-24 * m, at least 2^-120 so that subnormal rounding stays covered
        const float delta = fmaxf(mag * 3.814697265625e-06f, 7.52316384526264e-37f);
        const bool allBelow = hi < iso - delta;
        const bool allAbove = lo >= iso + delta;
        may = nan || !(allBelow || allAbove);
    }
    const unsigned b = __ballot_sync(0xffffffffu, may);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0 && i < numCells) bits[i >> 5] = b;
    if (!list) return;
    // the candidates, in any order: one atomic per block
    if (lane == 0) warpCount[warp] = __popc(b);
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned total = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            const unsigned n = warpCount[w];
            warpCount[w] = total;
            total += n;
        }
        blockBase = total ? atomicAdd(listCount, (unsigned long long)total) : 0ULL;
    }
    __syncthreads();
    if (may) list[blockBase + warpCount[warp] + __popc(b & ((1u << lane) - 1u))] = (uint32_t)i;
}

void launchCoarseMayCross(const RefinedView& g, float iso, uint32_t* bits, cudaStream_t s) {
    launchCoarseMayCross(g, iso, bits, nullptr, nullptr, s);
}

void launchCoarseMayCross(const RefinedView& g, float iso, uint32_t* bits, uint32_t* list, unsigned long long* listCount,
                          cudaStream_t s) {
    const int64_t n = (int64_t)(g.cX - 1) * (g.cY - 1) * (g.cZ - 1);
    if (n <= 0) return;
    countLaunch();
    kCoarseMayCross<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g.c, g.cX, g.cY, g.cZ, iso, bits, n, list, listCount,
                                                                g.divCX1, g.divCY1);
}


// ---------------------------------------------------------------------------
// row streaming.  A warp walks one x-row of cells in chunks of 32.  Each lane
// holds the four samples of its column (y/y+1 x z/z+1); the x+1 column comes
// from the next lane by shuffle, the last lane's from the next chunk.
// ---------------------------------------------------------------------------
template <class View>
struct RowWalker;

template <>
struct RowWalker<PlainView> {
    const float* r[4];  // sample rows (y,z) (y+1,z) (y,z+1) (y+1,z+1)
    int X;
    __device__ RowWalker(const PlainView& g, int y, int z) : X(g.X) {
        const size_t sy = g.X, sz = (size_t)g.X * g.Y;
        const float* b = g.v + (size_t)z * sz + (size_t)y * sy;
        r[0] = b;
        r[1] = b + sy;
        r[2] = b + sz;
        r[3] = b + sz + sy;
    }
    __device__ __forceinline__ void load(int x, float v[4]) const {
        if (x < X) {
#pragma unroll
            for (int k = 0; k < 4; ++k) v[k] = __ldg(r[k] + x);
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) v[k] = 0.f;
        }
    }
    __device__ __forceinline__ bool chunkMayCross(int) const { return true; }
};

// Refined rows: the four samples of a column (x; y, y+1; z, z+1) are
// refineGrid's trilinear interpolations.  They share the column's x position
// in the coarse grid and, per coarse row (cy, cz), the same x-lerp
// s(mx) + dx * (s(mx+1) - s(mx)); refineGrid computes exactly these lerps
// (a, b, c, e in Interpolation::interpolateTrilinearly) before its y and z
// lerps, so evaluating each distinct row lerp once gives bit-identical values.
// The rows needed are cy in {j0, j1, j2} x cz in {k0, k1, k2}, the third
// only when y+1 (z+1) falls into the next coarse cell.
template <>
struct RowWalker<RefinedView> {
    const RefinedView& g;
    int my, mz;          // coarse cell of the row (for chunk skipping)
    int J[3], K[3];      // clamped coarse row indices my, my+1, my+2 (and z)
    int ySecond[2];      // per sample row y, y+1: 0 -> rows (J0, J1), 1 -> rows (J1, J2)
    int zSecond[2];
    float dy[2], dz[2];  // in-cell weights of y, y+1 and z, z+1
    uint32_t rowOff[3][3];  // element offsets of the coarse rows (coarse grids have fewer than 2^32 samples)
    __device__ RowWalker(const RefinedView& view, int y, int z) : g(view) {
        int myy[2], mzz[2];
        for (int t = 0; t < 2; ++t) {
            const float qy = g.divf(g.unpad(y + t, g.Y));
            myy[t] = (int)floorf(qy);
            dy[t] = qy - (float)myy[t];
            const float qz = g.divf(g.unpad(z + t, g.Z));
            mzz[t] = (int)floorf(qz);
            dz[t] = qz - (float)mzz[t];
        }
        for (int t = 0; t < 3; ++t) {
            J[t] = min(max(myy[0] + t, 0), g.cY - 1);
            K[t] = min(max(mzz[0] + t, 0), g.cZ - 1);
        }
        for (int t = 0; t < 2; ++t) {
            ySecond[t] = myy[t] != myy[0] ? 1 : 0;
            zSecond[t] = mzz[t] != mzz[0] ? 1 : 0;
        }
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) rowOff[a][b] = ((uint32_t)K[b] * (uint32_t)g.cY + (uint32_t)J[a]) * (uint32_t)g.cX;
        my = g.coarseCell(y, g.Y, g.cY);
        mz = g.coarseCell(z, g.Z, g.cZ);
    }
    __device__ __forceinline__ void load(int x, float v[4]) const {
        if (x >= g.X) {
#pragma unroll
            for (int k = 0; k < 4; ++k) v[k] = 0.f;
            return;
        }
        const float qx = g.divf(g.unpad(x, g.X));
        const int mx = (int)floorf(qx);
        const float dx = qx - (float)mx;
        const int x0 = min(max(mx, 0), g.cX - 1), x1 = min(max(mx + 1, 0), g.cX - 1);
        auto lerpX = [&](int a, int b) {
            const uint32_t o = rowOff[a][b];
            const float s0 = __ldg(g.c + (o + (uint32_t)x0)), s1 = __ldg(g.c + (o + (uint32_t)x1));
            return s0 + dx * (s1 - s0);
        };
        const bool y2 = ySecond[1], z2 = zSecond[1];
        const float L00 = lerpX(0, 0), L10 = lerpX(1, 0), L01 = lerpX(0, 1), L11 = lerpX(1, 1);
        float L20 = 0.f, L21 = 0.f, L02 = 0.f, L12 = 0.f, L22 = 0.f;
        if (y2) {
            L20 = lerpX(2, 0);
            L21 = lerpX(2, 1);
        }
        if (z2) {
            L02 = lerpX(0, 2);
            L12 = lerpX(1, 2);
            if (y2) L22 = lerpX(2, 2);
        }
        // row lerp (j, k) by warp-uniform selects (no local-memory array)
        auto pick = [&](int j, int k) -> float {
            const float r0 = k == 0 ? L00 : (k == 1 ? L01 : L02);
            const float r1 = k == 0 ? L10 : (k == 1 ? L11 : L12);
            const float r2 = k == 0 ? L20 : (k == 1 ? L21 : L22);
            return j == 0 ? r0 : (j == 1 ? r1 : r2);
        };
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int ys = t & 1, zs = t >> 1;  // v[0] (y,z) v[1] (y+1,z) v[2] (y,z+1) v[3] (y+1,z+1)
            const int ja = ySecond[ys], kb = zSecond[zs];
            const float a = pick(ja, kb), b = pick(ja + 1, kb), c = pick(ja, kb + 1), e = pick(ja + 1, kb + 1);
            const float wy = dy[ys], wz = dz[zs];
            const float lo = (1.f - wy) * a + wy * b;
            const float hi = (1.f - wy) * c + wy * e;
            v[t] = (1.f - wz) * lo + wz * hi;
        }
    }
    // refined cells x in [start(m), end(m)) lie in coarse cell m (along x)
    __device__ __forceinline__ int coarseStart(int m) const { return g.pad ? (m == 0 ? 0 : m * (g.r + 1) + 1) : m * (g.r + 1); }
    __device__ __forceinline__ int coarseEnd(int m) const { return m == g.cX - 2 ? g.X - 1 : coarseStart(m + 1); }
    // may any cell x0..x0+31 of the row cross iso (uniform over the warp)
    __device__ __forceinline__ bool chunkMayCross(int x0) const {
        if (!g.mayCross) return true;
        const int lastCell = min(x0 + 31, g.X - 2);
        const int m0 = g.coarseCell(x0, g.X, g.cX), m1 = g.coarseCell(lastCell, g.X, g.cX);
        for (int m = m0; m <= m1; ++m)
            if (g.coarseMayCross(m, my, mz)) return true;
        return false;
    }
};

// the eight corner values of the lane's cell: own column and the next one
template <class View>
__device__ __forceinline__ void chunkCorners(const RowWalker<View>& w, int x0, int lane, float s[8]) {
    float cur[4], ext[4];
    w.load(x0 + lane, cur);
    if (lane == 31) w.load(x0 + 32, ext);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float right = __shfl_down_sync(0xffffffffu, cur[k], 1);
        s[2 * k] = cur[k];
        s[2 * k + 1] = lane == 31 ? ext[k] : right;
    }
}

// the same with the next chunk's columns already loaded (plain grids)
__device__ __forceinline__ void cellCorners(const float cur[4], const float nxt[4], int lane, float s[8]) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float right = __shfl_down_sync(0xffffffffu, cur[k], 1);
        const float wrap = __shfl_sync(0xffffffffu, nxt[k], 0);
        s[2 * k] = cur[k];
        s[2 * k + 1] = lane == 31 ? wrap : right;
    }
}

__device__ __forceinline__ int caseOf(const float s[8], float iso) {
    int cs = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) cs |= (s[i] >= iso ? 1 : 0) << i;
    return cs;
}

// quads owned by a cell: the three edges leaving corner 0 (local edges 0, 3,
// 8), when all four cells around the edge exist
__device__ __forceinline__ int ownedQuads(int cs, int x, int y, int z) {
    return ((((cs ^ (cs >> 1)) & 1) && y >= 1 && z >= 1) ? 1 : 0) +
           ((((cs ^ (cs >> 2)) & 1) && x >= 1 && z >= 1) ? 1 : 0) +
           ((((cs ^ (cs >> 4)) & 1) && x >= 1 && y >= 1) ? 1 : 0);
}

// ---------------------------------------------------------------------------
// the active-cell mask of a refined grid, one warp per candidate coarse cell:
// the refined samples of the coarse cell's block of refined cells, one z
// plane at a time (each sample is RefinedView::at, i.e. refineGrid's value),
// the cases of the block's cells, and their active bits OR-ed into the row
// words (cleared beforehand; refined cells of the other coarse cells are
// inactive, see kCoarseMayCross)
// ---------------------------------------------------------------------------
constexpr int kBlockMaskWarps = 8;
constexpr int kBlockSamplesMax = 512;  // per warp: a whole block's samples, or two z planes of (r + 4)^2

__device__ __forceinline__ int blockStart(const RefinedView& g, int m) { return g.pad ? (m == 0 ? 0 : m * (g.r + 1) + 1) : m * (g.r + 1); }
__device__ __forceinline__ int blockEnd(const RefinedView& g, int m, int n, int cn) {
    return m == cn - 2 ? n - 1 : blockStart(g, m + 1);
}

// ORs the active bit of the lane's cell (x, y, z) into its row word; lanes of
// the same word combine their bits first
__device__ __forceinline__ void orActive(uint32_t* mask, int W, int Y, bool active, int x, int y, int z) {
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (active) {
        const int64_t w = ((int64_t)z * (Y - 1) + y) * W + (x >> 5);
        const unsigned peers = __match_any_sync(act, w);
        const unsigned bits = __reduce_or_sync(peers, 1u << (x & 31));
        if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicOr(&mask[w], bits);
    }
}

// The 5x5x5 refined samples (xs..xs+4, ys..ys+4, zs..zs+4) of a standard
// block into buf[kz*25 + ky*5 + kx], evaluated separably: every sample is
// RefinedView::at's trilinear interpolation, whose x-lerps depend only on
// (kx, coarse row) and whose y-lerps only on (kx, ky, coarse z), so the 27
// coarse samples around the block are loaded once, the 45 distinct x-lerps and
// 75 distinct y-lerps are computed once and the 125 z-lerps finish them, each
// with the operations and operands at() uses.  Returns false (nothing
// written) when the block's coarse indices do not lie within a 3x3x3 range.
// the lane's element coordinates in the three stages (the same for every
// block): x-lerp i = lane + 32u -> (kx, ry, rz); y-lerp -> (kx, ky, rz);
// sample -> (kx, ky, kz); packed 4 bits each, 0xFFF past the end
struct SeparableLanes {
    uint16_t xl[2], yl[3], s[4];
    __device__ __forceinline__ explicit SeparableLanes(int lane) {
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int i = lane + 32 * u;
            xl[u] = i < 45 ? (uint16_t)((i % 5) | (((i / 5) % 3) << 4) | ((i / 15) << 8)) : 0xFFF;
        }
#pragma unroll
        for (int u = 0; u < 3; ++u) {
            const int i = lane + 32 * u;
            yl[u] = i < 75 ? (uint16_t)((i % 5) | (((i / 5) % 5) << 4) | ((i / 25) << 8)) : 0xFFF;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int i = lane + 32 * u;
            s[u] = i < 125 ? (uint16_t)((i % 5) | (((i / 5) % 5) << 4) | ((i / 25) << 8)) : 0xFFF;
        }
    }
};

__device__ bool blockSamples5(const RefinedView& g, int xs, int ys, int zs, int lane, const SeparableLanes& sl,
                              float* __restrict__ buf, float* __restrict__ sc, int* __restrict__ ax,
                              float* __restrict__ ad) {
    int i0 = 0, i1 = 0;
    float d = 0.f;
    if (lane < 15) {
        const int a = lane / 5, k = lane - 5 * a;
        const int n = a == 0 ? g.X : (a == 1 ? g.Y : g.Z);
        const int cn = a == 0 ? g.cX : (a == 1 ? g.cY : g.cZ);
        const int p = (a == 0 ? xs : (a == 1 ? ys : zs)) + k;
        const float q = g.divf(g.unpad(p, n));
        const int m = (int)floorf(q);
        d = q - (float)m;
        i0 = min(max(m, 0), cn - 1);
        i1 = min(max(m + 1, 0), cn - 1);
    }
    const int bx = __shfl_sync(0xffffffffu, i0, 0), by = __shfl_sync(0xffffffffu, i0, 5),
              bz = __shfl_sync(0xffffffffu, i0, 10);
    const int b = lane < 5 ? bx : (lane < 10 ? by : bz);
    const int r0 = i0 - b, r1 = i1 - b;
    if (__ballot_sync(0xffffffffu, lane < 15 && (r0 < 0 || r1 > 2 || r0 > r1)) != 0u) return false;
    if (lane < 15) {
        ax[lane] = r0;
        ax[15 + lane] = r1;
        ad[lane] = d;
    }
    if (lane < 27) {
        const int rx = lane % 3, ry = (lane / 3) % 3, rz = lane / 9;
        const int cx = min(bx + rx, g.cX - 1), cy = min(by + ry, g.cY - 1), cz = min(bz + rz, g.cZ - 1);
        sc[lane] = __ldg(g.c + ((size_t)cz * g.cY + cy) * g.cX + cx);
    }
    __syncwarp();
    float* xl = sc + 27;  // [rz][ry][kx], 45
    float* yl = sc + 72;  // [rz][ky][kx], 75
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        const int c = sl.xl[u];
        if (c == 0xFFF) continue;
        const int kx = c & 15, ry = (c >> 4) & 15, rz = c >> 8;
        const float s0 = sc[rz * 9 + ry * 3 + ax[kx]], s1 = sc[rz * 9 + ry * 3 + ax[15 + kx]];
        xl[lane + 32 * u] = s0 + ad[kx] * (s1 - s0);
    }
    __syncwarp();
#pragma unroll
    for (int u = 0; u < 3; ++u) {
        const int c = sl.yl[u];
        if (c == 0xFFF) continue;
        const int kx = c & 15, ky = (c >> 4) & 15, rz = c >> 8;
        const float dy = ad[5 + ky];
        const float a = xl[rz * 15 + ax[5 + ky] * 5 + kx], bb = xl[rz * 15 + ax[20 + ky] * 5 + kx];
        yl[lane + 32 * u] = (1.f - dy) * a + dy * bb;
    }
    __syncwarp();
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int c = sl.s[u];
        if (c == 0xFFF) continue;
        const int kx = c & 15, ky = (c >> 4) & 15, kz = c >> 8;
        const float dz = ad[10 + kz];
        const float lo = yl[ax[10 + kz] * 25 + ky * 5 + kx], hi = yl[ax[25 + kz] * 25 + ky * 5 + kx];
        buf[lane + 32 * u] = (1.f - dz) * lo + dz * hi;
    }
    __syncwarp();
    return true;
}

__global__ void __launch_bounds__(32 * kBlockMaskWarps, 4) kBlockMask(RefinedView g, float iso, const uint32_t* __restrict__ list,
                                                                 const unsigned long long* listCount,
                                                                 uint32_t* __restrict__ mask, int W, CaseBytes cases,
                                                                 uint32_t* status) {
    __shared__ float samples[kBlockMaskWarps][kBlockSamplesMax];
    __shared__ float sepSamples[kBlockMaskWarps][27 + 45 + 75];
    __shared__ int sepIndex[kBlockMaskWarps][30];
    __shared__ float sepFrac[kBlockMaskWarps][15];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float* buf = samples[warp];
    const SeparableLanes sl(lane);
    const int64_t count = (int64_t)*listCount;
    const int64_t nc = (int64_t)(g.cX - 1) * (g.cY - 1) * (g.cZ - 1);
    for (int64_t li = (int64_t)blockIdx.x * kBlockMaskWarps + warp; li < count;
         li += (int64_t)gridDim.x * kBlockMaskWarps) {
        const int64_t ci = list[li];
        if (ci < 0 || ci >= nc) {
            if (lane == 0) atomicOr(status, kStatusBadIndex);
            continue;
        }
        // coarse cells number fewer than 2^32 (refined grids have fewer samples)
        const uint32_t cu = (uint32_t)ci, ncx = (uint32_t)(g.cX - 1), ncy = (uint32_t)(g.cY - 1);
        const uint32_t crow = g.divCX1.div(cu), clayer = g.divCY1.div(crow);
        const int mx = (int)(cu - crow * ncx);
        const int my = (int)(crow - clayer * ncy);
        const int mz = (int)clayer;
        const int xs = blockStart(g, mx), xe = blockEnd(g, mx, g.X, g.cX);
        const int ys = blockStart(g, my), ye = blockEnd(g, my, g.Y, g.cY);
        const int zs = blockStart(g, mz), ze = blockEnd(g, mz, g.Z, g.cZ);
        const int ex = xe - xs, ey = ye - ys, ez = ze - zs;
        const int px = ex + 1, plane = px * (ey + 1);
        if (ex < 1 || ey < 1 || ez < 1 || 2 * plane > kBlockSamplesMax) {
            if (lane == 0) atomicOr(status, kStatusBadIndex);
            continue;
        }
        if (ex == 4 && ey == 4 && ez == 4 && ((xs & 31) + 4) <= 32) {
            // the standard block of a x4 refinement: 125 samples and 64 cells
            // with compile-time strides; the 4 cells of a row lie in one mask
            // word and occupy 4 aligned lanes, OR-ed by two shuffles
            if (!blockSamples5(g, xs, ys, zs, lane, sl, buf, sepSamples[warp], sepIndex[warp], sepFrac[warp])) {
                float v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int k = 32 * u + lane;
                    const int kk = k < 125 ? k : 0;
                    v[u] = g.at(xs + kk % 5, ys + (kk / 5) % 5, zs + kk / 25);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (32 * u + lane < 125) buf[32 * u + lane] = v[u];
                __syncwarp();
            }
#pragma unroll
            for (int k0 = 0; k0 < 64; k0 += 32) {
                const int k = k0 + lane;
                const int lx = k & 3, ly = (k >> 2) & 3, lz = k >> 4;
                const int o = lz * 25 + ly * 5 + lx;
                const float s[8] = {buf[o],      buf[o + 1],      buf[o + 5],      buf[o + 6],
                                    buf[o + 25], buf[o + 26], buf[o + 30], buf[o + 31]};
                const int cs = caseOf(s, iso);
                if (cases.mode == 2) cases.p[(size_t)ci * 64 + k] = (uint8_t)cs;
                const int x = xs + lx;
                unsigned bitv = (cs != 0 && cs != 255) ? (1u << (x & 31)) : 0u;
                bitv |= __shfl_xor_sync(0xffffffffu, bitv, 1);
                bitv |= __shfl_xor_sync(0xffffffffu, bitv, 2);
                if (lx == 0 && bitv) atomicOr(&mask[((int64_t)(zs + lz) * (g.Y - 1) + (ys + ly)) * W + (x >> 5)], bitv);
            }
            __syncwarp();
            continue;
        }
        if (plane * (ez + 1) <= kBlockSamplesMax) {
            // every sample of the block at once (loads of four rounds in flight)
            const int total = plane * (ez + 1);
            for (int k0 = 0; k0 < total; k0 += 128) {
                float v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int k = k0 + 32 * u + lane;
                    const int kk = k < total ? k : 0;
                    v[u] = g.at(xs + kk % px, ys + (kk % plane) / px, zs + kk / plane);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int k = k0 + 32 * u + lane;
                    if (k < total) buf[k] = v[u];
                }
            }
            __syncwarp();
            const int cells = ex * ey * ez;
            for (int k0 = 0; k0 < cells; k0 += 32) {
                const int k = k0 + lane;
                bool active = false;
                int x = 0, y = 0, z = 0;
                if (k < cells) {
                    const int lx = k % ex, ly = (k / ex) % ey, lz = k / (ex * ey);
                    x = xs + lx;
                    y = ys + ly;
                    z = zs + lz;
                    const int o = lz * plane + ly * px + lx;
                    const float s[8] = {buf[o],         buf[o + 1],         buf[o + px],         buf[o + px + 1],
                                        buf[o + plane], buf[o + plane + 1], buf[o + plane + px], buf[o + plane + px + 1]};
                    const int cs = caseOf(s, iso);
                    active = cs != 0 && cs != 255;
                }
                orActive(mask, W, g.Y, active, x, y, z);
            }
            __syncwarp();
            continue;
        }
        // large blocks: two z planes at a time
        float* p0 = buf;
        float* p1 = buf + plane;
        for (int k = lane; k < plane; k += 32) p0[k] = g.at(xs + k % px, ys + k / px, zs);
        for (int z = zs; z < ze; ++z) {
            for (int k = lane; k < plane; k += 32) p1[k] = g.at(xs + k % px, ys + k / px, z + 1);
            __syncwarp();
            for (int k0 = 0; k0 < ex * ey; k0 += 32) {
                const int k = k0 + lane;
                bool active = false;
                int x = 0, y = 0;
                if (k < ex * ey) {
                    const int lx = k % ex, ly = k / ex;
                    x = xs + lx;
                    y = ys + ly;
                    const int o = ly * px + lx;
                    const float s[8] = {p0[o], p0[o + 1], p0[o + px], p0[o + px + 1],
                                        p1[o], p1[o + 1], p1[o + px], p1[o + px + 1]};
                    const int cs = caseOf(s, iso);
                    active = cs != 0 && cs != 255;
                }
                orActive(mask, W, g.Y, active, x, y, z);
            }
            __syncwarp();
            float* t = p0;
            p0 = p1;
            p1 = t;
        }
        __syncwarp();
    }
}

void launchBlockMask(const RefinedView& g, float iso, const uint32_t* list, const unsigned long long* listCount,
                     uint32_t* mask, int W, CaseBytes cases, uint32_t* status, cudaStream_t s) {
    countLaunch();
    kBlockMask<<<152 * 8, 32 * kBlockMaskWarps, 0, s>>>(g, iso, list, listCount, mask, W, cases, status);
}

// Visits the cells of one row and calls f(x, s[8]) once per lane and step
// (warp-uniform calls; lanes without a cell get x = X, which every caller
// rejects).  Plain grids: chunks of 32 consecutive cells, the next chunk's
// columns loaded ahead.  Refined grids: only the cells of coarse cells that
// may cross iso, packed into the lanes (the g-th candidate coarse cell of a
// 32-cell mask word fills lanes g*W .. g*W+W-1, W = widest coarse cell), in
// increasing x.
template <class View, class F>
__device__ __forceinline__ void walkRow(const View& g, int y, int z, int lane, F&& f) {
    const RowWalker<View> w(g, y, z);
    if constexpr (View::kRefined) {
        const int nc = g.cX - 1;  // coarse cells along x
        if (!g.mayCross || nc < 1) {
            for (int x0 = 0; x0 < g.X - 1; x0 += 32) {
                float s[8];
                chunkCorners(w, x0, lane, s);
                f(x0 + lane, s);
            }
            return;
        }
        const int W = (g.r + 1) + (g.pad ? 2 : 0);
        const size_t rowBit = ((size_t)w.mz * (g.cY - 1) + w.my) * (size_t)nc;
        for (int wb = 0; wb < nc; wb += 32) {
            // the 32 coarse cells wb .. wb+31 of this row (the bits may straddle two words)
            const size_t b0 = rowBit + wb;
            const uint32_t lo = __ldg(g.mayCross + (b0 >> 5)), hi = __ldg(g.mayCross + (b0 >> 5) + 1);
            uint32_t word = (b0 & 31) ? ((lo >> (b0 & 31)) | (hi << (32 - (b0 & 31)))) : lo;
            if (nc - wb < 32) word &= (1u << (nc - wb)) - 1u;
            const int nset = __popc(word);
            if (W <= 32) {
                const int G = 32 / W;
                for (int g0 = 0; g0 < nset; g0 += G) {
                    const int gi = g0 + lane / W, k = lane % W;
                    int x = g.X;
                    if (lane < G * W && gi < nset) {
                        const int m = wb + (int)__fns(word, 0, gi + 1);
                        const int xs = w.coarseStart(m);
                        if (xs + k < w.coarseEnd(m)) x = xs + k;
                    }
                    float cur[4], nxt[4], s[8];
                    w.load(x, cur);
                    w.load(x + 1, nxt);
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        s[2 * t] = cur[t];
                        s[2 * t + 1] = nxt[t];
                    }
                    f(x, s);
                }
            } else {
                for (int gi = 0; gi < nset; ++gi) {
                    const int m = wb + (int)__fns(word, 0, gi + 1);
                    const int xs = w.coarseStart(m), xe = w.coarseEnd(m);
                    for (int k0 = 0; k0 < xe - xs; k0 += 32) {
                        const int x = (xs + k0 + lane < xe) ? xs + k0 + lane : g.X;
                        float cur[4], nxt[4], s[8];
                        w.load(x, cur);
                        w.load(x + 1, nxt);
#pragma unroll
                        for (int t = 0; t < 4; ++t) {
                            s[2 * t] = cur[t];
                            s[2 * t + 1] = nxt[t];
                        }
                        f(x, s);
                    }
                }
            }
        }
    } else {
        float cur[4], nxt[4];
        w.load(lane, cur);
        for (int x0 = 0; x0 < g.X - 1; x0 += 32) {
            w.load(x0 + 32 + lane, nxt);
            float s[8];
            cellCorners(cur, nxt, lane, s);
            f(x0 + lane, s);
#pragma unroll
            for (int k = 0; k < 4; ++k) cur[k] = nxt[k];
        }
    }
}

// per-row (active cells, owned quads)
template <class View>
__global__ void __launch_bounds__(256) kRowCount(View g, float iso, int4* __restrict__ rowCounts, int numRows) {
    const int lane = threadIdx.x & 31;
    const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= numRows) return;
    const int y = row % (g.Y - 1), z = row / (g.Y - 1);
    int a = 0, q = 0;
    walkRow(g, y, z, lane, [&](int x, const float s[8]) {
        if (x < g.X - 1) {
            const int cs = caseOf(s, iso);
            if (cs != 0 && cs != 255) {
                ++a;
                q += ownedQuads(cs, x, y, z);
            }
        }
    });
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        q += __shfl_down_sync(0xffffffffu, q, o);
    }
    if (lane == 0) rowCounts[row] = make_int4(a, q, 0, 0);
}

void launchRowCount(const GridDesc& g, float iso, int4* rowCounts, int numRows, cudaStream_t s) {
    countLaunch();
    if (g.refined) kRowCount<RefinedView><<<(numRows + 7) / 8, 256, 0, s>>>(g.ref, iso, rowCounts, numRows);
    else kRowCount<PlainView><<<(numRows + 7) / 8, 256, 0, s>>>(g.plain, iso, rowCounts, numRows);
}

// The active-cell mask: bit x of word (row, x / 32) is set when cell x of the
// row is active (case neither 0 nor 255).  Plain rows store whole ballots;
// refined rows visit only candidate cells and OR their bits into words
// cleared beforehand.
template <class View>
__global__ void __launch_bounds__(256) kRowMask(View g, float iso, uint32_t* __restrict__ mask, int numRows, int W,
                                                CaseBytes cases) {
    const int lane = threadIdx.x & 31;
    const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= numRows) return;
    const int y = row % (g.Y - 1), z = row / (g.Y - 1);
    uint32_t* words = mask + (int64_t)row * W;
    uint8_t* rowCases = cases.mode == 1 ? cases.p + ((size_t)z * g.Y + y) * g.X : nullptr;
    walkRow(g, y, z, lane, [&](int x, const float s[8]) {
        bool active = false;
        if (x < g.X - 1) {
            const int cs = caseOf(s, iso);
            active = cs != 0 && cs != 255;
            if (rowCases) rowCases[x] = (uint8_t)cs;
        }
        if constexpr (View::kRefined) {
            if (active) atomicOr(&words[x >> 5], 1u << (x & 31));
        } else {
            const unsigned ballot = __ballot_sync(0xffffffffu, active);
            if (lane == 0 && x < g.X - 1) words[x >> 5] = ballot;
        }
    });
}

void launchRowMask(const GridDesc& g, float iso, uint32_t* mask, int numRows, int W, CaseBytes cases, cudaStream_t s) {
    if (numRows <= 0) return;
    countLaunch();
    if (g.refined) kRowMask<RefinedView><<<(numRows + 7) / 8, 256, 0, s>>>(g.ref, iso, mask, numRows, W, CaseBytes{});
    else kRowMask<PlainView><<<(numRows + 7) / 8, 256, 0, s>>>(g.plain, iso, mask, numRows, W, cases);
}

// The linear cell id of every active cell, in row-major order: one thread
// per mask word; the index of the word's first active cell comes from the
// scan of the word counts.
__global__ void kScatterCells(const uint32_t* __restrict__ mask, const int* __restrict__ first, int64_t numWords, int W,
                              int X, int Y, uint32_t* __restrict__ cellIds, int numActive, uint32_t* status) {
    const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= numWords) return;
    uint32_t m = mask[w];
    if (!m) return;
    const uint32_t row = (uint32_t)w / (uint32_t)W;  // fewer than 2^32 words
    const int x0 = (int)((uint32_t)w - row * (uint32_t)W) * 32;
    const int y = row % (Y - 1), z = row / (Y - 1);
    const uint32_t base = (uint32_t)(((size_t)z * Y + y) * X + x0);
    int j = first[w];
    while (m) {
        const int b = __ffs(m) - 1;
        m &= m - 1;
        if (inb(j, numActive)) cellIds[j] = base + (uint32_t)b;
        else atomicOr(status, kStatusCountMismatch);
        ++j;
    }
}

// The same during the scan's apply pass, which has just computed the word's
// first index: ids beyond `capacity` are not written (the caller then runs
// kScatterCells once it knows the count and has the room).
struct CellScatter {
    static constexpr bool kStaged = false;
    static constexpr bool kPrefixes = true;
    const uint32_t* __restrict__ mask;
    uint32_t* __restrict__ cellIds;
    int64_t capacity;
    int W, X, Y;
    FastDiv divW, divRows;  // by W and by Y - 1 (multiplications instead of divisions)
    __device__ __forceinline__ void operator()(int64_t w, int first, int count) const {
        if (!count) return;
        uint32_t m = mask[w];
        const uint32_t row = divW.div((uint32_t)w);  // fewer than 2^32 words
        const int x0 = (int)((uint32_t)w - row * (uint32_t)W) * 32;
        const uint32_t zq = divRows.div(row);
        const int y = (int)(row - zq * (uint32_t)(Y - 1)), z = (int)zq;
        const uint32_t base = (uint32_t)(((size_t)z * Y + y) * X + x0);
        int64_t j = first;
        while (m) {
            const int b = __ffs(m) - 1;
            m &= m - 1;
            if (j < capacity) cellIds[j] = base + (uint32_t)b;
            ++j;
        }
    }
    __device__ __forceinline__ void total(int64_t, int) const {}
};

bool scanMaskScatter(const uint32_t* mask, int* first, int64_t numWords, int W, int X, int Y, uint32_t* cellIds,
                     int64_t capacity, int* scratch, cudaStream_t s) {
    return exclusiveScanOf<int>(PopcRead{mask}, first, numWords, scratch, s,
                                CellScatter{mask, cellIds, capacity, W, X, Y, FastDiv((uint32_t)W),
                                            FastDiv((uint32_t)(Y - 1))});
}

// The apply hook of the scan of the active cells' (vertex, quad) counts:
// each cell's first vertex and quad id into its record, the owner of each of
// its quads (the first capQ), and at the end the counts for the one read-back
// (gathered: active cells, vertices, quads; -1, -1 for the last two when
// there were more active cells than the scan covered).
struct FinishPost {
    static constexpr bool kStaged = true;
    static constexpr bool kPrefixes = false;  // (the records get the offsets; the counts array is not read)
    ActiveCell* __restrict__ act;
    int* __restrict__ quadOwner;
    int capQ;
    const int* numActiveDev;  // the uncapped active-cell count (nullptr: the scan's n)
    int capA;
    int* gathered;
    int* gatheredHost;  // the same three counts into mapped host memory (optional)
    __device__ __forceinline__ void operator()(int64_t i, int2 first, int2 count) const {
        act[i].pad = first.x;
        act[i].qbase = first.y;
        for (int r = 0; r < count.y; ++r)
            if (inb(first.y + r, capQ)) quadOwner[first.y + r] = (int)i;
    }
    __device__ __forceinline__ void total(int64_t n, int2 t) const {
        const int raw = numActiveDev ? *numActiveDev : (int)n;
        const bool all = raw >= 0 && raw <= capA;
        gathered[0] = raw;
        gathered[1] = all ? t.x : -1;
        gathered[2] = all ? t.y : -1;
        if (gatheredHost) {
            gatheredHost[0] = raw;
            gatheredHost[1] = all ? t.x : -1;
            gatheredHost[2] = all ? t.y : -1;
            __threadfence_system();
        }
    }
};

bool scanCellCounts(int2* counts, int64_t capA, const int* numActiveDev, ActiveCell* act, int* quadOwner, int64_t capQ,
                    int* gathered, int* gatheredHost, int2* scratch, cudaStream_t s) {
    return exclusiveScanOf<int2>(ArrayRead<int2>{counts}, counts, capA, scratch, s,
                                 FinishPost{act, quadOwner, (int)std::min<int64_t>(capQ, 0x7FFFFFFF), numActiveDev,
                                            (int)capA, gathered, gatheredHost},
                                 numActiveDev);
}

void launchScatterCells(const uint32_t* mask, const int* first, int64_t numWords, int W, int X, int Y, uint32_t* cellIds,
                        int numActive, uint32_t* status, cudaStream_t s) {
    if (numWords <= 0) return;
    countLaunch();
    kScatterCells<<<(unsigned)((numWords + 255) / 256), 256, 0, s>>>(mask, first, numWords, W, X, Y, cellIds, numActive,
                                                                     status);
}

// Records of the active cells: the cell, its case and edge -> contour map,
// and its number of contours (= vertices) and owned quads.  One thread per
// active cell; the corner samples come from the same column evaluation as
// the mask pass, so the case is the one that set the cell's mask bit.
template <class View>
__global__ void __launch_bounds__(128) kEmitActive(View g, float iso, const uint32_t* __restrict__ cellIds,
                                                   ActiveCell* __restrict__ act, int2* __restrict__ counts,
                                                   int numActive, const int* numActiveDev, CaseBytes cases,
                                                   uint32_t* status) {
    __shared__ uint32_t edgeMaps[256];  // per case: edge -> contour map | contours << 24
    for (int i = threadIdx.x; i < 256; i += blockDim.x) edgeMaps[i] = kCaseTables.edgeMaps[i];
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (numActiveDev) numActive = min(max(*numActiveDev, 0), numActive);
    if (j >= numActive) return;
    const uint32_t cell = cellIds[j];
    const uint32_t line = g.divX.div(cell), layer = g.divY.div(line);
    const int x = (int)(cell - line * (uint32_t)g.X), y = (int)(line - layer * (uint32_t)g.Y), z = (int)layer;
    if (x >= g.X - 1 || y >= g.Y - 1 || z >= g.Z - 1) {
        atomicOr(status, kStatusCountMismatch);
        return;
    }
    // the case the mask pass found, when it left one
    int cs = -1;
    if constexpr (View::kRefined) {
        if (cases.mode == 2) {
            const uint32_t coarse = ((uint32_t)(z >> 2) * (uint32_t)(g.cY - 1) + (uint32_t)(y >> 2)) *
                                        (uint32_t)(g.cX - 1) + (uint32_t)(x >> 2);
            cs = cases.p[(size_t)coarse * 64 + ((z & 3) << 4) + ((y & 3) << 2) + (x & 3)];
        }
    } else {
        if (cases.mode == 1) cs = cases.p[cell];
    }
    // the contours' edge map: the case's table entry, or from the asymptotic
    // decider's contours for the ambiguous cases (which need the corners)
    uint32_t em = cs >= 0 ? edgeMaps[cs] : 0xFFFFFFFFu;
    if (em == 0xFFFFFFFFu) {
        const RowWalker<View> walker(g, y, z);
        float cur[4], nxt[4];
        walker.load(x, cur);
        walker.load(x + 1, nxt);
        float s[8];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            s[2 * k] = cur[k];
            s[2 * k + 1] = nxt[k];
        }
        const int c2 = caseOf(s, iso);
        if (cs >= 0 && c2 != cs) atomicOr(status, kStatusCountMismatch);
        cs = c2;
        em = edgeMaps[cs];
        if (em == 0xFFFFFFFFu) em = kDecisionTables.edgeMaps[asymptoticEntry(s, iso)];
    }
    if (cs == 0 || cs == 255) {
        atomicOr(status, kStatusCountMismatch);
        return;
    }
    const int n = (int)(em >> 24);
    const uint32_t emap = em & 0xFFFFFFu;
    ActiveCell rec;
    rec.cell = cell;
    rec.qbase = 0;
    rec.info = (uint32_t)cs | (emap << 8);
    rec.pad = 0;
    act[j] = rec;
    counts[j] = make_int2(n, ownedQuads(cs, x, y, z));
}

void launchEmitActive(const GridDesc& g, float iso, const uint32_t* cellIds, ActiveCell* act, int2* counts,
                      int numActive, CaseBytes cases, uint32_t* status, cudaStream_t s, const int* numActiveDev) {
    if (numActive <= 0) return;
    countLaunch();
    const unsigned blocks = (unsigned)((numActive + 127) / 128);
    if (g.refined)
        kEmitActive<RefinedView><<<blocks, 128, 0, s>>>(g.ref, iso, cellIds, act, counts, numActive, numActiveDev,
                                                        cases, status);
    else
        kEmitActive<PlainView><<<blocks, 128, 0, s>>>(g.plain, iso, cellIds, act, counts, numActive, numActiveDev,
                                                      cases, status);
}

// ---------------------------------------------------------------------------
// vertices of the active cells (sliceP's vertex part, D/CellIntersection.inl:
// 368-439), one thread per active cell
// ---------------------------------------------------------------------------
// resident blocks per SM the register allocation aims at: 5 (96 registers)
// for the per-sample stencils (0.19 ms instead of 0.22 ms at 114 registers on
// the 512^3-cell blobs), 6 (80 registers, no spills) for the separable one
// (0.116 ms instead of 0.121 ms at 5); the pooled pass below: 7 (72
// registers, no spills; 256^3 noise 2.15 -> 2.0 ms against 5)
template <class Stencil>
struct VerticesBlocks {
    static constexpr int value = 5;
};
constexpr int kPooledVerticesBlocks = 7;
template <>
struct VerticesBlocks<SepStencil> {
    static constexpr int value = 6;
};
template <class View, class Stencil>
__global__ void __launch_bounds__(128, VerticesBlocks<Stencil>::value) kVertices(View g, float iso, int surfaceIteration,
                                                 const ActiveCell* __restrict__ act, int numActive,
                                                 int numVertices, float* __restrict__ pos,
                                                 float* __restrict__ nrm, int* __restrict__ degree,
                                                 uint8_t* __restrict__ flagsInit, int* __restrict__ starInit,
                                                 uint32_t* status, DeviceCounts counts) {
    if (counts.dev) {
        int a, v, q;
        if (!counts.fits(a, v, q)) return;
        numActive = a;
        numVertices = v;
    }
    __shared__ uint64_t table[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) table[i] = kCaseTables.words[i];  // ambiguous ones tagged
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= numActive) return;
    const ActiveCell rec = act[i];
    const uint32_t line = g.divX.div(rec.cell), layer = g.divY.div(line);
    const int x = (int)(rec.cell - line * (uint32_t)g.X);
    const int y = (int)(line - layer * (uint32_t)g.Y);
    const int z = (int)layer;
    const int vb = rec.pad;  // first vertex id
    const int cs = (int)(rec.info & 255u);
    const Stencil st(g, x, y, z);
    float s[8];
    stencilCorners(st, s);
    const uint64_t word = table[cs];
    const uint64_t c = taggedContours(word, s, iso);
    const int n = numContours(c);
    if (vb < 0 || vb + n > numVertices) {
        atomicOr(status, kStatusCountMismatch);
        return;
    }
    F3 normals[8];
    stencilGradients(st, s, g.deltas(), normals);
    const bool diagonalFace = word == 0;  // (the tag of ambiguous cases with a diagonal face)
    int before = 0;
    for (int t = 0; t < n; ++t) {
        F3 q = f3(0.f, 0.f, 0.f);
        int deg = 0;  // quads around the vertex: contour edges inside the grid's interior
        const int csz = nib(c, t);
        for (int k = 0; k < csz; ++k) {
            const int e = (int)((c >> (16 + 4 * (before + k))) & 0xF);
            const int a0 = edgeV0(e), a1 = edgeV1(e);
            {
                // the edge's start point; its quad exists when all four cells
                // around the edge do (the owner test of the quad pass)
                const int ea = edgeAxis(e);
                const int gx = x + (a0 & 1), gy = y + ((a0 >> 1) & 1), gz = z + ((a0 >> 2) & 1);
                deg += ((ea == 0 || (gx >= 1 && gx <= g.X - 2)) && (ea == 1 || (gy >= 1 && gy <= g.Y - 2)) &&
                        (ea == 2 || (gz >= 1 && gz <= g.Z - 2)))
                           ? 1
                           : 0;
            }
            const float w = (iso - s[a0]) / (s[a1] - s[a0]);
            // computeLocalCoordinateOffset (:176-200): the edge's axis gets the
            // crossing, the other two axes corner a0's coordinate
            const int ax = edgeAxis(e);
            q = q + f3(ax == 0 ? w : (float)(a0 & 1), ax == 1 ? w : (float)((a0 >> 1) & 1),
                       ax == 2 ? w : (float)((a0 >> 2) & 1));
        }
        before += csz;
        q = q / (float)csz;
        if (surfaceIteration) {
            SurfaceIterator it{s, iso};
            it.move(q);
        }
        const F3 nm = gnormalize(trilinear3(normals, q));
        const F3 wp = g.origin() + (f3((float)x, (float)y, (float)z) + q) * g.deltas();
        const int64_t vi = (int64_t)vb + t;
        pos[3 * vi] = wp.x;
        pos[3 * vi + 1] = wp.y;
        pos[3 * vi + 2] = wp.z;
        nrm[3 * vi] = nm.x;
        nrm[3 * vi + 1] = nm.y;
        nrm[3 * vi + 2] = nm.z;
        degree[vi] = deg == csz && !diagonalFace ? deg : -deg;
        if (flagsInit) {  // what the quad pass starts from (no flags, no outgoing halfedge yet)
            flagsInit[vi] = 0;
            starInit[vi] = 0x7F7F7F7F;
        }
    }
}

// Plain grids (where noise makes cells of several contours common): two
// phases per block of 128 active cells.  Phase 1, one thread per cell: the
// stencil, the corner values, the contours and the corner gradients go to
// shared memory, and the block's vertices (1 to 4 per cell) are listed there.
// Phase 2, one thread per vertex (each warp takes 32 of the list at a time):
// the mean of the contour's edge crossings, the surface iteration, the
// normal and the writes.  The same float operations as one thread doing all
// of a cell's vertices, with lanes no longer idle while another lane of the
// warp works through a second, third or fourth contour (256^3 noise: 5.5 ->
// 4.6 ms).  On smooth refined grids nearly every cell has one contour and
// the shared-memory round trip only costs (106 -> 127 us on the 512^3-cell
// blobs), so they keep kVertices, one thread per cell.
template <class View, class Stencil>
__global__ void __launch_bounds__(128, kPooledVerticesBlocks) kVerticesPooled(View g, float iso, int surfaceIteration,
                                                 const ActiveCell* __restrict__ act, int numActive,
                                                 int numVertices, float* __restrict__ pos,
                                                 float* __restrict__ nrm, int* __restrict__ degree,
                                                 uint8_t* __restrict__ flagsInit, int* __restrict__ starInit,
                                                 uint32_t* status, DeviceCounts counts) {
    if (counts.dev) {
        int a, v, q;
        if (!counts.fits(a, v, q)) return;
        numActive = a;
        numVertices = v;
    }
    __shared__ uint64_t table[256];
    __shared__ float cellS[128][8];        // corner values
    __shared__ float cellN[128][24];       // corner gradients
    __shared__ uint64_t cellC[128];        // contours
    __shared__ int cellXYZ[128][4];        // x, y, z, first vertex id
    __shared__ uint8_t cellDiag[128];      // an ambiguous case with a diagonal face
    __shared__ uint32_t items[512];        // cell slot | contour << 8 | edges before << 12
    __shared__ int warpSum[4];
    for (int k = threadIdx.x; k < 256; k += blockDim.x) table[k] = kCaseTables.words[k];  // ambiguous ones tagged
    __syncthreads();
    const int slot = threadIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int n = 0;
    if (i < numActive) {
        const ActiveCell rec = act[i];
        const uint32_t line = g.divX.div(rec.cell), layer = g.divY.div(line);
        const int x = (int)(rec.cell - line * (uint32_t)g.X);
        const int y = (int)(line - layer * (uint32_t)g.Y);
        const int z = (int)layer;
        const int vb = rec.pad;  // first vertex id
        const int cs = (int)(rec.info & 255u);
        const Stencil st(g, x, y, z);
        float sv[8];
        stencilCorners(st, sv);
        const uint64_t word = table[cs];
        const uint64_t c = taggedContours(word, sv, iso);
        n = numContours(c);
        if (vb < 0 || vb + n > numVertices) {
            atomicOr(status, kStatusCountMismatch);
            n = 0;
        } else {
            F3 gr[8];
            stencilGradients(st, sv, g.deltas(), gr);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                cellS[slot][k] = sv[k];
                cellN[slot][3 * k] = gr[k].x;
                cellN[slot][3 * k + 1] = gr[k].y;
                cellN[slot][3 * k + 2] = gr[k].z;
            }
            cellC[slot] = c;
            cellXYZ[slot][0] = x;
            cellXYZ[slot][1] = y;
            cellXYZ[slot][2] = z;
            cellXYZ[slot][3] = vb;
            cellDiag[slot] = word == 0 ? 1 : 0;  // (the tag of ambiguous cases with a diagonal face)
        }
    }
    // the block's vertex list: exclusive scan of the contour counts
    int incl = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) warpSum[warp] = incl;
    __syncthreads();
    int off = incl - n, total = 0;
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        if (w < warp) off += warpSum[w];
        total += warpSum[w];
    }
    if (n > 0) {
        const uint64_t c = cellC[slot];
        int before = 0;
        for (int t = 0; t < n; ++t) {
            items[off + t] = (uint32_t)slot | ((uint32_t)t << 8) | ((uint32_t)before << 12);
            before += nib(c, t);
        }
    }
    __syncthreads();
    for (int k = warp * 32 + lane; k - lane < total; k += 128) {
        if (k >= total) continue;
        const uint32_t it = items[k];
        const int cslot = (int)(it & 255u), t = (int)((it >> 8) & 3u), before = (int)(it >> 12);
        const int x = cellXYZ[cslot][0], y = cellXYZ[cslot][1], z = cellXYZ[cslot][2], vb = cellXYZ[cslot][3];
        const uint64_t c = cellC[cslot];
        float sv[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) sv[q] = cellS[cslot][q];
        F3 q = f3(0.f, 0.f, 0.f);
        int deg = 0;  // quads around the vertex: contour edges inside the grid's interior
        const int csz = nib(c, t);
        for (int k2 = 0; k2 < csz; ++k2) {
            const int e = (int)((c >> (16 + 4 * (before + k2))) & 0xF);
            const int a0 = edgeV0(e), a1 = edgeV1(e);
            {
                // the edge's start point; its quad exists when all four cells
                // around the edge do (the owner test of the quad pass)
                const int ea = edgeAxis(e);
                const int gx = x + (a0 & 1), gy = y + ((a0 >> 1) & 1), gz = z + ((a0 >> 2) & 1);
                deg += ((ea == 0 || (gx >= 1 && gx <= g.X - 2)) && (ea == 1 || (gy >= 1 && gy <= g.Y - 2)) &&
                        (ea == 2 || (gz >= 1 && gz <= g.Z - 2)))
                           ? 1
                           : 0;
            }
            const float w = (iso - sv[a0]) / (sv[a1] - sv[a0]);
            // computeLocalCoordinateOffset (:176-200): the edge's axis gets the
            // crossing, the other two axes corner a0's coordinate
            const int ax = edgeAxis(e);
            q = q + f3(ax == 0 ? w : (float)(a0 & 1), ax == 1 ? w : (float)((a0 >> 1) & 1),
                       ax == 2 ? w : (float)((a0 >> 2) & 1));
        }
        q = q / (float)csz;
        if (surfaceIteration) {
            SurfaceIterator itr{sv, iso};
            itr.move(q);
        }
        F3 normals[8];
#pragma unroll
        for (int m = 0; m < 8; ++m)
            normals[m] = f3(cellN[cslot][3 * m], cellN[cslot][3 * m + 1], cellN[cslot][3 * m + 2]);
        const F3 nm = gnormalize(trilinear3(normals, q));
        const F3 wp = g.origin() + (f3((float)x, (float)y, (float)z) + q) * g.deltas();
        const int64_t vi = (int64_t)vb + t;
        pos[3 * vi] = wp.x;
        pos[3 * vi + 1] = wp.y;
        pos[3 * vi + 2] = wp.z;
        nrm[3 * vi] = nm.x;
        nrm[3 * vi + 1] = nm.y;
        nrm[3 * vi + 2] = nm.z;
        degree[vi] = deg == csz && !cellDiag[cslot] ? deg : -deg;
        if (flagsInit) {  // what the quad pass starts from (no flags, no outgoing halfedge yet)
            flagsInit[vi] = 0;
            starInit[vi] = 0x7F7F7F7F;
        }
    }
}

void launchVertices(const GridDesc& g, float iso, int surfaceIteration, const ActiveCell* act, int numActive,
                    int numVertices, float* pos, float* nrm, int* degree, uint8_t* flagsInit, int* starInit,
                    uint32_t* status, cudaStream_t s, const DeviceCounts* counts) {
    if (numActive <= 0) return;
    countLaunch();
    const unsigned blocks = (unsigned)((numActive + 127) / 128);
    const DeviceCounts dc = counts ? *counts : DeviceCounts{nullptr, 0, 0, 0};
    if (g.refined && sepStencilApplies(g.ref.r, g.ref.X, g.ref.Y, g.ref.Z))
        kVertices<RefinedView, SepStencil><<<blocks, 128, 0, s>>>(g.ref, iso, surfaceIteration, act, numActive,
                                                                  numVertices, pos, nrm, degree, flagsInit, starInit, status, dc);
    else if (g.refined)
        kVertices<RefinedView, CellStencil<RefinedView>><<<blocks, 128, 0, s>>>(
            g.ref, iso, surfaceIteration, act, numActive, numVertices, pos, nrm, degree, flagsInit, starInit, status, dc);
    else
        kVerticesPooled<PlainView, CellStencil<PlainView>><<<blocks, 128, 0, s>>>(
            g.plain, iso, surfaceIteration, act, numActive, numVertices, pos, nrm, degree, flagsInit, starInit, status, dc);
}

// ---------------------------------------------------------------------------
// cell index: the active-cell mask of every x-row of cells (32 cells per word)
// and, per word, the index of its first active cell in the active-cell list,
// so a cell's record is one load away
// ---------------------------------------------------------------------------
struct CellIndex {
    const uint32_t* mask;
    const int* first;
    int X, Y, Z, W;
    FastDiv divX, divY;  // by X and Y (decoding linear cell ids)
    // index of cell (x,y,z) in the active-cell list, -1 if inactive or outside.
    // Without a branch: a cell outside reads word 0 and is then rejected, so
    // that a caller's lookups can all be in flight together.
    __device__ __forceinline__ int find(int x, int y, int z) const {
        const bool in =
            (unsigned)x <= (unsigned)(X - 2) && (unsigned)y <= (unsigned)(Y - 2) && (unsigned)z <= (unsigned)(Z - 2);
        // (mask words number fewer than 2^27: grids have fewer than 2^32 samples)
        const uint32_t w = in ? ((uint32_t)z * (uint32_t)(Y - 1) + (uint32_t)y) * (uint32_t)W + (uint32_t)(x >> 5) : 0u;
        const uint32_t m = __ldg(mask + w);
        const int f = __ldg(first + w);
        const uint32_t bit = 1u << (x & 31);
        return (in && (m & bit)) ? f + __popc(m & (bit - 1u)) : -1;
    }
};

// does the cell at (x,y,z) with case cs own the quad of its corner-0 edge along axis
__device__ __forceinline__ bool ownsAxis(int cs, int axis, int x, int y, int z) {
    if (!((cs ^ (cs >> (1 << axis))) & 1)) return false;
    if (axis == 0) return y >= 1 && z >= 1;
    if (axis == 1) return x >= 1 && z >= 1;
    return x >= 1 && y >= 1;
}

// local index of the cell edge leaving corner `corner` (bit 0 x, 1 y, 2 z)
// along `axis`; the corner's bit for that axis is 0
__host__ __device__ constexpr int localEdge(int corner, int axis) {
    if (axis == 0) return corner;                                                        // 0, 2, 4, 6
    if (axis == 1) return (0x5713 >> (4 * ((corner & 1) | ((corner >> 1) & 2)))) & 0xF;  // 3, 1, 7, 5
    return (0xAB98 >> (4 * corner)) & 0xF;                                               // 8, 9, 11, 10
}

__device__ __forceinline__ int axisBit(int a) { return 1 << a; }

// The fixed geometry of a quad's halfedges, by the quad's axis a, the sign of
// its owner cell's corner 0 (edgy: the slot order of the four cells around the
// quad's edge) and the halfedge's slot hi.  Cell k around the edge is
// p - (k & 1) e_b - (k >> 1) e_c (b < c the other axes); halfedge hi runs from
// the vertex of cell A (slot hi) to that of cell B (slot hi + 1), which share a
// face.  The only quads that can hold the same vertex pair are those of the
// face's three other grid edges: cand 0 parallel to the quad's edge on the
// face's far side, cand 1 and 2 across the face at the edge's lower and upper
// end.
//   head[6 * hi + 2 * a + edgy]: cell A's k (2 bits) and A's local index of
//     the quad's edge (4), then per candidate the two corners (3 + 3) of its
//     edge in A (the edge crosses iso when their signs differ);
//   cand[6 * (3 * hi + cand) + 2 * a + edgy]: the candidate edge's local index
//     in A and in B (4 + 4), its axis (2), which loaded record holds its owner
//     cell (4: 0..2 cells around the quad's edge, 4..8 the five others), the
//     owner's offset from p plus one along x, y, z (2 + 2 + 2), and for each
//     sign of A's corner at the edge's start the shared halfedge's slot in the
//     candidate quad (2), "its origin is A's vertex" (1) and "valid" (1).
// Built at compile time from the same index arithmetic a per-halfedge
// evaluation would run.
struct QuadGeom {
    uint32_t head[24];
    uint32_t cand[72];
};

constexpr QuadGeom makeQuadGeom() {
    QuadGeom g{};
    for (int axis = 0; axis < 3; ++axis)
        for (int edgy = 0; edgy < 2; ++edgy) {
            const int ae = 2 * axis + edgy;
            const int b = axis == 0 ? 1 : 0, c = axis == 2 ? 1 : 2;
            const int leWord = axis == 0 ? 0x6420 : (axis == 1 ? 0x5713 : 0xAB98);
            int le[4] = {0, 0, 0, 0}, quadK[4] = {0, 0, 0, 0};
            for (int k = 0; k < 4; ++k) le[k] = (leWord >> (4 * k)) & 0xF;
            // slot -> cell: edges with v0 inside take the reverse cycle
            // (quadSlot, computeVertexPosition, D/CellIntersection.inl:361-366)
            for (int k = 0; k < 4; ++k) quadK[quadSlot(le[k], edgy)] = k;
            for (int hi = 0; hi < 4; ++hi) {
                const int kA = quadK[hi], kB = quadK[(hi + 1) & 3];
                // A and B differ along t (bit 0 of k: along b, bit 1: along c);
                // u is the remaining axis of the face
                const bool alongB = ((kA ^ kB) & 1) != 0;
                const int t = alongB ? b : c, u = alongB ? c : b;
                const int aMinusT = alongB ? (kA & 1) : (kA >> 1);  // A = p - e_t ?
                const int aMinusU = alongB ? (kA >> 1) : (kA & 1);  // A = p - e_u ?
                // A's corner offsets of the face's grid edges: the t offset is 1
                // where A lies below the face
                const int cT = aMinusT, cTB = 1 - aMinusT;
                uint32_t head = (uint32_t)kA | ((uint32_t)le[kA] << 2);
                for (int cand = 0; cand < 3; ++cand) {
                    const int al = cand == 0 ? axis : u;
                    const int offU = cand == 0 ? (aMinusU ? 0 : 1) : 0;
                    const int offA = cand == 2 ? 1 : 0;
                    const int ca = (cT << t) | (offU << u) | (offA << axis);
                    const int cb = (cTB << t) | (offU << u) | (offA << axis);
                    const int eA = localEdge(ca, al), eB = localEdge(cb, al);
                    head |= (uint32_t)(edgeV0(eA) | (edgeV1(eA) << 3)) << (6 + 6 * cand);
                    // the grid edge's origin: p + du e_u + offA e_a; its owner is a
                    // cell around the quad's edge (p, p - e_u) or p + e_u (du = 1),
                    // p + e_a (du = 0) or p - e_u + e_a (du = -1)
                    const int du = offU - aMinusU;
                    int d[3] = {0, 0, 0};
                    for (int x = 0; x < 3; ++x) d[x] = (u == x ? du : 0) + (axis == x ? offA : 0);
                    const int ko = du == 0 ? 0 : (u == b ? 1 : 2);
                    const int kx = offA == 0 ? (u == b ? 0 : 1) : (du == 0 ? 2 : (u == b ? 3 : 4));
                    const int slot = (offA == 0 && du <= 0) ? ko : 4 + kx;
                    uint32_t code[2] = {0, 0};
                    for (int eo = 0; eo < 2; ++eo) {
                        const int sA = quadSlot(eA, eo), sB = quadSlot(eB, eo);
                        if (((sA + 1) & 3) == sB) code[eo] = (uint32_t)sA | 4u | 8u;
                        else if (((sB + 1) & 3) == sA) code[eo] = (uint32_t)sB | 8u;
                    }
                    g.cand[6 * (3 * hi + cand) + ae] =
                        (uint32_t)eA | ((uint32_t)eB << 4) | ((uint32_t)al << 8) | ((uint32_t)slot << 10) |
                        ((uint32_t)(d[0] + 1) << 14) | ((uint32_t)(d[1] + 1) << 16) | ((uint32_t)(d[2] + 1) << 18) |
                        (code[0] << 20) | (code[1] << 24);
                }
                g.head[6 * hi + ae] = head;
            }
        }
    return g;
}
__device__ const QuadGeom kQuadGeom = makeQuadGeom();

// The quads (mapQuadrilaterals, D/DualMarchingCubes.cu:72-85), their halfedges
// (collectHalfedgeElements, D/Halfedges/HalfedgeMesh.cu:14-60) and the twins
// and flags of connectHalfedgeTwins / refresh*Flags (:92-291), without an edge
// table, one thread per quad.  Halfedge i of quad q runs between the vertices
// of the face-adjacent cells A (slot i) and B (slot i+1); the only quads that
// can hold the same vertex pair are those of the four grid edges of the A|B
// face, and each of them does exactly when its edge lies in the same contours
// of A and of B.  That set is the reference's edge-table bucket; sorted, it
// gives the twins by the reference's rules.  The nine cell records a quad
// needs sit in the thread's own column of shared memory, so that a record
// picked by a table entry is one load, not a chain of selects.
#ifndef MDMC_QUADS_MIN_BLOCKS
#define MDMC_QUADS_MIN_BLOCKS 4
#endif
constexpr int kQuadThreads = 256;
__global__ void __launch_bounds__(kQuadThreads, MDMC_QUADS_MIN_BLOCKS) kQuads(const ActiveCell* __restrict__ act, const int* __restrict__ quadOwner,
                                              int numActive, CellIndex ix, int4* __restrict__ he,
                                              int* __restrict__ faceFirst, uint16_t* __restrict__ faceAttr,
                                              uint8_t* vflags, uint32_t* __restrict__ heValence4,
                                              int4* __restrict__ nmList, int nmCapacity, int numQuads, int numVertices,
                                              int4* __restrict__ quadsOut, int* vertexHE,
                                              DevCounters* ctr, int qBegin, int qEnd) {
    __shared__ uint32_t sHead[24], sCand[72];
    // records: 0..3 the cells around the quad's edge (k), 4..8 the five others
    __shared__ uint32_t sInfo[9][kQuadThreads];
    __shared__ int sQbase[9][kQuadThreads];
    __shared__ int sVbase[4][kQuadThreads];
    for (int i = threadIdx.x; i < 96; i += blockDim.x) {
        if (i < 24) sHead[i] = kQuadGeom.head[i];
        else sCand[i - 24] = kQuadGeom.cand[i - 24];
    }
    __syncthreads();
    const int tid = threadIdx.x;
    const int q = qBegin + blockIdx.x * blockDim.x + threadIdx.x;
    int nE = 0, nE3 = 0, nE4 = 0;
    int nmEdges = -1;  // halfedges of this quad on edges of more than two faces
    bool ok = q < qEnd && q < numQuads;
    const int j = ok ? quadOwner[q] : 0;
    if (ok && !inb(j, numActive)) {
        atomicOr(&ctr->status, kStatusBadIndex);
        ok = false;
    }
    if (ok) {
        const ActiveCell rec = act[j];
        const int cs = (int)(rec.info & 255u);
        const uint32_t line = ix.divX.div(rec.cell), layer = ix.divY.div(line);
        const int px = (int)(rec.cell - line * (uint32_t)ix.X), py = (int)(line - layer * (uint32_t)ix.Y),
                  pz = (int)layer;
        // the rank-th owned axis of the owner
        int axis = -1, rank = q - rec.qbase;
#pragma unroll
        for (int a = 0; a < 3; ++a)
            if (axis < 0 && ownsAxis(cs, a, px, py, pz) && rank-- == 0) axis = a;
        if (axis < 0) {
            atomicOr(&ctr->status, kStatusBadIndex);
            ok = false;
        }
        if (ok) {
            // the other axes b < c; cell k = p - (k&1) e_b - (k>>1) e_c
            const int b = axis == 0 ? 1 : 0, c = axis == 2 ? 1 : 2;
            // the cells around the quad's edge (k = 1..3), and the five other
            // cells that can own a quad of one of the face buckets:
            // p + e_b, p + e_c, p + e_a, p - e_b + e_a, p - e_c + e_a.  All
            // eight lookups are issued before any record is used.
            int jk[4], jx[5];
            jk[0] = j;
#pragma unroll
            for (int k = 1; k < 4; ++k) {
                const int db = k & 1, dc = k >> 1;
                jk[k] = ix.find(px - (b == 0 ? db : 0) - (c == 0 ? dc : 0), py - (b == 1 ? db : 0) - (c == 1 ? dc : 0),
                                pz - (c == 2 ? dc : 0));
            }
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                const int dA = k >= 2 ? 1 : 0;
                const int dB = k == 0 ? 1 : (k == 3 ? -1 : 0);
                const int dC = k == 1 ? 1 : (k == 4 ? -1 : 0);
                jx[k] = ix.find(px + (axis == 0 ? dA : 0) + (b == 0 ? dB : 0),
                                py + (axis == 1 ? dA : 0) + (b == 1 ? dB : 0) + (c == 1 ? dC : 0),
                                pz + (axis == 2 ? dA : 0) + (c == 2 ? dC : 0));
            }
            // the eight records, all loads issued before any is used (a
            // missing cell loads record j and is then replaced)
            ActiveCell r2[8];
#pragma unroll
            for (int k = 0; k < 3; ++k) r2[k] = act[inb(jk[k + 1], numActive) ? jk[k + 1] : j];
#pragma unroll
            for (int k = 0; k < 5; ++k) r2[3 + k] = act[inb(jx[k], numActive) ? jx[k] : j];
            sInfo[0][tid] = rec.info;
            sQbase[0][tid] = rec.qbase;
            sVbase[0][tid] = rec.pad;
#pragma unroll
            for (int k = 1; k < 4; ++k) {
                const bool have = inb(jk[k], numActive);
                if (!have) ok = false;
                sInfo[k][tid] = have ? r2[k - 1].info : 0u;
                sQbase[k][tid] = have ? r2[k - 1].qbase : 0;
                sVbase[k][tid] = have ? r2[k - 1].pad : 0;
            }
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                const bool have = inb(jx[k], numActive);
                sInfo[4 + k][tid] = have ? r2[3 + k].info : 0u;
                sQbase[4 + k][tid] = have ? r2[3 + k].qbase : -1;  // -1: no such active cell
            }
            if (!ok) atomicOr(&ctr->status, kStatusMissingCell);
            const int ae = 2 * axis + ((cs & 1) ? 0 : 1);
            // per slot: its cell's record, the contour of the quad's edge in
            // that cell, and the vertex (the slot's halfedge's origin)
            uint32_t head[4], info[4];
            int contour[4], quadV[4];
#pragma unroll
            for (int sl = 0; sl < 4; ++sl) {
                head[sl] = sHead[6 * sl + ae];
                const int k = (int)(head[sl] & 3u);
                info[sl] = sInfo[k][tid];
                contour[sl] = (int)((info[sl] >> (8 + 2 * ((head[sl] >> 2) & 15u))) & 3u);
                quadV[sl] = sVbase[k][tid] + contour[sl];
                if (!inb(quadV[sl], numVertices)) ok = false;
            }
            if (!ok) {
                atomicOr(&ctr->status, kStatusCountMismatch);
            } else {
                const int h0 = 4 * q;
                const int baseColor = (px & 1) | ((py & 1) << 1) | ((pz & 1) << 2);
                uint32_t attr = (uint32_t)(3 * baseColor + axis);
                uint32_t valences = 0;
                int4 out[4];
#pragma unroll
                for (int hi = 0; hi < 4; ++hi) {
                    const uint32_t infoA = info[hi], infoB = info[(hi + 1) & 3];
                    const int tA = contour[hi], tB = contour[(hi + 1) & 3];
                    const uint32_t csA = infoA & 255u;
                    const uint32_t hd = head[hi];
                    const int self = h0 + hi;
                    int ids[4], org[4];
                    ids[0] = self;
                    org[0] = quadV[hi];
                    ids[1] = ids[2] = ids[3] = 0x7FFFFFFF;
                    org[1] = org[2] = org[3] = -1;
                    // The candidates that cross iso are found first and then gone
                    // through with one body of code, so that lanes whose crossing
                    // edge is a different candidate run it together.
                    uint32_t crossing = 0;
#pragma unroll
                    for (int cand = 0; cand < 3; ++cand)
                        crossing |= (((csA >> ((hd >> (6 + 6 * cand)) & 7u)) ^ (csA >> ((hd >> (9 + 6 * cand)) & 7u))) &
                                     1u) << cand;
                    // (the three table entries are loaded before the loop, and the
                    // owner record of a candidate before its tests, so that each
                    // iteration waits on one shared load at most)
                    const uint32_t en0 = sCand[6 * (3 * hi) + ae], en1 = sCand[6 * (3 * hi + 1) + ae],
                                   en2 = sCand[6 * (3 * hi + 2) + ae];
                    int found = 0;
                    while (crossing) {
                        const int cand = __ffs(crossing) - 1;
                        crossing &= crossing - 1;
                        const uint32_t en = cand == 0 ? en0 : (cand == 1 ? en1 : en2);
                        const int slot = (int)((en >> 10) & 15u);
                        const int oqbase = sQbase[slot][tid];
                        const uint32_t oinfo = sInfo[slot][tid];
                        if ((int)((infoA >> (8 + 2 * (en & 15u))) & 3u) != tA) continue;
                        if ((int)((infoB >> (8 + 2 * ((en >> 4) & 15u))) & 3u) != tB) continue;
                        // the grid edge's origin and the quad its owner holds
                        const int al = (int)((en >> 8) & 3u);
                        const int ox = px + (int)((en >> 14) & 3u) - 1;
                        const int oy = py + (int)((en >> 16) & 3u) - 1;
                        const int oz = pz + (int)((en >> 18) & 3u) - 1;
                        if (((al != 0 && ox < 1) || (al != 1 && oy < 1) || (al != 2 && oz < 1))) continue;
                        if (oqbase < 0) continue;
                        const int cso = (int)(oinfo & 255u);
                        if (!ownsAxis(cso, al, ox, oy, oz)) continue;
                        int r = 0;
#pragma unroll
                        for (int a2 = 0; a2 < 2; ++a2)
                            if (a2 < al && ownsAxis(cso, a2, ox, oy, oz)) ++r;
                        const int q2 = oqbase + r;
                        // the shared halfedge's slot in that quad, by the sign of
                        // A's corner at the candidate edge's start
                        const uint32_t v0 = (hd >> (6 + 6 * cand)) & 7u;
                        const uint32_t code = (en >> (((csA >> v0) & 1u) ? 20 : 24)) & 15u;
                        int id = 0x7FFFFFFF, o = -1;
                        if (code & 8u) {
                            id = 4 * q2 + (int)(code & 3u);
                            o = (code & 4u) ? quadV[hi] : quadV[(hi + 1) & 3];
                            ++found;
                        } else {
                            atomicOr(&ctr->status, kStatusBadIndex);
                        }
                        if (cand == 0) {
                            ids[1] = id;
                            org[1] = o;
                        } else if (cand == 1) {
                            ids[2] = id;
                            org[2] = o;
                        } else {
                            ids[3] = id;
                            org[3] = o;
                        }
                    }
                    const int n = 1 + found;
                    int me = 0, twin = -1;
                    if (found <= 1) {  // at most one other halfedge: the pair needs no sorting
                        const int other = min(ids[1], min(ids[2], ids[3]));
                        if (found == 1) {
                            twin = other;
                            me = other < self ? 1 : 0;
                        }
                    } else {
                        // sort the bucket (absent entries last) with its origins
#define MDMC_CX(i0, i1)                                   \
    if (ids[i1] < ids[i0]) {                              \
        const int ti = ids[i0], to = org[i0];             \
        ids[i0] = ids[i1];                                \
        org[i0] = org[i1];                                \
        ids[i1] = ti;                                     \
        org[i1] = to;                                     \
    }
                        MDMC_CX(0, 1) MDMC_CX(2, 3) MDMC_CX(0, 2) MDMC_CX(1, 3) MDMC_CX(1, 2)
#undef MDMC_CX
                        me = (ids[1] == self) ? 1 : (ids[2] == self) ? 2 : (ids[3] == self) ? 3 : 0;
                        int partner = -1;
                        if (n == 3) {
                            partner = me == 2 ? 0 : me + 1;
                        } else if (n == 4) {  // "HACKY_OLD_WAY", HalfedgeMesh.cu:250-281
                            if (org[0] != org[1]) partner = me ^ 1;       // (0,1) (2,3)
                            else if (org[0] != org[2]) partner = me ^ 2;  // (0,2) (1,3)
                            else partner = 3 - me;                        // (0,3) (1,2)
                        }
#pragma unroll
                        for (int t2 = 0; t2 < 4; ++t2)
                            if (partner == t2) twin = ids[t2];
                    }
                    out[hi] = make_int4(quadV[hi], q, h0 + ((hi + 1) & 3), twin);
                    valences |= (uint32_t)n << (8 * hi);
                    const int origin = quadV[hi];
                    if (n == 4) {
                        attr |= MDMC_FACE_NON_MANIFOLD;
                        orVertexFlag(vflags, origin, MDMC_VERTEX_NON_MANIFOLD);
                    } else if (n == 3) {
                        orVertexFlag(vflags, origin, MDMC_VERTEX_WEIRD);
                    } else if (n == 1) {
                        orVertexFlag(vflags, origin, MDMC_VERTEX_BOUNDARY);
                    }
                    if (me == 0) {  // the bucket's smallest halfedge counts it
                        ++nE;
                        if (n == 3) ++nE3;
                        if (n == 4) {
                            ++nE4;
                            const unsigned long long slot = atomicAdd(&ctr->nmBuckets, 1ULL);
                            if (slot < (unsigned long long)nmCapacity)
                                nmList[slot] = make_int4(ids[0], ids[1], ids[2], ids[3]);
                            else
                                atomicOr(&ctr->status, kStatusBadIndex);
                        }
                    }
                }
#pragma unroll
                for (int hi = 0; hi < 4; ++hi) he[h0 + hi] = out[hi];
                heValence4[q] = valences;
                faceFirst[q] = h0;
                faceAttr[q] = (uint16_t)attr;
                // what the output pass reads off the finished mesh, valid while
                // no later pass changes faces or vertices: the face's vertices,
                // its count of edges with more than two faces, each vertex's
                // smallest outgoing halfedge and out-degree
                quadsOut[q] = make_int4(quadV[0], quadV[1], quadV[2], quadV[3]);
                nmEdges = 0;
#pragma unroll
                for (int hi = 0; hi < 4; ++hi) {
                    nmEdges += ((valences >> (8 * hi)) & 0xFFu) > 2 ? 1 : 0;
                    atomicMin(&vertexHE[quadV[hi]], h0 + hi);
                }
            }
        }
    }
    // the seven counters packed into one word for one warp reduction: edges
    // (<= 4 per quad) in 16 bits, the others (<= 4, <= 1 per quad) in 8 bits
    unsigned long long packed = (unsigned long long)nE | ((unsigned long long)nE3 << 16) |
                                ((unsigned long long)nE4 << 24);
#pragma unroll
    for (int k = 1; k <= 4; ++k) packed |= (unsigned long long)(nmEdges == k ? 1 : 0) << (24 + 8 * k);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) packed += __shfl_down_sync(0xffffffffu, packed, o);
    if ((threadIdx.x & 31) == 0 && packed) {
        const unsigned long long e = packed & 0xFFFFu, e3 = (packed >> 16) & 0xFFu, e4 = (packed >> 24) & 0xFFu;
        if (e) atomicAdd(&ctr->edges, e);
        if (e3) atomicAdd(&ctr->edges3, e3);
        if (e4) atomicAdd(&ctr->edges4, e4);
#pragma unroll
        for (int k = 1; k <= 4; ++k) {
            const unsigned long long qk = (packed >> (24 + 8 * k)) & 0xFFu;
            if (qk) atomicAdd(&ctr->quadsNM[k], qk);
        }
    }
}

void launchQuads(const ActiveCell* act, const int* quadOwner, int numActive, const uint32_t* cellMask,
                 const int* cellFirst, int X, int Y, int Z, int W, int4* he, int* faceFirst, uint16_t* faceAttr,
                 uint8_t* vflags, uint8_t* heValence, int4* nmList, int nmCapacity, int numQuads, int numVertices,
                 int4* quadsOut, int* vertexHE, DevCounters* ctr, int qBegin, int qEnd, cudaStream_t s) {
    if (qEnd <= qBegin) return;
    countLaunch();
    CellIndex ix;
    ix.mask = cellMask;
    ix.first = cellFirst;
    ix.X = X;
    ix.Y = Y;
    ix.Z = Z;
    ix.W = W;
    ix.divX = FastDiv((uint32_t)X);
    ix.divY = FastDiv((uint32_t)Y);
    kQuads<<<(qEnd - qBegin + kQuadThreads - 1) / kQuadThreads, kQuadThreads, 0, s>>>(act, quadOwner, numActive, ix, he, faceFirst, faceAttr, vflags,
                                                        reinterpret_cast<uint32_t*>(heValence), nmList, nmCapacity,
                                                        numQuads, numVertices, quadsOut, vertexHE, ctr, qBegin,
                                                        qEnd);
}

}  // namespace mdmc
