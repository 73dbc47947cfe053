// Grid preparation and the Dual Marching Cubes stage.
//
// Reference: performDualMarchingCubes + mapQuadrilaterals
// (D/DualMarchingCubes.cu:38-85), CellIntersection::sliceP
// (D/CellIntersection.inl:368-439), collectHalfedgeElements
// (D/Halfedges/HalfedgeMesh.cu:14-60), refineGrid (D/UniformGrid.inl:279-319).
//
// GB300 design: one warp per x-row of cells.  Two streaming passes over the
// grid (count, emit) replace the reference's single global atomic vertex
// counter and its 20M-bucket quad hash table: the count pass gives per-row
// (active cells, vertices, owned quads), an exclusive scan turns them into
// row offsets, and the emit pass writes vertices and active-cell records at
// deterministic offsets using warp ballots and shuffles.  Each quad is then
// built by the cell that owns its grid edge (the cell at the edge's origin),
// which looks up the three other cells' records by row, so no quad hash is
// needed; the same thread writes the quad's four halfedges and inserts its
// edges into the edge table.
#include <cuda_runtime.h>

#include "mdmc_device.cuh"
#include "mdmc_edge_hash.cuh"
#include "mdmc_kernels.h"

namespace mdmc {

// ---------------------------------------------------------------------------
// refineGrid, D/UniformGrid.inl:279-319
// ---------------------------------------------------------------------------
__global__ void kRefine(const float* __restrict__ in, int3 din, float* __restrict__ out, int3 dout, int r,
                        int pad) {
    const int64_t n = (int64_t)dout.x * dout.y * dout.z;
    const float f = (float)(r + 1);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int x = (int)(i % dout.x);
        int y = (int)((i / dout.x) % dout.y);
        int z = (int)(i / ((int64_t)dout.x * dout.y));
        if (pad) {
            x = min(max(x, 1), dout.x - 2) - 1;
            y = min(max(y, 1), dout.y - 2) - 1;
            z = min(max(z, 1), dout.z - 2) - 1;
        }
        float qx = (float)x / f, qy = (float)y / f, qz = (float)z / f;
        int mx = (int)floorf(qx), my = (int)floorf(qy), mz = (int)floorf(qz);
        F3 diff = f3(qx - (float)mx, qy - (float)my, qz - (float)mz);
        float s[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            int cx = min(max(mx + (c & 1), 0), din.x - 1);
            int cy = min(max(my + ((c >> 1) & 1), 0), din.y - 1);
            int cz = min(max(mz + ((c >> 2) & 1), 0), din.z - 1);
            s[c] = __ldg(in + ((int64_t)cz * din.y + cy) * din.x + cx);
        }
        out[i] = trilinear(s, diff);
    }
}

void launchRefine(const float* in, int3 din, float* out, int3 dout, int r, int pad, cudaStream_t s) {
    const int64_t n = (int64_t)dout.x * dout.y * dout.z;
    int blocks = (int)std::min<int64_t>((n + 255) / 256, 152 * 32);
    countLaunch();
    kRefine<<<blocks, 256, 0, s>>>(in, din, out, dout, r, pad);
}

// ---------------------------------------------------------------------------
// cell classification
// ---------------------------------------------------------------------------
struct CellClass {
    int cs;      // case
    int nv;      // vertices (contours)
    int nq;      // quads owned
    uint64_t c;  // contour word
};

// cells are interior (x <= X-2, ...), so the reference's clamped corner fetch
// (D/UniformGrid.inl:414-427) reads the unclamped corners
__device__ __forceinline__ void classify(const GridView& g, int x, int y, int z, float iso,
                                         const uint64_t* table, float s[8], CellClass& cc) {
    const float* p = g.v + ((size_t)z * g.Y + y) * g.X + x;
    const size_t sy = g.X, sz = (size_t)g.X * g.Y;
    s[0] = __ldg(p);
    s[1] = __ldg(p + 1);
    s[2] = __ldg(p + sy);
    s[3] = __ldg(p + sy + 1);
    s[4] = __ldg(p + sz);
    s[5] = __ldg(p + sz + 1);
    s[6] = __ldg(p + sz + sy);
    s[7] = __ldg(p + sz + sy + 1);
    int cs = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) cs |= (s[i] >= iso ? 1 : 0) << i;
    cc.cs = cs;
    cc.nv = 0;
    cc.nq = 0;
    cc.c = 0;
    if (cs == 0 || cs == 255) return;
    cc.c = cellContours(cs, s, iso, table);
    cc.nv = numContours(cc.c);
    // quads owned: the three edges leaving corner 0 (local edges 0, 3, 8),
    // when all four cells around the edge exist
    cc.nq = ((((cs ^ (cs >> 1)) & 1) && y >= 1 && z >= 1) ? 1 : 0) +
            ((((cs ^ (cs >> 2)) & 1) && x >= 1 && z >= 1) ? 1 : 0) +
            ((((cs ^ (cs >> 4)) & 1) && x >= 1 && y >= 1) ? 1 : 0);
}

__device__ __forceinline__ void stageTable(uint64_t* sh) {
    for (int i = threadIdx.x; i < 256; i += blockDim.x) sh[i] = kContourTable[i];
    __syncthreads();
}

// per-row (active cells, vertices, owned quads)
__global__ void __launch_bounds__(256) kRowCount(GridView g, float iso, int4* __restrict__ rowCounts, int numRows) {
    __shared__ uint64_t table[256];
    stageTable(table);
    const int lane = threadIdx.x & 31;
    const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= numRows) return;
    const int y = row % (g.Y - 1), z = row / (g.Y - 1);
    int a = 0, v = 0, q = 0;
    for (int x0 = 0; x0 < g.X - 1; x0 += 32) {
        const int x = x0 + lane;
        if (x < g.X - 1) {
            float s[8];
            CellClass cc;
            classify(g, x, y, z, iso, table, s, cc);
            a += cc.nv > 0 ? 1 : 0;
            v += cc.nv;
            q += cc.nq;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        v += __shfl_down_sync(0xffffffffu, v, o);
        q += __shfl_down_sync(0xffffffffu, q, o);
    }
    if (lane == 0) rowCounts[row] = make_int4(a, v, q, 0);
}

void launchRowCount(const GridView& g, float iso, int4* rowCounts, int numRows, cudaStream_t s) {
    countLaunch();
    kRowCount<<<(numRows + 7) / 8, 256, 0, s>>>(g, iso, rowCounts, numRows);
}

// one active cell: vertices (sliceP, D/CellIntersection.inl:368-439) and record
__device__ void emitCell(const GridView& g, int x, int y, int z, float iso, bool surfaceIteration,
                         const float s[8], const CellClass& cc, int vbase, int qbase, ActiveCell* act, int aIdx,
                         float* __restrict__ pos, float* __restrict__ nrm) {
    F3 normals[8];
    cornerGradients(g, x, y, z, s, normals);
    const int n = cc.nv;
    uint32_t emap = 0;
    int before = 0;
    for (int t = 0; t < n; ++t) {
        const int sz = nib(cc.c, t);
        F3 p = f3(0.f, 0.f, 0.f);
        for (int i = 0; i < sz; ++i) {
            const int e = (int)((cc.c >> (16 + 4 * (before + i))) & 0xF);
            const int a0 = edgeV0(e), a1 = edgeV1(e);
            const float w = (iso - s[a0]) / (s[a1] - s[a0]);
            // computeLocalCoordinateOffset (:176-200): the edge's axis gets the
            // crossing, the other two axes corner a0's coordinate
            const int ax = edgeAxis(e);
            F3 off = f3(ax == 0 ? w : (float)(a0 & 1), ax == 1 ? w : (float)((a0 >> 1) & 1),
                        ax == 2 ? w : (float)((a0 >> 2) & 1));
            p = p + off;
            emap |= (uint32_t)t << (2 * e);
        }
        before += sz;
        p = p / (float)sz;
        if (surfaceIteration) {
            SurfaceIterator it{s, iso};
            it.move(p);
        }
        F3 nm = gnormalize(trilinear3(normals, p));
        F3 wp = g.origin() + (f3((float)x, (float)y, (float)z) + p) * g.deltas();
        const int64_t vi = (int64_t)vbase + t;
        pos[3 * vi] = wp.x;
        pos[3 * vi + 1] = wp.y;
        pos[3 * vi + 2] = wp.z;
        nrm[3 * vi] = nm.x;
        nrm[3 * vi + 1] = nm.y;
        nrm[3 * vi + 2] = nm.z;
    }
    ActiveCell rec;
    rec.cell = (uint32_t)(((size_t)z * g.Y + y) * g.X + x);
    rec.vbase = vbase;
    rec.qbase = qbase;
    rec.info = (uint32_t)cc.cs | (emap << 8);
    act[aIdx] = rec;
}

__global__ void __launch_bounds__(256) kRowEmit(GridView g, float iso, int surfaceIteration,
                                                const int4* __restrict__ rowOffsets, int numRows,
                                                ActiveCell* __restrict__ act, float* __restrict__ pos,
                                                float* __restrict__ nrm, int numActive, int numVertices,
                                                uint32_t* status) {
    __shared__ uint64_t table[256];
    stageTable(table);
    const int lane = threadIdx.x & 31;
    const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= numRows) return;
    const int y = row % (g.Y - 1), z = row / (g.Y - 1);
    const int4 base = rowOffsets[row];
    int aRun = base.x, vRun = base.y, qRun = base.z;
    const unsigned ltMask = (1u << lane) - 1u;
    for (int x0 = 0; x0 < g.X - 1; x0 += 32) {
        const int x = x0 + lane;
        float s[8];
        CellClass cc;
        cc.nv = 0;
        cc.nq = 0;
        if (x < g.X - 1) classify(g, x, y, z, iso, table, s, cc);
        const bool active = cc.nv > 0;
        const unsigned ballot = __ballot_sync(0xffffffffu, active);
        int vInc = cc.nv, qInc = cc.nq;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int u = __shfl_up_sync(0xffffffffu, vInc, o);
            int w = __shfl_up_sync(0xffffffffu, qInc, o);
            if (lane >= o) { vInc += u; qInc += w; }
        }
        const int vTot = __shfl_sync(0xffffffffu, vInc, 31);
        const int qTot = __shfl_sync(0xffffffffu, qInc, 31);
        if (active) {
            const int aIdx = aRun + __popc(ballot & ltMask), vIdx = vRun + vInc - cc.nv;
            // the counts of the first pass bound every write of this one
            if (aIdx < numActive && vIdx + cc.nv <= numVertices)
                emitCell(g, x, y, z, iso, surfaceIteration != 0, s, cc, vIdx, qRun + qInc - cc.nq, act, aIdx, pos, nrm);
            else
                atomicOr(status, kStatusCountMismatch);
        }
        aRun += __popc(ballot);
        vRun += vTot;
        qRun += qTot;
    }
}

void launchRowEmit(const GridView& g, float iso, int surfaceIteration, const int4* rowOffsets, int numRows,
                   ActiveCell* act, float* pos, float* nrm, int numActive, int numVertices, uint32_t* status,
                   cudaStream_t s) {
    countLaunch();
    kRowEmit<<<(numRows + 7) / 8, 256, 0, s>>>(g, iso, surfaceIteration, rowOffsets, numRows, act, pos, nrm, numActive,
                                                numVertices, status);
}

// ---------------------------------------------------------------------------
// quads, halfedges and edge-table inserts
// ---------------------------------------------------------------------------
__device__ __forceinline__ int findActive(const ActiveCell* __restrict__ act, const int4* __restrict__ rowOffsets,
                                          int row, uint32_t cell) {
    int lo = rowOffsets[row].x, hi = rowOffsets[row + 1].x;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        uint32_t c = act[mid].cell;
        if (c < cell) lo = mid + 1;
        else hi = mid;
    }
    if (lo < rowOffsets[row + 1].x && act[lo].cell == cell) return lo;
    return -1;
}

// The four cells around the grid edge leaving cell (x,y,z)'s corner 0 along
// `axis`, each with the local index of that edge inside the cell.  The slot
// each contributes follows from the edge index and its orientation
// (computeVertexPosition, D/CellIntersection.inl:361-366).
__device__ __forceinline__ void cellsAroundEdge(int axis, int d[4][3], int e[4]) {
    // axis 0: cells p, p-y, p-z, p-y-z with local edges 0, 2, 4, 6
    // axis 1: cells p, p-x, p-z, p-x-z with local edges 3, 1, 7, 5
    // axis 2: cells p, p-x, p-y, p-x-y with local edges 8, 9, 11, 10
    const int b = axis == 0 ? 1 : 0;  // first other axis
    const int c = axis == 2 ? 1 : 2;  // second other axis
    const int le[3][4] = {{0, 2, 4, 6}, {3, 1, 7, 5}, {8, 9, 11, 10}};
    for (int k = 0; k < 4; ++k) {
        d[k][0] = d[k][1] = d[k][2] = 0;
        if (k & 1) d[k][b] = -1;
        if (k & 2) d[k][c] = -1;
        e[k] = le[axis][k];
    }
}

__global__ void kQuads(const ActiveCell* __restrict__ act, int numActive, const int4* __restrict__ rowOffsets, int X,
                       int Y, Bucket* __restrict__ table, unsigned long long cap, int4* __restrict__ he,
                       int* __restrict__ faceFirst, uint16_t* __restrict__ faceAttr, int numQuads, int numVertices,
                       uint32_t* status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= numActive) return;
    const ActiveCell rec = act[i];
    const int cs = (int)(rec.info & 255u);
    const int x = (int)(rec.cell % (uint32_t)X);
    const int y = (int)((rec.cell / (uint32_t)X) % (uint32_t)Y);
    const int z = (int)(rec.cell / ((uint32_t)X * (uint32_t)Y));
    int qi = rec.qbase;
    for (int axis = 0; axis < 3; ++axis) {
        // edges 0, 3, 8 run from corner 0 to corners 1, 2, 4
        if (!((cs ^ (cs >> (1 << axis))) & 1)) continue;
        if (axis == 0 && !(y >= 1 && z >= 1)) continue;
        if (axis == 1 && !(x >= 1 && z >= 1)) continue;
        if (axis == 2 && !(x >= 1 && y >= 1)) continue;
        int d[4][3], le[4];
        cellsAroundEdge(axis, d, le);
        int quad[4] = {-1, -1, -1, -1};
        for (int k = 0; k < 4; ++k) {
            ActiveCell r2 = rec;
            if (k > 0) {
                const int cx = x + d[k][0], cy = y + d[k][1], cz = z + d[k][2];
                const uint32_t cell = (uint32_t)(((size_t)cz * Y + cy) * X + cx);
                const int j = findActive(act, rowOffsets, cz * (Y - 1) + cy, cell);
                if (j < 0) {
                    atomicOr(status, kStatusMissingCell);
                    continue;
                }
                r2 = act[j];
            }
            const int e = le[k];
            const int t = (int)((r2.info >> (8 + 2 * e)) & 3u);
            const int edgy = ((r2.info >> edgeV0(e)) & 1u) ? 0 : 1;  // s[v0] < iso
            const int slot = quadSlot(e, edgy);
            if (quad[slot] != -1) atomicOr(status, kStatusSlotConflict);
            quad[slot] = r2.vbase + t;
        }
        if (qi >= numQuads || quad[0] < 0 || quad[1] < 0 || quad[2] < 0 || quad[3] < 0 || quad[0] >= numVertices ||
            quad[1] >= numVertices || quad[2] >= numVertices || quad[3] >= numVertices) {
            atomicOr(status, kStatusCountMismatch);
            return;
        }
        const int h0 = 4 * qi;
#pragma unroll
        for (int k = 0; k < 4; ++k) he[h0 + k] = make_int4(quad[k], qi, h0 + ((k + 1) & 3), -1);
        faceFirst[qi] = h0;
        const int baseColor = (x & 1) | ((y & 1) << 1) | ((z & 1) << 2);
        faceAttr[qi] = (uint16_t)(3 * baseColor + axis);
#pragma unroll
        for (int k = 0; k < 4; ++k) edgeInsert(table, cap, quad[k], quad[(k + 1) & 3], h0 + k, status);
        ++qi;
    }
}

void launchQuads(const ActiveCell* act, int numActive, const int4* rowOffsets, int X, int Y, Bucket* table,
                 unsigned long long cap, int4* he, int* faceFirst, uint16_t* faceAttr, int numQuads, int numVertices,
                 uint32_t* status, cudaStream_t s) {
    if (numActive <= 0) return;
    countLaunch();
    kQuads<<<(numActive + 255) / 256, 256, 0, s>>>(act, numActive, rowOffsets, X, Y, table, cap, he, faceFirst,
                                                   faceAttr, numQuads, numVertices, status);
}

}  // namespace mdmc
