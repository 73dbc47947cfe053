// Standard Marching Cubes (the older CLI version's standard_mc,
// O/DualMarchingCubes.cu:201-307, and map_triangles, :316-328): one vertex
// per intersected grid edge, triangles from the case table.
//
// The reference deduplicates edge vertices through a hash table and numbers
// vertices and triangles in atomic order.  Here the active cells of the DMC
// front end mark their intersected edges in a bit mask laid out like the
// global edge ids (3 * sample + axis, one row of words per (y, z) sample
// row); a popcount scan of that mask numbers the vertices in edge-id order,
// and a scan of the cells' triangle counts numbers the triangles in cell
// order, so the mesh is the same on every run and equals the oracle's.
#include <cuda_runtime.h>

#include "mc_triangle_table.h"
#include "mdmc.h"
#include "mdmc_kernels.h"

namespace mdmc {
namespace {

// cell edge e runs from corner kMCEdgeV0[e] along axis kMCEdgeAxis[e]
// (corner bit 0 = +x, bit 1 = +y, bit 2 = +z)
__constant__ int kMCEdgeV0[12] = {0, 1, 2, 0, 4, 5, 6, 4, 0, 1, 3, 2};
__constant__ int kMCEdgeAxis[12] = {0, 1, 0, 1, 0, 1, 0, 1, 2, 2, 2, 2};

// mask word and bit of the edge (x, y, z, axis)
__device__ __forceinline__ int64_t edgeWord(int x, int y, int z, int axis, int Y, int W3, uint32_t& bit) {
    const int b = 3 * x + axis;
    bit = 1u << (b & 31);
    return ((int64_t)z * Y + y) * W3 + (b >> 5);
}

__device__ __forceinline__ void cellOf(uint32_t cell, int X, int Y, int& x, int& y, int& z) {
    const uint32_t line = cell / (uint32_t)X;
    x = (int)(cell - line * (uint32_t)X);
    y = (int)(line % (uint32_t)Y);
    z = (int)(line / (uint32_t)Y);
}

// central difference with clamped neighbours (UniformGrid::gradient,
// O/UniformGrid.h:279-321, one corner's entry)
template <class View>
__device__ __forceinline__ F3 pointGradient(const View& g, int x, int y, int z) {
    F3 n;
    n.x = 0.5f * (atClamped(g, x + 1, y, z) - atClamped(g, x - 1, y, z)) / g.dx;
    n.y = 0.5f * (atClamped(g, x, y + 1, z) - atClamped(g, x, y - 1, z)) / g.dy;
    n.z = 0.5f * (atClamped(g, x, y, z + 1) - atClamped(g, x, y, z - 1)) / g.dz;
    return n;
}

// per active cell: its case, its triangle count, and its intersected edges
// or-ed into the edge mask
template <class View>
__global__ void __launch_bounds__(128) kMCMarkEdges(View g, float iso, const uint32_t* __restrict__ cellIds, int numActive,
                                                    int W3, uint32_t* __restrict__ edgeMask, uint8_t* __restrict__ cases,
                                                    int* __restrict__ triCount, uint32_t* status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= numActive) return;
    int x, y, z;
    cellOf(cellIds[i], g.X, g.Y, x, y, z);
    if (x >= g.X - 1 || y >= g.Y - 1 || z >= g.Z - 1) {
        atomicOr(status, kStatusCountMismatch);
        triCount[i] = 0;
        cases[i] = 0;
        return;
    }
    float u[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) u[k] = g.at(x + (k & 1), y + ((k >> 1) & 1), z + ((k >> 2) & 1));
    int cs = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) cs |= (u[k] >= iso ? 1 : 0) << k;
    cases[i] = (uint8_t)cs;
    triCount[i] = (int)(kTriangleTable[cs] & 0xF);
    if (cs == 0 || cs == 255) {
        atomicOr(status, kStatusCountMismatch);
        return;
    }
#pragma unroll
    for (int e = 0; e < 12; ++e) {
        const int a0 = kMCEdgeV0[e], axis = kMCEdgeAxis[e];
        const int a1 = a0 | (1 << axis);
        if (((cs >> a0) & 1) == ((cs >> a1) & 1)) continue;
        uint32_t bit;
        const int64_t w = edgeWord(x + (a0 & 1), y + ((a0 >> 1) & 1), z + ((a0 >> 2) & 1), axis, g.Y, W3, bit);
        atomicOr(edgeMask + w, bit);
    }
}

// global edge id of every vertex, in edge-id order
__global__ void kMCScatterEdges(const uint32_t* __restrict__ edgeMask, const int* __restrict__ first, int64_t numWords,
                                int W3, int X, uint32_t* __restrict__ edgeIds, int numVertices, uint32_t* status) {
    const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= numWords) return;
    uint32_t m = edgeMask[w];
    if (!m) return;
    const int64_t row = (uint32_t)w / (uint32_t)W3;  // fewer than 2^32 words
    const int b0 = (int)(w - row * W3) * 32;
    int j = first[w];
    while (m) {
        const int b = b0 + __ffs(m) - 1;
        m &= m - 1;
        if (inb(j, numVertices)) edgeIds[j] = (uint32_t)(3 * (row * X + b / 3) + b % 3);
        else atomicOr(status, kStatusCountMismatch);
        ++j;
    }
}

// one vertex per intersected edge: the linear crossing from the edge's low
// end, and the interpolated corner gradients over their length
template <class View>
__global__ void __launch_bounds__(128) kMCVertices(View g, float iso, const uint32_t* __restrict__ edgeIds,
                                                   int numVertices, float* __restrict__ pos, float* __restrict__ nrm) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= numVertices) return;
    const uint32_t id = edgeIds[j];
    const int axis = (int)(id % 3u);
    int x, y, z;
    cellOf(id / 3u, g.X, g.Y, x, y, z);
    const int x1 = x + (axis == 0), y1 = y + (axis == 1), z1 = z + (axis == 2);
    const float u0 = g.at(x, y, z), u1 = g.at(x1, y1, z1);
    const float l = (iso - u0) / (u1 - u0);
    const float p0x = g.ox + (float)x * g.dx, p0y = g.oy + (float)y * g.dy, p0z = g.oz + (float)z * g.dz;
    const float p1x = g.ox + (float)x1 * g.dx, p1y = g.oy + (float)y1 * g.dy, p1z = g.oz + (float)z1 * g.dz;
    const F3 n0 = pointGradient(g, x, y, z), n1 = pointGradient(g, x1, y1, z1);
    float nx = n0.x + l * (n1.x - n0.x), ny = n0.y + l * (n1.y - n0.y), nz = n0.z + l * (n1.z - n0.z);
    const float f = sqrtf(nx * nx + ny * ny + nz * nz);
    nx /= f;
    ny /= f;
    nz /= f;
    pos[3 * (int64_t)j + 0] = p0x + l * (p1x - p0x);
    pos[3 * (int64_t)j + 1] = p0y + l * (p1y - p0y);
    pos[3 * (int64_t)j + 2] = p0z + l * (p1z - p0z);
    nrm[3 * (int64_t)j + 0] = nx;
    nrm[3 * (int64_t)j + 1] = ny;
    nrm[3 * (int64_t)j + 2] = nz;
}

// triangles of every active cell, at the cell's offset, vertex ids from the
// edge mask's rank
__global__ void __launch_bounds__(128) kMCTriangles(const uint32_t* __restrict__ cellIds, const uint8_t* __restrict__ cases,
                                                    const int* __restrict__ triOffset, int numActive, int X, int Y, int W3,
                                                    const uint32_t* __restrict__ edgeMask, const int* __restrict__ edgeFirst,
                                                    int64_t numWords, int* __restrict__ tris, int numTriangles,
                                                    uint32_t* status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= numActive) return;
    int x, y, z;
    cellOf(cellIds[i], X, Y, x, y, z);
    const unsigned long long w = kTriangleTable[cases[i]];
    const int n = (int)(w & 0xF);
    const int t0 = triOffset[i];
    if (!inb(t0, (int64_t)numTriangles - n + 1)) {
        if (n) atomicOr(status, kStatusCountMismatch);
        return;
    }
    for (int k = 0; k < 3 * n; ++k) {
        const int e = (int)((w >> (4 + 4 * k)) & 0xF);
        const int a0 = kMCEdgeV0[e];
        uint32_t bit;
        const int64_t word = edgeWord(x + (a0 & 1), y + ((a0 >> 1) & 1), z + ((a0 >> 2) & 1), kMCEdgeAxis[e], Y, W3, bit);
        int v = -1;
        if (inb(word, numWords)) {
            const uint32_t m = edgeMask[word];
            if (m & bit) v = edgeFirst[word] + __popc(m & (bit - 1));
        }
        if (v < 0) atomicOr(status, kStatusBadIndex);
        tris[3 * (int64_t)t0 + k] = v;
    }
}

}  // namespace

void launchMCMarkEdges(const GridDesc& g, float iso, const uint32_t* cellIds, int numActive, int W3, uint32_t* edgeMask,
                       uint8_t* cases, int* triCount, uint32_t* status, cudaStream_t s) {
    if (numActive <= 0) return;
    countLaunch();
    const unsigned blocks = (unsigned)((numActive + 127) / 128);
    if (g.refined)
        kMCMarkEdges<RefinedView><<<blocks, 128, 0, s>>>(g.ref, iso, cellIds, numActive, W3, edgeMask, cases, triCount,
                                                         status);
    else
        kMCMarkEdges<PlainView><<<blocks, 128, 0, s>>>(g.plain, iso, cellIds, numActive, W3, edgeMask, cases, triCount,
                                                       status);
}

void launchMCScatterEdges(const uint32_t* edgeMask, const int* first, int64_t numWords, int W3, int X, uint32_t* edgeIds,
                          int numVertices, uint32_t* status, cudaStream_t s) {
    if (numWords <= 0) return;
    countLaunch();
    kMCScatterEdges<<<(unsigned)((numWords + 255) / 256), 256, 0, s>>>(edgeMask, first, numWords, W3, X, edgeIds,
                                                                       numVertices, status);
}

void launchMCVertices(const GridDesc& g, float iso, const uint32_t* edgeIds, int numVertices, float* pos, float* nrm,
                      cudaStream_t s) {
    if (numVertices <= 0) return;
    countLaunch();
    const unsigned blocks = (unsigned)((numVertices + 127) / 128);
    if (g.refined)
        kMCVertices<RefinedView><<<blocks, 128, 0, s>>>(g.ref, iso, edgeIds, numVertices, pos, nrm);
    else
        kMCVertices<PlainView><<<blocks, 128, 0, s>>>(g.plain, iso, edgeIds, numVertices, pos, nrm);
}

void launchMCTriangles(const uint32_t* cellIds, const uint8_t* cases, const int* triOffset, int numActive, int X, int Y,
                       int W3, const uint32_t* edgeMask, const int* edgeFirst, int64_t numWords, int* tris,
                       int numTriangles, uint32_t* status, cudaStream_t s) {
    if (numActive <= 0) return;
    countLaunch();
    kMCTriangles<<<(unsigned)((numActive + 127) / 128), 128, 0, s>>>(cellIds, cases, triOffset, numActive, X, Y, W3,
                                                                     edgeMask, edgeFirst, numWords, tris, numTriangles,
                                                                     status);
}

}  // namespace mdmc
