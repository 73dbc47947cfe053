// Consumers of the finished mesh from the older CLI version:
//  * face coloring, FaceColoring::colorFaces (O/FaceColoring.cu:5-141): the
//    24 colors the DMC inherits from its grid-edge coloring are reduced to 5
//    (0-4): classes 5..23 in turn, each face taking the first of 0..4 that
//    none of its edge neighbours (faces of its halfedges' twins) holds, then
//    the faces of color 4 trying 0..3 once more;
//  * quadrilateral_to_triangle (O/DualMarchingCubes.cu:51-60): quad
//    (v0, v1, v2, v3) -> triangles (v0, v1, v3), (v3, v2, v0);
//  * mean_ratio_measure / QualityMeasure::mean_ratio (O/DualMarchingCubes.cu:
//    93-107, O/QualityMeasure.h:45-66): 2 sqrt(3) |cross| / sum of squared
//    edge lengths per triangle (1 for an equilateral triangle, 0 for a
//    degenerate one).
//
// Coloring order: the reference colors the faces of one class concurrently,
// reading its neighbours' live colors.  Two faces of one class are never
// neighbours while the grid-edge coloring is proper; where they are (after
// the manifold repair), a face here sees a same-class neighbour with the
// color that neighbour had before the class's pass, so the result does not
// depend on thread timing.  The same holds for the color-4 pass.  Only the
// color bits (0-4) of the face attributes change.
#include <cuda_runtime.h>

#include "mdmc.h"
#include "mdmc_kernels.h"

namespace mdmc {
namespace {

// first color of 0..4 that none of n0..n3 holds, the color-4 test with the
// reference's c2-twice comparison (FaceColoring.cu:63); -1 if none is free
__device__ __forceinline__ int firstFreeColor(int c0, int c1, int c2, int c3, int last) {
    for (int k = 0; k < 4 && k <= last; ++k)
        if (c0 != k && c1 != k && c2 != k && c3 != k) return k;
    if (last >= 4 && c0 != 4 && c1 != 4 && c2 != 4) return 4;
    return -1;
}

// colors of the faces across the four edges of face f (-1 across a boundary),
// read from cur except for faces whose class is the one being recolored
__device__ __forceinline__ void neighbourColors(const int4* __restrict__ he, const int* __restrict__ faceFirst,
                                                const uint8_t* __restrict__ orig, const uint16_t* __restrict__ attr,
                                                int f, int cls, int numFaces, int numHalfedges, int nc[4]) {
    int e = faceFirst[f];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        nc[k] = -1;
        if (!inb(e, numHalfedges)) continue;
        const int4 h = he[e];
        if (h.w > -1 && inb(h.w, numHalfedges)) {
            const int g = he[h.w].y;
            if (inb(g, numFaces)) nc[k] = orig[g] == cls ? cls : (int)(attr[g] & 0x1F);
        }
        e = h.z;
    }
}

__global__ void kSaveColors(const uint16_t* __restrict__ attr, int numFaces, uint8_t* __restrict__ orig) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f < numFaces) orig[f] = (uint8_t)(attr[f] & 0x1F);
}

// recolor the faces of class cls (5..23) from 0..4
__global__ void kColorClass(const int4* __restrict__ he, const int* __restrict__ faceFirst, const uint8_t* __restrict__ orig,
                            uint16_t* __restrict__ attr, int numFaces, int numHalfedges, int cls) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= numFaces || orig[f] != cls) return;
    int nc[4];
    neighbourColors(he, faceFirst, orig, attr, f, cls, numFaces, numHalfedges, nc);
    const int c = firstFreeColor(nc[0], nc[1], nc[2], nc[3], 4);
    if (c >= 0) attr[f] = (uint16_t)((attr[f] & ~0x1F) | c);
}

// faces of color 4 try 0..3 (optimize_face_coloring, FaceColoring.cu:67-116);
// the faces of color 4 before this pass are marked 4 in orig
__global__ void kMarkColor4(const uint16_t* __restrict__ attr, int numFaces, uint8_t* __restrict__ orig) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f < numFaces) orig[f] = (attr[f] & 0x1F) == 4 ? 4 : 0xFF;
}

__global__ void kRecolor4(const int4* __restrict__ he, const int* __restrict__ faceFirst, const uint8_t* __restrict__ orig,
                          uint16_t* __restrict__ attr, int numFaces, int numHalfedges) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= numFaces || orig[f] != 4) return;
    int nc[4];
    neighbourColors(he, faceFirst, orig, attr, f, 4, numFaces, numHalfedges, nc);
    const int c = firstFreeColor(nc[0], nc[1], nc[2], nc[3], 3);
    if (c >= 0) attr[f] = (uint16_t)((attr[f] & ~0x1F) | c);
}

__global__ void kQuadsToTriangles(const int4* __restrict__ quads, int64_t numQuads, int* __restrict__ tris) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= numQuads) return;
    const int4 v = quads[q];
    int* t = tris + 6 * q;
    t[0] = v.x;
    t[1] = v.y;
    t[2] = v.w;
    t[3] = v.w;
    t[4] = v.z;
    t[5] = v.x;
}

__global__ void kMeanRatio(const float* __restrict__ pos, const int* __restrict__ tris, int64_t numTriangles,
                           int64_t numVertices, float* __restrict__ q, uint32_t* __restrict__ bad) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= numTriangles) return;
    const int i0 = tris[3 * t], i1 = tris[3 * t + 1], i2 = tris[3 * t + 2];
    if (!inb(i0, numVertices) || !inb(i1, numVertices) || !inb(i2, numVertices)) {
        q[t] = __int_as_float(0x7fc00000);
        if (bad) atomicOr(bad, 1u);
        return;
    }
    const float ax = pos[3 * (int64_t)i0], ay = pos[3 * (int64_t)i0 + 1], az = pos[3 * (int64_t)i0 + 2];
    const float bx = pos[3 * (int64_t)i1], by = pos[3 * (int64_t)i1 + 1], bz = pos[3 * (int64_t)i1 + 2];
    const float cx = pos[3 * (int64_t)i2], cy = pos[3 * (int64_t)i2 + 1], cz = pos[3 * (int64_t)i2 + 2];
    const float l0 = (bx - ax) * (bx - ax) + (by - ay) * (by - ay) + (bz - az) * (bz - az);
    const float l1 = (cx - bx) * (cx - bx) + (cy - by) * (cy - by) + (cz - bz) * (cz - bz);
    const float l2 = (ax - cx) * (ax - cx) + (ay - cy) * (ay - cy) + (az - cz) * (az - cz);
    const float l = l0 + l1 + l2;
    const float x1 = bx - ax, x2 = cx - ax, y1 = by - ay, y2 = cy - ay, z1 = bz - az, z2 = cz - az;
    const float a1 = (y1 * z2 - z1 * y2) * (y1 * z2 - z1 * y2);
    const float a2 = (x1 * z2 - z1 * x2) * (x1 * z2 - z1 * x2);
    const float a3 = (x1 * y2 - y1 * x2) * (x1 * y2 - y1 * x2);
    const float a = sqrtf(a1 + a2 + a3);
    q[t] = 2.0f * sqrtf(3.0f) * a / l;
}

}  // namespace

void launchColorFaces(const int4* he, const int* faceFirst, uint16_t* attr, uint8_t* orig, int numFaces, int numHalfedges,
                      cudaStream_t s) {
    if (numFaces <= 0) return;
    const unsigned blocks = (unsigned)((numFaces + 255) / 256);
    countLaunch(2 + 19 + 1);
    kSaveColors<<<blocks, 256, 0, s>>>(attr, numFaces, orig);
    for (int cls = 5; cls < 24; ++cls)
        kColorClass<<<blocks, 256, 0, s>>>(he, faceFirst, orig, attr, numFaces, numHalfedges, cls);
    kMarkColor4<<<blocks, 256, 0, s>>>(attr, numFaces, orig);
    kRecolor4<<<blocks, 256, 0, s>>>(he, faceFirst, orig, attr, numFaces, numHalfedges);
}

}  // namespace mdmc

using namespace mdmc;

extern "C" MDMC_API mdmc_status mdmc_quads_to_triangles(const int32_t* quads, int64_t num_quads, int32_t* triangles,
                                                         void* stream) {
    if (num_quads < 0 || (num_quads > 0 && (!quads || !triangles))) return MDMC_ERROR_INVALID_ARGUMENT;
    if (num_quads == 0) return MDMC_OK;
    countLaunch();
    kQuadsToTriangles<<<(unsigned)((num_quads + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const int4*>(quads), num_quads, triangles);
    return cudaGetLastError() == cudaSuccess ? MDMC_OK : MDMC_ERROR_CUDA;
}

extern "C" MDMC_API mdmc_status mdmc_mean_ratio(const float* positions, int64_t num_vertices, const int32_t* triangles,
                                                int64_t num_triangles, float* quality, uint32_t* bad_index,
                                                void* stream) {
    if (num_triangles < 0 || num_vertices < 0 || (num_triangles > 0 && (!positions || !triangles || !quality)))
        return MDMC_ERROR_INVALID_ARGUMENT;
    if (num_triangles == 0) return MDMC_OK;
    countLaunch();
    kMeanRatio<<<(unsigned)((num_triangles + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        positions, triangles, num_triangles, num_vertices, quality, bad_index);
    return cudaGetLastError() == cudaSuccess ? MDMC_OK : MDMC_ERROR_CUDA;
}
