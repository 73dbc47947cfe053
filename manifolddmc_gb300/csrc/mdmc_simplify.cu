// Valence-pattern simplifications, run right after the halfedge mesh is
// built: simplify3X3Y (colour based), simplify3X3YOld and simplify3333
// (D/Halfedges/HalfedgeMesh.cu:296-683, host sequences :859-1048), each
// ending in a rebuild of the halfedge mesh from the reduced vertex and quad
// lists.  Where the reference is not deterministic or reads outside its
// arrays, the oracle's fixed behaviour is followed: a quad edge without a twin
// makes the quad ineligible (the reference reads halfedges[-1]); vertices and
// quads are compacted in order (the reference appends with atomics); in the
// 3333 pass every face's pattern bits are cleared before any face marks a
// neighbour for removal (the reference's threads race there).  Concurrent
// merges on one vertex (possible only in degenerate configurations) resolve
// to the largest face id, the oracle's sequential order.
#include <cuda_runtime.h>

#include "mdmc_device.cuh"
#include "mdmc_kernels.h"

namespace mdmc {
namespace {

constexpr uint32_t kAttrPattern = 0x40, kAttrRemove = 0x80, kAttrBoundary = 0x100;
constexpr int kTypeRemovable = 3, kTypePattern = 1;

__device__ __forceinline__ uint32_t attrOf(const uint16_t* a, int f) {
    return (uint32_t)(*(volatile const uint16_t*)(a + f));
}
__device__ __forceinline__ void andFaceAttr(uint16_t* attr, int f, uint32_t keep) {
    const uint32_t mask = (f & 1) ? ((keep << 16) | 0xFFFFu) : (keep | 0xFFFF0000u);
    atomicAnd(reinterpret_cast<uint32_t*>(attr) + (f >> 1), mask);
}

// the four halfedges and vertices of face f
__device__ __forceinline__ bool faceRing(const int4* he, const int* faceFirst, int f, MeshDims md, int hs[4], int q[4]) {
    int h = faceFirst[f];
    for (int i = 0; i < 4; ++i) {
        if (!inb(h, md.H)) return false;
        const int4 e = he[h];
        if (!inb(e.x, md.V)) return false;
        hs[i] = h;
        q[i] = e.x;
        h = e.z;
    }
    return true;
}

// computeVertexValence, :296-312
__global__ void kValence(const int4* __restrict__ he, MeshDims md, int* __restrict__ val) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= md.H) return;
    const int4 e = he[h];
    if (inb(e.x, md.V)) atomicAdd(&val[e.x], 1);
    if (e.w == -1 && inb(e.z, md.H)) {
        const int n = he[e.z].x;
        if (inb(n, md.V)) atomicAdd(&val[n], 1);
    }
}

__device__ __forceinline__ bool patternA(const int* val, const int q[4]) {
    return val[q[0]] == 3 && val[q[1]] >= 5 && val[q[2]] == 3 && val[q[3]] >= 5;
}
__device__ __forceinline__ bool patternB(const int* val, const int q[4]) {
    return val[q[0]] >= 5 && val[q[1]] == 3 && val[q[2]] >= 5 && val[q[3]] == 3;
}

// markElementsP3X3Y (:318-340) / countVerticesP3X3Y (:342-364)
__global__ void kMark3X3Y(const int4* __restrict__ he, const int* __restrict__ faceFirst, MeshDims md,
                          const int* __restrict__ val, int color, uint16_t* attr, int* count, uint32_t* status) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= md.F) return;
    int hs[4], q[4];
    if (!faceRing(he, faceFirst, f, md, hs, q)) {
        atomicOr(status, kStatusBadIndex);
        return;
    }
    const uint32_t a = attrOf(attr, f);
    if (color) {
        if (a & (MDMC_FACE_NON_MANIFOLD | kAttrBoundary)) return;
        andFaceAttr(attr, f, 0x3Fu | 0xFF00u);
        if (patternA(val, q) || patternB(val, q)) orFaceAttr(attr, f, kAttrPattern);
    } else {
        andFaceAttr(attr, f, 0x3Fu | 0xFF00u);
        if (patternA(val, q)) {
            atomicAdd(&count[q[0]], 1);
            atomicAdd(&count[q[2]], 1);
            orFaceAttr(attr, f, kAttrPattern);
        } else if (patternB(val, q)) {
            atomicAdd(&count[q[1]], 1);
            atomicAdd(&count[q[3]], 1);
            orFaceAttr(attr, f, kAttrPattern);
        }
    }
}

// mergeVerticesP3X3YColor (:381-442) / mergeVerticesP3X3Y (:448-496): the
// decision (vertices a, b, c, d of handleMerge packed into `merge`, -1 none)
// and a claim on a and c by the largest face id
__global__ void kDecide3X3Y(const int4* __restrict__ he, const int* __restrict__ faceFirst, MeshDims md,
                            const int* __restrict__ val, const int* __restrict__ count, int color,
                            const uint16_t* attr, int4* __restrict__ merge, int* claimA, int* claimC) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= md.F) return;
    merge[f] = make_int4(-1, -1, -1, -1);
    const uint32_t a = attrOf(attr, f);
    if (!color && (a & (MDMC_FACE_NON_MANIFOLD | kAttrBoundary))) return;
    if (!(a & kAttrPattern)) return;
    int hs[4], q[4];
    if (!faceRing(he, faceFirst, f, md, hs, q)) return;
    int nb[4];
    for (int i = 0; i < 4; ++i) {
        const int t = he[hs[i]].w;
        if (!inb(t, md.H)) return;
        nb[i] = he[t].y;
        if (!inb(nb[i], md.F)) return;
        // the reference tests the neighbour's NM flag and the quad's own boundary flag
        if ((attrOf(attr, nb[i]) & MDMC_FACE_NON_MANIFOLD) || (a & kAttrBoundary)) return;
    }
    if (color) {
        const uint32_t c = a & 0x1Fu;
        for (int i = 0; i < 4; ++i) {
            const uint32_t na = attrOf(attr, nb[i]);
            if ((na & kAttrPattern) && (na & 0x1Fu) <= c) return;
        }
    }
    int4 m = make_int4(-1, -1, -1, -1);
    if (patternA(val, q) && (color || (count[q[0]] == 1 && count[q[2]] == 1))) m = make_int4(q[0], q[1], q[2], q[3]);
    else if (patternB(val, q) && (color || (count[q[1]] == 1 && count[q[3]] == 1))) m = make_int4(q[1], q[0], q[3], q[2]);
    if (m.x < 0) return;
    merge[f] = m;
    atomicMax(&claimA[m.x], f);
    atomicMax(&claimC[m.z], f);
}

// handleMerge, :358-378
__global__ void kApply3X3Y(MeshDims md, const int4* __restrict__ merge, const int* __restrict__ claimA,
                           const int* __restrict__ claimC, float* pos, float* nrm, uint16_t* attr, int* type,
                           int* target) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= md.F) return;
    const int4 m = merge[f];
    if (m.x < 0) return;
    if (claimA[m.x] == f) {
        const F3 pb = f3(pos[3 * (int64_t)m.y], pos[3 * (int64_t)m.y + 1], pos[3 * (int64_t)m.y + 2]);
        const F3 pd = f3(pos[3 * (int64_t)m.w], pos[3 * (int64_t)m.w + 1], pos[3 * (int64_t)m.w + 2]);
        const F3 nb = f3(nrm[3 * (int64_t)m.y], nrm[3 * (int64_t)m.y + 1], nrm[3 * (int64_t)m.y + 2]);
        const F3 nd = f3(nrm[3 * (int64_t)m.w], nrm[3 * (int64_t)m.w + 1], nrm[3 * (int64_t)m.w + 2]);
        const F3 p = pb + 0.5f * (pd - pb);
        const F3 n = gnormalize(nb + 0.5f * (nd - nb));
        pos[3 * (int64_t)m.x] = p.x;
        pos[3 * (int64_t)m.x + 1] = p.y;
        pos[3 * (int64_t)m.x + 2] = p.z;
        nrm[3 * (int64_t)m.x] = n.x;
        nrm[3 * (int64_t)m.x + 1] = n.y;
        nrm[3 * (int64_t)m.x + 2] = n.z;
    }
    if (claimC[m.z] == f) {
        type[m.z] = kTypeRemovable;
        target[m.z] = m.x;
    }
    orFaceAttr(attr, f, kAttrRemove);
}

// markElementsP3333 (:544-625), after every face's pattern bits were cleared
__global__ void kClear3333(MeshDims md, uint16_t* attr) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= md.F) return;
    if (!(attrOf(attr, f) & (MDMC_FACE_NON_MANIFOLD | kAttrBoundary))) andFaceAttr(attr, f, 0x3Fu | 0xFF00u);
}

__global__ void kMark3333(const int4* __restrict__ he, const int* __restrict__ faceFirst, MeshDims md,
                          const int* __restrict__ val, uint16_t* attr, int* type, int* target) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= md.F) return;
    if (attrOf(attr, f) & (MDMC_FACE_NON_MANIFOLD | kAttrBoundary)) return;
    int hs[4], q[4];
    if (!faceRing(he, faceFirst, f, md, hs, q)) return;
    for (int i = 0; i < 4; ++i)
        if (val[q[i]] != 3) return;
    int nb[4], nv[4], nval[4];
    for (int i = 0; i < 4; ++i) {
        const int t = he[hs[i]].w;
        if (!inb(t, md.H)) return;
        nb[i] = he[t].y;
        if (!inb(nb[i], md.F)) return;
        if (attrOf(attr, nb[i]) & (MDMC_FACE_NON_MANIFOLD | kAttrBoundary)) return;
        const int n1 = he[t].z;
        if (!inb(n1, md.H)) return;
        const int n2 = he[n1].z;
        if (!inb(n2, md.H)) return;
        nv[i] = he[n2].x;
        if (!inb(nv[i], md.V)) return;
        nval[i] = val[nv[i]];
        if (nval[i] == 3) return;
    }
    if (nval[0] == 4 && nval[1] == 4 && nval[2] == 4 && nval[3] == 4) return;
    orFaceAttr(attr, f, kAttrPattern);
    for (int i = 0; i < 4; ++i) {
        orFaceAttr(attr, nb[i], kAttrRemove);
        type[q[i]] = kTypePattern;
        target[q[i]] = nv[i];
    }
}

// compaction flags
__global__ void kKeepVertices(const int* __restrict__ type, int removedType, int numVertices, int* __restrict__ keep) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < numVertices) keep[v] = type[v] != removedType ? 1 : 0;
}
__global__ void kKeepFaces(const uint16_t* __restrict__ attr, int numFaces, int* __restrict__ keep) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f < numFaces) keep[f] = (attr[f] & kAttrRemove) ? 0 : 1;
}

__global__ void kGatherVertices(const int* __restrict__ type, int removedType, const int* __restrict__ addr,
                                int numVertices, const float* __restrict__ pos, const float* __restrict__ nrm,
                                float* __restrict__ pos2, float* __restrict__ nrm2) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= numVertices || type[v] == removedType) return;
    const int64_t o = addr[v];
    for (int a = 0; a < 3; ++a) {
        pos2[3 * o + a] = pos[3 * (int64_t)v + a];
        nrm2[3 * o + a] = nrm[3 * (int64_t)v + a];
    }
}

// removeQuadrilateralsP3X3Y (:517-537) / removeQuadsP3333 (:653-683): the kept
// quads' remapped vertices and new attributes
__global__ void kRemapQuads(const int4* __restrict__ he, const int* __restrict__ faceFirst, MeshDims md,
                            const uint16_t* __restrict__ attr, const int* __restrict__ faceAddr,
                            const int* __restrict__ type, const int* __restrict__ target, const int* __restrict__ addr,
                            int removedType, int remapPattern, int newVertices, int4* __restrict__ quads,
                            uint16_t* __restrict__ attr2, uint32_t* status) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= md.F) return;
    const uint32_t a = attr[f];
    if (a & kAttrRemove) return;
    int hs[4], q[4];
    if (!faceRing(he, faceFirst, f, md, hs, q)) {
        atomicOr(status, kStatusBadIndex);
        return;
    }
    int r[4];
    for (int i = 0; i < 4; ++i) {
        int v = q[i];
        if (remapPattern ? (a & kAttrPattern) != 0 : type[v] == removedType) v = target[v];
        int n = inb(v, md.V) ? addr[v] : -1;
        if (!inb(n, newVertices) || type[inb(v, md.V) ? v : 0] == removedType) {
            atomicOr(status, kStatusMappingSwap);
            n = 0;
        }
        r[i] = n;
    }
    const int o = faceAddr[f];
    quads[o] = make_int4(r[0], r[1], r[2], r[3]);
    attr2[o] = (uint16_t)(0x1Fu | (a & MDMC_FACE_NON_MANIFOLD) | (a & kAttrBoundary));
}

// collectHalfedgeElements (:14-60) for the reduced quads
__global__ void kCollectHalfedges(const int4* __restrict__ quads, const uint16_t* __restrict__ attr2, int numFaces,
                                  int4* __restrict__ he, int* __restrict__ faceFirst, uint16_t* __restrict__ attr) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= numFaces) return;
    const int4 v = quads[q];
    const int h0 = 4 * q;
    he[h0] = make_int4(v.x, q, h0 + 1, -1);
    he[h0 + 1] = make_int4(v.y, q, h0 + 2, -1);
    he[h0 + 2] = make_int4(v.z, q, h0 + 3, -1);
    he[h0 + 3] = make_int4(v.w, q, h0, -1);
    faceFirst[q] = h0;
    attr[q] = attr2[q];
}

}  // namespace

void launchValence(const int4* he, MeshDims md, int* val, cudaStream_t s) {
    if (md.H <= 0) return;
    countLaunch();
    kValence<<<(md.H + 255) / 256, 256, 0, s>>>(he, md, val);
}

void launchSimplify3X3Y(const int4* he, const int* faceFirst, MeshDims md, const int* val, int color, uint16_t* attr,
                        int* count, int4* merge, int* claimA, int* claimC, float* pos, float* nrm, int* type,
                        int* target, uint32_t* status, cudaStream_t s) {
    if (md.F <= 0) return;
    countLaunch(3);
    const unsigned b = (unsigned)((md.F + 255) / 256);
    kMark3X3Y<<<b, 256, 0, s>>>(he, faceFirst, md, val, color, attr, count, status);
    kDecide3X3Y<<<b, 256, 0, s>>>(he, faceFirst, md, val, count, color, attr, merge, claimA, claimC);
    kApply3X3Y<<<b, 256, 0, s>>>(md, merge, claimA, claimC, pos, nrm, attr, type, target);
}

void launchSimplify3333(const int4* he, const int* faceFirst, MeshDims md, const int* val, uint16_t* attr, int* type,
                        int* target, cudaStream_t s) {
    if (md.F <= 0) return;
    countLaunch(2);
    const unsigned b = (unsigned)((md.F + 255) / 256);
    kClear3333<<<b, 256, 0, s>>>(md, attr);
    kMark3333<<<b, 256, 0, s>>>(he, faceFirst, md, val, attr, type, target);
}

void launchKeepFlags(const int* type, int removedType, int numVertices, int* keepV, const uint16_t* attr, int numFaces,
                     int* keepF, cudaStream_t s) {
    if (numVertices > 0) {
        countLaunch();
        kKeepVertices<<<(numVertices + 255) / 256, 256, 0, s>>>(type, removedType, numVertices, keepV);
    }
    if (numFaces > 0) {
        countLaunch();
        kKeepFaces<<<(numFaces + 255) / 256, 256, 0, s>>>(attr, numFaces, keepF);
    }
}

void launchCompactMesh(const int4* he, const int* faceFirst, MeshDims md, const uint16_t* attr, const int* type,
                       const int* target, int removedType, int remapPattern, const int* vAddr, const int* fAddr,
                       int newVertices, const float* pos, const float* nrm, float* pos2, float* nrm2, int4* quads,
                       uint16_t* attr2, uint32_t* status, cudaStream_t s) {
    if (md.V > 0) {
        countLaunch();
        kGatherVertices<<<(md.V + 255) / 256, 256, 0, s>>>(type, removedType, vAddr, md.V, pos, nrm, pos2, nrm2);
    }
    if (md.F > 0) {
        countLaunch();
        kRemapQuads<<<(md.F + 255) / 256, 256, 0, s>>>(he, faceFirst, md, attr, fAddr, type, target, vAddr, removedType,
                                                       remapPattern, newVertices, quads, attr2, status);
    }
}

void launchCollectHalfedges(const int4* quads, const uint16_t* attr2, int numFaces, int4* he, int* faceFirst,
                            uint16_t* attr, cudaStream_t s) {
    if (numFaces <= 0) return;
    countLaunch();
    kCollectHalfedges<<<(numFaces + 255) / 256, 256, 0, s>>>(quads, attr2, numFaces, he, faceFirst, attr);
}

}  // namespace mdmc
