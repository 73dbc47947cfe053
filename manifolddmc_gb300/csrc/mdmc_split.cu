// Non-manifold edge splitting (ManifoldSplitter, D/PostProcesses/ManifoldSplitter.cu).
//
// Working-copy layout (deterministic; the reference appends with atomics):
// with n non-manifold faces taken in ascending face order, face k owns copy
// vertices 4k..4k+3 and copy halfedges 4k..4k+3 (its corners and edges), copy
// face k, and, once subdivided, new vertices 4n+4k..4n+4k+3, new halfedges
// 4n+16k..4n+16k+15 (inner ring, then three per boundary quad) and new faces
// n+4k..n+4k+3.  Merge-partner lists are sorted after the collapse so that
// the partner closure and "first valid twin" do not depend on atomic order.
#include <cuda_runtime.h>

#include "mdmc_device.cuh"
#include "mdmc_kernels.h"
#include "mdmc_scan.cuh"

namespace mdmc {

constexpr uint32_t kRemove = 16;      // Flags::setRemoveFlag
constexpr uint32_t kNonManifold = 1;  // Flags::setNonManifoldFlag
constexpr int kNone = -1;

// countNonManifoldFaces + the list of those faces in one prefix sum: the scan
// reads each face's flag from its attributes, and its apply pass writes every
// flagged face id to its place (no flag array, no compaction pass)
struct FaceNMRead {
    static constexpr bool kFour = true;
    const uint16_t* __restrict__ attr;
    __device__ __forceinline__ int operator[](int64_t f) const {
        return (attr[f] & MDMC_FACE_NON_MANIFOLD) ? 1 : 0;
    }
    __device__ __forceinline__ void four(int64_t f, int v[4]) const {  // (8 bytes: four attributes)
        const uint2 q = *reinterpret_cast<const uint2*>(attr + f);
        const uint32_t w[2] = {q.x, q.y};
#pragma unroll
        for (int k = 0; k < 4; ++k) v[k] = ((w[k >> 1] >> (16 * (k & 1))) & MDMC_FACE_NON_MANIFOLD) ? 1 : 0;
    }
    bool vectorOk() const { return (reinterpret_cast<uintptr_t>(attr) & 15u) == 0; }
};
struct CompactPost {
    static constexpr bool kStaged = false;
    static constexpr bool kPrefixes = false;  // (only the total and the compacted list are read)
    int* out;
    __device__ __forceinline__ void operator()(int64_t i, int at, int v) const {
        if (v) out[at] = (int)i;
    }
    __device__ __forceinline__ void total(int64_t, int) const {}
};
bool scanNMFaces(const uint16_t* attr, int numFaces, int* offsets, int* nmFaces, int* scratch, cudaStream_t s) {
    return exclusiveScanOf<int>(FaceNMRead{attr}, offsets, numFaces, scratch, s, CompactPost{nmFaces});
}

// copy-back selection (kept elements without an original are appended), read
// by the scan that numbers them
struct AppendRead {
    static constexpr bool kFour = true;
    const uint32_t* __restrict__ fl;
    const int* __restrict__ c2o;
    __device__ __forceinline__ int operator[](int64_t i) const {
        return (!(fl[i] & 16u) && c2o[i] == -1) ? 1 : 0;  // kRemove, kNone
    }
    __device__ __forceinline__ void four(int64_t i, int v[4]) const {
        const uint4 f = *reinterpret_cast<const uint4*>(fl + i);
        const int4 c = *reinterpret_cast<const int4*>(c2o + i);
        v[0] = (!(f.x & 16u) && c.x == -1) ? 1 : 0;
        v[1] = (!(f.y & 16u) && c.y == -1) ? 1 : 0;
        v[2] = (!(f.z & 16u) && c.z == -1) ? 1 : 0;
        v[3] = (!(f.w & 16u) && c.w == -1) ? 1 : 0;
    }
    bool vectorOk() const {
        return ((reinterpret_cast<uintptr_t>(fl) | reinterpret_cast<uintptr_t>(c2o)) & 15u) == 0;
    }
};
// (assignHalfedgeIDs: an appended element's mesh id, base + its number,
// written by the apply pass into its copy -> original map; the per-element
// numbers are then not written, only their total)
struct AssignPost {
    static constexpr bool kStaged = false;
    static constexpr bool kPrefixes = false;
    int* c2o;
    int base;
    __device__ __forceinline__ void operator()(int64_t i, int at, int v) const {
        if (v) c2o[i] = base + at;
    }
    __device__ __forceinline__ void total(int64_t, int) const {}
};
bool scanAppends(const uint32_t* fl, int* c2o, int count, int* offsets, int* scratch, cudaStream_t s, int assignBase) {
    if (assignBase >= 0)
        return exclusiveScanOf<int>(AppendRead{fl, c2o}, offsets, count, scratch, s, AssignPost{c2o, assignBase});
    return exclusiveScanOf<int>(AppendRead{fl, c2o}, offsets, count, scratch, s);
}

__global__ void kFillInt(int* p, int64_t n, int v) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}
void launchFillInt(int* p, int64_t n, int v, cudaStream_t s) {
    if (n <= 0) return;
    int blocks = (int)std::min<int64_t>((n + 255) / 256, 152 * 16);
    countLaunch();
    kFillInt<<<blocks, 256, 0, s>>>(p, n, v);
}

// copyVerticesToWorkingCopy / copyHalfedgesToWorkingCopy / copyFacesToWorkingCopy
// (:307-446).  Every original vertex maps to its smallest copy (the
// reference keeps whichever copy wrote last; all copies hold the same data).
__global__ void kCopyOut(const int* __restrict__ nmFaces, int n, const int4* __restrict__ he,
                         const int* __restrict__ faceFirst, const uint16_t* __restrict__ faceAttr,
                         const float* __restrict__ pos, const float* __restrict__ nrm, SplitWork w, uint32_t* status) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int f = nmFaces[k];
    if (!inb(f, w.F)) {
        atomicOr(status, kStatusBadIndex);
        return;
    }
    int h = faceFirst[f];
    // a face of the DMC mesh holds halfedges 4f'..4f'+3 in walk order: load
    // them together (and check the order), else walk
    int4 e4[4];
    bool direct = (h & 3) == 0 && inb(h + 3, w.H);
    if (direct) {
#pragma unroll
        for (int i = 0; i < 4; ++i) e4[i] = he[h + i];
#pragma unroll
        for (int i = 0; i < 4; ++i) direct = direct && e4[i].z == h + ((i + 1) & 3);
    }
    // copies 4k..4k+3: gathered in registers, written as whole vectors
    int vs[4], hs[4];
    float pq[12], nq[12];
    for (int i = 0; i < 4; ++i) {
        if (!inb(h, w.H) || !inb(direct ? e4[i].x : he[h].x, w.V)) {
            atomicOr(status, kStatusBadIndex);
            return;
        }
        const int4 e = direct ? e4[i] : he[h];
        const int c = 4 * k + i;
        const int v = e.x;
        for (int a = 0; a < 3; ++a) {
            pq[3 * i + a] = pos[3 * (int64_t)v + a];
            nq[3 * i + a] = nrm[3 * (int64_t)v + a];
        }
        vs[i] = v;
        hs[i] = h;
        if (w.touched && v < w.dmcV) w.touched[v] = 1;
        atomicMin(&w.vO2C[v], c);
        w.he[c] = e;
        w.hO2C[h] = c;
        h = e.z;
    }
    float4* pd = reinterpret_cast<float4*>(w.pos + 12 * (int64_t)k);
    float4* nd = reinterpret_cast<float4*>(w.nrm + 12 * (int64_t)k);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        pd[q] = make_float4(pq[4 * q], pq[4 * q + 1], pq[4 * q + 2], pq[4 * q + 3]);
        nd[q] = make_float4(nq[4 * q], nq[4 * q + 1], nq[4 * q + 2], nq[4 * q + 3]);
    }
    const int4 v4 = make_int4(vs[0], vs[1], vs[2], vs[3]), h4 = make_int4(hs[0], hs[1], hs[2], hs[3]);
    *reinterpret_cast<int4*>(w.vC2O + 4 * (int64_t)k) = v4;
    *reinterpret_cast<int4*>(w.origV + 4 * (int64_t)k) = v4;
    *reinterpret_cast<int4*>(w.hC2O + 4 * (int64_t)k) = h4;
    *reinterpret_cast<int4*>(w.origH + 4 * (int64_t)k) = h4;
    w.first[k] = 4 * k;  // hO2C of the face's first halfedge
    w.attr[k] = faceAttr[f];
    w.fC2O[k] = f;
    w.fO2C[f] = k;
}

// updateWorkingCopyHalfedges (:463-505); twins outside the copy become -twin-2
__global__ void kUpdateRefs(int n, SplitWork w, uint32_t* status) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= 4 * n) return;
    int4 e = w.he[c];
    if (!inb(e.x, w.V) || !inb(e.y, w.F) || !inb(e.z, w.H) || (e.w >= 0 && !inb(e.w, w.H))) {
        atomicOr(status, kStatusBadIndex);
        return;
    }
    e.x = w.vO2C[e.x];
    e.y = w.fO2C[e.y];
    e.z = w.hO2C[e.z];
    if (e.w >= 0) {
        const int t = w.hO2C[e.w];
        e.w = (t == kNone) ? -e.w - 2 : t;
    }
    if (!inb(e.x, w.nv) || !inb(e.y, w.nf) || !inb(e.z, w.nh)) atomicOr(status, kStatusBadIndex);
    w.he[c] = e;
}

// markHalfedgesAsNonManifold (:527-555)
__global__ void kMarkNM(const int4* __restrict__ nmList, const DevCounters* ctr,
                        SplitWork w, uint32_t* status) {
    const int count = min((int)ctr->nmBuckets, w.H / 4 + 1);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const NMIds b(nmList[i]);
        for (int k = 0; k < 4; ++k) {
            const int id = b.ids[k];
            const int c = inb(id, w.H) ? w.hO2C[id] : kNone;
            if (!inb(c, w.nh) || !inb(w.he[c].x, w.nv)) {
                atomicOr(status, kStatusBadTwin);
                continue;
            }
            atomicOr(&w.hfl[c], kNonManifold);
            atomicOr(&w.vfl[w.he[c].x], kNonManifold);
        }
    }
}

// performSubdivideQuads (:650-731): four inner vertices at (0.33|0.67)^2,
// an inner quad that keeps the face's id and four boundary quads that take
// the original edges.
__global__ void kSubdivide(int n, SplitWork w, uint32_t* status) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float uvs[4][2] = {{0.33f, 0.33f}, {0.67f, 0.33f}, {0.67f, 0.67f}, {0.33f, 0.67f}};
    int hid[4], vid[4];
    int4 orig[4];  // the face's halfedge records
    // the copy of face k holds halfedges 4k..4k+3 in walk order (kCopyOut,
    // kUpdateRefs): load them together, walk only if that does not hold
#pragma unroll
    for (int i = 0; i < 4; ++i) orig[i] = w.he[4 * k + i];
    bool direct = w.first[k] == 4 * k;
#pragma unroll
    for (int i = 0; i < 4; ++i) direct = direct && orig[i].z == 4 * k + ((i + 1) & 3);
    if (direct) {
#pragma unroll
        for (int i = 0; i < 4; ++i) hid[i] = 4 * k + i;
    } else {
        int h = w.first[k];
        for (int i = 0; i < 4; ++i) {
            if (!inb(h, w.nh)) {
                atomicOr(status, kStatusBadIndex);
                return;
            }
            hid[i] = h;
            orig[i] = w.he[h];
            h = orig[i].z;
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (!inb(orig[i].x, w.nv)) {
            atomicOr(status, kStatusBadIndex);
            return;
        }
        vid[i] = orig[i].x;
    }
    F3 P[4], N[4];
    for (int i = 0; i < 4; ++i) {
        P[i] = f3(w.pos[3 * (int64_t)vid[i]], w.pos[3 * (int64_t)vid[i] + 1], w.pos[3 * (int64_t)vid[i] + 2]);
        N[i] = f3(w.nrm[3 * (int64_t)vid[i]], w.nrm[3 * (int64_t)vid[i] + 1], w.nrm[3 * (int64_t)vid[i] + 2]);
    }
    auto mix = [](F3 a, F3 b, float t) { return a * (1.f - t) + b * t; };
    // inner vertices 4n+4k..4n+4k+3: positions and normals as three float4 each
    float pq[12], nq[12];
    int inner[4];
    for (int i = 0; i < 4; ++i) {
        const float u = uvs[i][0], v = uvs[i][1];
        const F3 pp = mix(mix(P[0], P[1], u), mix(P[3], P[2], u), v);
        const F3 nn = mix(mix(N[0], N[1], u), mix(N[3], N[2], u), v);
        pq[3 * i] = pp.x; pq[3 * i + 1] = pp.y; pq[3 * i + 2] = pp.z;
        nq[3 * i] = nn.x; nq[3 * i + 1] = nn.y; nq[3 * i + 2] = nn.z;
        inner[i] = 4 * n + 4 * k + i;
    }
    {
        const int64_t c0 = 4 * (int64_t)n + 4 * (int64_t)k;
        float4* pd = reinterpret_cast<float4*>(w.pos + 3 * c0);
        float4* nd = reinterpret_cast<float4*>(w.nrm + 3 * c0);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            pd[q] = make_float4(pq[4 * q], pq[4 * q + 1], pq[4 * q + 2], pq[4 * q + 3]);
            nd[q] = make_float4(nq[4 * q], nq[4 * q + 1], nq[4 * q + 2], nq[4 * q + 3]);
        }
        // the differentiable path's parent of inner vertex i: corner i
        *reinterpret_cast<int4*>(w.origV + c0) =
            make_int4(w.vC2O[vid[0]], w.vC2O[vid[1]], w.vC2O[vid[2]], w.vC2O[vid[3]]);
    }
    // halfedges 4n+16k..+15, each written once with its twin: the inner ring
    // (i -> i+1, twin: the second halfedge of boundary quad i+1), then three
    // per boundary quad j (corner j -> inner j -> inner j-1 -> the original
    // edge j-1, which closes it)
    const int hb = 4 * n + 16 * k;
    int ih[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) ih[i] = hb + i;
#pragma unroll
    for (int i = 0; i < 4; ++i)
        w.he[ih[i]] = make_int4(inner[i], k, ih[(i + 1) & 3], hb + 4 + 3 * ((i + 1) & 3) + 1);
    w.first[k] = ih[0];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int prev = (j + 3) & 3;
        const int q = hb + 4 + 3 * j;
        const int nf = n + 4 * k + j;
        w.he[q] = make_int4(vid[j], nf, q + 1, hb + 4 + 3 * ((j + 1) & 3) + 2);
        w.he[q + 1] = make_int4(inner[j], nf, q + 2, ih[prev]);
        w.he[q + 2] = make_int4(inner[prev], nf, hid[prev], hb + 4 + 3 * prev);
        // the original edge keeps origin and twin, joins the boundary quad
        w.he[hid[prev]] = make_int4(orig[prev].x, nf, q, orig[prev].w);
        w.first[nf] = q;
        w.attr[nf] = 0x1F;  // HalfedgeFace(): INVALID_COLOR
    }
    // swapHalfedgeMappings (:629-648): the inner ring takes over the original
    // halfedge slots, the original edges become new halfedges
    for (int i = 0; i < 4; ++i) {
        const int a = hid[i], b = ih[i];
        const int ao = w.hC2O[a], bo = w.hC2O[b];
        w.hC2O[a] = bo;
        w.hC2O[b] = ao;
        if (ao != kNone && bo == kNone && inb(ao, w.H)) w.hO2C[ao] = b;
        else atomicOr(status, kStatusMappingSwap);
    }
}

// DeviceMergeList::mark (:749-765); partner slots are sorted afterwards
__device__ __forceinline__ void markPartner(int* num, int* slots, int count, int a, int b, uint32_t* status) {
    if (!inb(a, count) || !inb(b, count)) {
        atomicOr(status, kStatusBadIndex);
        return;
    }
    const int idx = atomicAdd(&num[a], 1);
    if (idx - 1 < 4) slots[4 * (int64_t)a + idx - 1] = b;
    if (idx > 2) atomicOr(status, kStatusPartnerOverflow);
}

// performCollapseNonManifoldHalfedges + collapseHalfedge (:767-868)
__global__ void kCollapse(SplitWork w, uint32_t* status) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= w.nh) return;
    if (!(w.hfl[t] & kNonManifold)) return;
    const int tw = w.he[t].w;
    if (!inb(tw, w.nh)) {
        atomicOr(status, kStatusBadTwin);
        return;
    }
    if (tw < t) return;
    int f0[4], f1[4];
    int4 cur = w.he[t], ctw = w.he[tw];
    f0[0] = t;
    f1[0] = tw;
    for (int i = 1; i < 4; ++i) {
        if (!inb(cur.z, w.nh) || !inb(ctw.z, w.nh)) {
            atomicOr(status, kStatusBadIndex);
            return;
        }
        f0[i] = cur.z;
        f1[4 - i] = ctw.z;
        cur = w.he[cur.z];
        ctw = w.he[ctw.z];
    }
    const int fa = w.he[f0[0]].y, fb = w.he[f1[0]].y;
    if (!inb(fa, w.nf) || !inb(fb, w.nf)) {
        atomicOr(status, kStatusBadIndex);
        return;
    }
    for (int i = 0; i < 4; ++i) {
        atomicOr(&w.hfl[f0[i]], kRemove);
        atomicOr(&w.hfl[f1[i]], kRemove);
    }
    atomicOr(&w.ffl[fa], kRemove);
    atomicOr(&w.ffl[fb], kRemove);
    {
        const int a = w.he[f0[2]].x, b = w.he[f1[1]].x;
        markPartner(w.vNum, w.vSlots, w.nv, a, b, status);
        markPartner(w.vNum, w.vSlots, w.nv, b, a, status);
        if (a < w.cornerLimit || b < w.cornerLimit) w.flags[0] = 1;
    }
    {
        const int a = w.he[f0[3]].x, b = w.he[f1[2]].x;
        markPartner(w.vNum, w.vSlots, w.nv, a, b, status);
        markPartner(w.vNum, w.vSlots, w.nv, b, a, status);
        if (a < w.cornerLimit || b < w.cornerLimit) w.flags[0] = 1;
    }
    for (int i = 1; i < 4; ++i) {
        const int a = f0[i], b = f1[i];
        const int at = w.he[a].w, bt = w.he[b].w;
        if (at < 0 || bt < 0) {
            atomicOr(status, kStatusBadTwin);
            continue;
        }
        markPartner(w.hNum, w.hSlots, w.nh, a, bt, status);
        markPartner(w.hNum, w.hSlots, w.nh, bt, a, status);
        markPartner(w.hNum, w.hSlots, w.nh, b, at, status);
        markPartner(w.hNum, w.hSlots, w.nh, at, b, status);
    }
}

__global__ void kSortPartners(int* num, int* slots, int count) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= count) return;
    const int n = min(num[a] - 1, 4);
    if (n < 2) return;
    int s[4];
    for (int i = 0; i < n; ++i) s[i] = slots[4 * (int64_t)a + i];
    for (int i = 1; i < n; ++i) {
        int v = s[i], j = i - 1;
        while (j >= 0 && s[j] > v) { s[j + 1] = s[j]; --j; }
        s[j + 1] = v;
    }
    for (int i = 0; i < n; ++i) slots[4 * (int64_t)a + i] = s[i];
}

// DeviceMergeList::getAllPartnersOf (:25-62): breadth-first closure, at most
// 12 partners.  Slots only hold ids checked by markPartner.
__device__ int closure(const int* num, const int* slots, int v, int out[12], uint32_t* status) {
    auto cnt = [&](int x) { return min(num[x], 5); };
    int np = cnt(v);
    if (np <= 1) return np;
    for (int i = 0; i < np - 1; ++i) out[i] = slots[4 * (int64_t)v + i];
    for (int i = 0; i < np - 1; ++i) {
        const int p = out[i];
        const int npp = cnt(p);
        for (int k = 0; k < npp - 1; ++k) {
            const int pp = slots[4 * (int64_t)p + k];
            bool contained = (pp == v);
            for (int z = 0; z < np - 1; ++z) contained = contained || out[z] == pp;
            if (!contained) {
                if (np - 1 >= 12) {
                    atomicOr(status, kStatusPartnerOverflow);
                    continue;
                }
                out[np - 1] = pp;
                ++np;
            }
        }
    }
    return np;
}

// mergeVertices (:936-990) for vertex v; the survivor's normal receives the
// averaged position, as in the reference (:989).  Returns the survivor (v
// itself, or the smaller partner that replaces it), or v with np <= 1.
__device__ __forceinline__ int mergeVertex(const SplitWork& w, int v, uint32_t* status) {
    int part[12];
    const int np = closure(w.vNum, w.vSlots, v, part, status);
    if (np <= 1) return v;
    if (np > 12) {
        atomicOr(status, kStatusPartnerOverflow);
        return v;
    }
    int smallest = v;
    F3 p = f3(w.pos[3 * (int64_t)v], w.pos[3 * (int64_t)v + 1], w.pos[3 * (int64_t)v + 2]);
    bool obsolete = false;
    for (int i = 0; i < np - 1; ++i) {
        const int q = part[i];
        p = p + f3(w.pos[3 * (int64_t)q], w.pos[3 * (int64_t)q + 1], w.pos[3 * (int64_t)q + 2]);
        if (q < smallest) {
            obsolete = true;
            smallest = q;
        }
    }
    if (obsolete) {
        atomicOr(&w.vfl[v], kRemove);
        return smallest;
    }
    p = p / (float)np;
    w.pos[3 * (int64_t)smallest] = p.x; w.pos[3 * (int64_t)smallest + 1] = p.y; w.pos[3 * (int64_t)smallest + 2] = p.z;
    w.nrm[3 * (int64_t)smallest] = p.x; w.nrm[3 * (int64_t)smallest + 1] = p.y; w.nrm[3 * (int64_t)smallest + 2] = p.z;
    return smallest;
}

// every copy vertex, grid-stride; only when a corner copy has merge partners
// (flags[0]) or without subdivision (else kMergeInner does the work)
__global__ void kMergeVertices(SplitWork w, uint32_t* status) {
    if (w.cornerLimit < w.nv && w.flags[0] == 0) return;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < w.nv; v += gridDim.x * blockDim.x) mergeVertex(w, v, status);
}

// updateHalfedgeVertexIDs (:992-1019), grid-stride over the halfedges; only
// when a corner copy has merge partners (flags[0]) or without subdivision
__global__ void kUpdateOrigins(SplitWork w, uint32_t* status) {
    if (w.cornerLimit < w.nv && w.flags[0] == 0) return;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < w.nh; t += gridDim.x * blockDim.x) {
        const int v = w.he[t].x;
        if (!inb(v, w.nv)) continue;
        int part[12];
        const int np = closure(w.vNum, w.vSlots, v, part, status);
        if (np <= 1) continue;
        int s = v;
        for (int i = 0; i < np - 1; ++i) s = min(s, part[i]);
        w.he[t].x = s;
    }
}

// Subdivided copies whose merge partners are all inner vertices (no corner
// has partners): one thread per inner vertex merges it (mergeVertex) and
// points its halfedges at the survivor (updateHalfedgeVertexIDs).  Inner
// vertex i of face k is the origin of exactly three halfedges: its
// inner-ring halfedge and the second and third halfedge of two boundary
// quads (kSubdivide's numbering).
__global__ void kMergeInner(SplitWork w, int n, uint32_t* status) {
    if (w.flags[0] != 0) return;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= 4 * n) return;
    const int v = 4 * n + j;
    const int sm = mergeVertex(w, v, status);
    if (sm == v) return;
    const int k = j >> 2, i = j & 3;
    const int hb = 4 * n + 16 * k;
    const int hs[3] = {hb + i, hb + 4 + 3 * i + 1, hb + 4 + 3 * ((i + 1) & 3) + 2};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        int* x = reinterpret_cast<int*>(w.he) + 4 * (int64_t)hs[q];
        if (*x == v) *x = sm;
        else atomicOr(status, kStatusMappingSwap);
    }
}

// mergeHalfedges (:1021-1067) as the oracle states it: every decision reads
// the twins as they were before the pass, and the pairs (t, valid) are then
// applied in increasing t, a later pair overwriting an earlier one.  Here
// the decisions write nothing into the halfedges: each pair offers
// ((t + 1) << 32 | value) to both of its halfedges by a 64-bit atomicMax,
// so that every halfedge keeps the value of its last pair, and
// kApplyMergedTwins writes those values afterwards.  (Writing the twins in
// the deciding pass raced with decisions that read a kept partner's twin:
// on one grid of 96 a batch run once gave 1243 non-manifold vertices instead
// of 1242.)
__global__ void kMergeHalfedges(SplitWork w, uint32_t* status) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= w.nh) return;
    if (w.hfl[t] & kRemove) return;
    int part[12];
    const int np = closure(w.hNum, w.hSlots, t, part, status);
    if (np <= 1) return;
    int valid = -1;
    for (int i = 0; i < np - 1; ++i) {
        const int tw = w.he[part[i]].w;
        if (!inb(tw, w.nh)) continue;
        if (!(w.hfl[tw] & kRemove)) {
            valid = tw;
            break;
        }
    }
    if (valid == -1 || valid < t) return;
    const unsigned long long tag = (unsigned long long)(t + 1) << 32;
    atomicMax(w.hTwinBest + t, tag | (uint32_t)valid);
    atomicMax(w.hTwinBest + valid, tag | (uint32_t)t);
}

__global__ void kApplyMergedTwins(SplitWork w) {
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < w.nh; x += gridDim.x * blockDim.x) {
        const unsigned long long b = w.hTwinBest[x];
        if (b) reinterpret_cast<int*>(w.he)[4 * (int64_t)x + 3] = (int)(uint32_t)b;
    }
}

// A corner copy other than the smallest copy of its original vertex: after
// kUpdateRefs no halfedge names it, and it holds the same data as the
// smallest copy (both move identically), so the copy-back leaves it to that
// copy.  (The moving pass moves it anyway: the check costs it more than the
// skipped moves save.)
__device__ __forceinline__ bool spareCorner(const SplitWork& w, int v) {
    if (v >= w.cornerLimit) return false;
    const int o = w.vC2O[v];
    return inb(o, w.V) && w.vO2C[o] != v;
}

// performMoveVerticesToSurface (:1130-1160)
template <class View>
__global__ void kMoveVertices(View g, float iso, SplitWork w) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= w.nv) return;
    if (w.vfl[v] & kRemove) return;
    const F3 p = f3(w.pos[3 * (int64_t)v], w.pos[3 * (int64_t)v + 1], w.pos[3 * (int64_t)v + 2]);
    int idx[3];
    g.cellOf(p, idx);
    float s[8];
    corners(g, idx[0], idx[1], idx[2], s);
    const F3 fi = f3((float)idx[0], (float)idx[1], (float)idx[2]);
    const F3 fi1 = f3((float)(idx[0] + 1), (float)(idx[1] + 1), (float)(idx[2] + 1));
    const F3 mn = g.origin() + fi * g.deltas();
    const F3 mx = g.origin() + fi1 * g.deltas();
    F3 local = (p - mn) / (mx - mn);
    SurfaceIterator it{s, iso};
    it.move(local);
    const F3 q = g.origin() + (fi + local) * g.deltas();
    w.pos[3 * (int64_t)v] = q.x; w.pos[3 * (int64_t)v + 1] = q.y; w.pos[3 * (int64_t)v + 2] = q.z;
}

// copyVerticesBack / copyHalfedgesBack / copyFacesBack (:1176-1260); V2, H2
// and F2 are the mesh sizes after the appends
__global__ void kCopyBackVertices(SplitWork w, const int* __restrict__ app, int V2, float* pos, float* nrm,
                                  uint32_t* status) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= w.nv) return;
    if ((w.vfl[v] & kRemove) || spareCorner(w, v)) return;
    int o = w.vC2O[v];
    if (o == kNone) {
        o = w.V + app[v];
        w.vC2O[v] = o;
        // the DMC vertex it descends from (parents of earlier appends resolved)
        const int p = w.origV[v];
        const int parent = !inb(p, w.V) ? -1 : (p < w.dmcV ? p : w.appParent[p - w.dmcV]);
        // (after a simplification the mesh has fewer vertices than the DMC
        // produced and no appended vertex has a slot here)
        if (o >= w.dmcV && o < V2) w.appParent[o - w.dmcV] = parent;
    }
    if (!inb(o, V2)) {
        atomicOr(status, kStatusBadIndex);
        return;
    }
    for (int a = 0; a < 3; ++a) {
        pos[3 * (int64_t)o + a] = w.pos[3 * (int64_t)v + a];
        nrm[3 * (int64_t)o + a] = w.nrm[3 * (int64_t)v + a];
    }
}
__global__ void kCopyBackFaces(SplitWork w, const int* __restrict__ app, int H2, int F2, int* faceFirst,
                               uint16_t* faceAttr, uint32_t* status) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= w.nf) return;
    if (w.ffl[f] & kRemove) return;
    int o = w.fC2O[f];
    if (o == kNone) {
        o = w.F + app[f];
        w.fC2O[f] = o;
    }
    const int fh = w.first[f];
    const int first = inb(fh, w.nh) ? w.hC2O[fh] : kNone;
    if (!inb(o, F2) || !inb(first, H2)) {
        atomicOr(status, kStatusBadIndex);
        return;
    }
    faceFirst[o] = first;
    faceAttr[o] = w.attr[f];
}
// copyHalfedgesBack + updateHalfedgesBack (:1205-1295)
__global__ void kCopyBackHalfedges(SplitWork w, int V2, int H2, int F2, int4* he, uint32_t* status) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= w.nh) return;
    if (w.hfl[t] & kRemove) return;
    int4 e = w.he[t];
    const int self = w.hC2O[t];
    if (!inb(self, H2) || !inb(e.z, w.nh) || !inb(e.y, w.nf) || !inb(e.x, w.nv) || (e.w >= 0 && !inb(e.w, w.nh))) {
        atomicOr(status, kStatusBadIndex);
        return;
    }
    e.z = w.hC2O[e.z];
    e.y = w.fC2O[e.y];
    e.x = w.vC2O[e.x];
    if (e.w < 0) {
        e.w = -e.w - 2;
        if (e.w != -1) {
            if (inb(e.w, w.H)) setTwinOut(he, e.w, self);
            else atomicOr(status, kStatusBadIndex);
        }
    } else {
        e.w = w.hC2O[e.w];
    }
    if (!inb(e.z, H2) || !inb(e.y, F2) || !inb(e.x, V2)) atomicOr(status, kStatusBadIndex);
    he[self] = e;
}

// after an iteration: clear the dense original->copy maps it touched
__global__ void kResetMaps(int n, const int* __restrict__ nmFaces, SplitWork w) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= 4 * n) return;
    if (inb(w.origV[c], w.V)) w.vO2C[w.origV[c]] = 0x7FFFFFFF;
    if (inb(w.origH[c], w.H)) w.hO2C[w.origH[c]] = kNone;
    if ((c & 3) == 0 && inb(nmFaces[c >> 2], w.F)) w.fO2C[nmFaces[c >> 2]] = kNone;
}

// ---------------------------------------------------------------------------
// Local refresh (refreshHashTable, D/Halfedges/HalfedgeMesh.cu:1063-1100,
// restricted to what an iteration can change).  Let D be the corners of the
// iteration's non-manifold faces plus the vertices it appends.  Every
// halfedge the copy-back writes runs between two vertices of D, and every
// other halfedge keeps its ends, its next and its face.  So only edges with
// both ends in D change their halfedge sets: their old sets (from the rows
// of the last full refresh, before the copy-back) are counted out and their
// new sets counted in.  Vertex flags follow from per-vertex member counts,
// face flags from per-face edge counts, and the edge counters from the
// per-edge differences; the result equals a full refresh of the new mesh.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool inD(const SplitWork& w, int v) { return inb(v, w.V) && w.vO2C[v] != 0x7FFFFFFF; }

// the corner copy that stands for original vertex d (its smallest copy), or -1
__device__ __forceinline__ int distinctCorner(const SplitWork& w, int c) {
    const int d = w.origV[c];
    return (inb(d, w.V) && w.vO2C[d] == c) ? d : -1;
}

__global__ void kCensusCountOld(SplitWork w, int n, const int* __restrict__ rowStart, const int2* __restrict__ adj,
                                const int4* __restrict__ he, int* out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    int nOld = 0, nSame = 0;
    if (c < 4 * n) {
        const int d = distinctCorner(w, c);
        if (d >= 0)
            for (int k = rowStart[d]; k < rowStart[d + 1]; ++k) {
                const int2 r = adj[k];
                if (!inD(w, r.x >= 0 ? r.x : ~r.x) || !inb(r.y, w.H) || !inb(he[r.y].y, w.F)) continue;
                ++nOld;
                if (w.hO2C[r.y] == kNone) ++nSame;
            }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        nOld += __shfl_down_sync(0xffffffffu, nOld, o);
        nSame += __shfl_down_sync(0xffffffffu, nSame, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (nOld) atomicAdd(out, nOld);
        if (nSame) atomicAdd(out + 1, nSame);
    }
}

__global__ void kCensusCollectOld(SplitWork w, int n, const int* __restrict__ rowStart, const int2* __restrict__ adj,
                                  const int4* __restrict__ he, CensusRec* oldRecs, CensusRec* newRecs, int* fill,
                                  int2 caps, uint32_t* status) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= 4 * n) return;
    const int d = distinctCorner(w, c);
    if (d < 0) return;
    for (int k = rowStart[d]; k < rowStart[d + 1]; ++k) {
        const int2 r = adj[k];
        const int o = r.x >= 0 ? r.x : ~r.x;
        if (!inD(w, o)) continue;
        const int f = inb(r.y, w.H) ? he[r.y].y : -1;
        if (!inb(f, w.F)) {
            atomicOr(status, kStatusBadIndex);
            continue;
        }
        CensusRec rec;
        rec.lo = d;
        rec.hi = o;
        rec.h = r.y;
        rec.origin = r.x >= 0 ? d : o;
        rec.face = f;
        rec.slot = -1;
        const int a = atomicAdd(fill, 1);
        if (a < caps.x) oldRecs[a] = rec;
        if (w.hO2C[r.y] == kNone) {
            const int b = atomicAdd(fill + 1, 1);
            if (b < caps.y) newRecs[b] = rec;
        }
    }
}

__global__ void kCensusCollectNew(SplitWork w, const int4* __restrict__ he, MeshDims md, CensusRec* newRecs, int* fill,
                                  int cap, uint32_t* status) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= w.nh || (w.hfl[t] & kRemove)) return;
    const int self = w.hC2O[t];
    if (!inb(self, md.H)) {
        atomicOr(status, kStatusBadIndex);
        return;
    }
    const int4 e = he[self];
    if (!inb(e.z, md.H) || !inb(e.x, md.V) || !inb(e.y, md.F)) {
        atomicOr(status, kStatusBadIndex);
        return;
    }
    const int b = he[e.z].x;
    if (!inb(b, md.V)) {
        atomicOr(status, kStatusBadIndex);
        return;
    }
    CensusRec rec;
    rec.lo = min(e.x, b);
    rec.hi = max(e.x, b);
    rec.h = self;
    rec.origin = e.x;
    rec.face = e.y;
    rec.slot = -1;
    const int at = atomicAdd(fill + 1, 1);
    if (at < cap) newRecs[at] = rec;
}

// each record finds (or opens) its edge's slot and counts itself in
__global__ void kCensusInsert(CensusRec* recs, const int* fill, int cap, CensusTable t, uint32_t* status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= min(*fill, cap)) return;
    CensusRec& r = recs[i];
    const unsigned long long key = ((unsigned long long)(uint32_t)r.lo << 32) | (uint32_t)r.hi;
    const uint32_t mask = (uint32_t)t.capacity - 1u;
    uint32_t slot = (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> 32) & mask;
    for (int probe = 0; probe < t.capacity; ++probe) {
        const unsigned long long k = atomicCAS(t.keys + slot, ~0ull, key);
        if (k == ~0ull || k == key) {
            const int idx = atomicAdd(t.count + slot, 1);
            if (idx < 4) t.members[4 * (int64_t)slot + idx] = r.h;
            r.slot = (int)slot;
            return;
        }
        slot = (slot + 1u) & mask;
    }
    atomicOr(status, kStatusBadIndex);  // table full (sized to twice the records: not reached)
}

// each record counts itself out (sign < 0) or in (sign > 0); the edge's
// first record to claim it settles the edge-level counters
__global__ void kCensusApply(const CensusRec* __restrict__ recs, const int* fill, int cap, CensusTable t, int sign,
                             uint32_t* vcount, uint8_t* faceNM, int4* nmList, int nmCapacity, DevCounters* ctr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= min(*fill, cap)) return;
    const CensusRec r = recs[i];
    if (r.slot < 0) return;
    const int cnt = t.count[r.slot];
    const unsigned long long one = sign > 0 ? 1ull : ~0ull;
    if (atomicExch(t.claim + r.slot, 1) == 0) {
        atomicAdd(&ctr->edges, one);
        if (cnt == 3) atomicAdd(&ctr->edges3, one);
        if (cnt == 4) atomicAdd(&ctr->edges4, one);
        if (sign > 0 && cnt > 4) atomicOr(&ctr->status, kStatusBucketOverflow);
        if (sign > 0 && cnt == 4) {  // the new mesh's 4-face edges, ascending ids
            int m[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) m[k] = t.members[4 * (int64_t)r.slot + k];
#define MDMC_CX(a, b)          \
    if (m[b] < m[a]) {          \
        const int x = m[a];     \
        m[a] = m[b];            \
        m[b] = x;               \
    }
            MDMC_CX(0, 1) MDMC_CX(2, 3) MDMC_CX(0, 2) MDMC_CX(1, 3) MDMC_CX(1, 2)
#undef MDMC_CX
            const unsigned long long at = atomicAdd(&ctr->nmBuckets, 1ull);
            if (at < (unsigned long long)nmCapacity) nmList[at] = make_int4(m[0], m[1], m[2], m[3]);
            else atomicOr(&ctr->status, kStatusBadIndex);
        }
    }
    if (cnt != 2 && cnt <= 4) {
        const int sh = cnt == 1 ? kVCountShiftBoundary : (cnt == 3 ? kVCountShiftWeird : kVCountShiftNM);
        const uint32_t old = atomicAdd(vcount + r.origin, sign > 0 ? (1u << sh) : (0u - (1u << sh)));
        if (sign > 0 && ((old >> sh) & 0x3FFu) >= 1000u) atomicOr(&ctr->status, kStatusCountOverflow);
    }
    if (cnt > 2) {
        const uint32_t add = (cnt == 4 ? 0x11u : 0x01u) << ((r.face & 3) * 8);
        atomicAdd(reinterpret_cast<uint32_t*>(faceNM) + (r.face >> 2), sign > 0 ? add : 0u - add);
    }
}

// flags of every vertex and face a record names, from the final counts
__global__ void kCensusFinish(const CensusRec* __restrict__ recs, const int* fill, int cap,
                              const uint32_t* __restrict__ vcount, const uint8_t* __restrict__ faceNM, uint8_t* vflags,
                              uint16_t* faceAttr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= min(*fill, cap)) return;
    const CensusRec r = recs[i];
    const uint32_t vc = vcount[r.origin];
    vflags[r.origin] = (uint8_t)((((vc >> kVCountShiftBoundary) & 0x3FFu) ? MDMC_VERTEX_BOUNDARY : 0u) |
                                 (((vc >> kVCountShiftWeird) & 0x3FFu) ? MDMC_VERTEX_WEIRD : 0u) |
                                 (((vc >> kVCountShiftNM) & 0x3FFu) ? MDMC_VERTEX_NON_MANIFOLD : 0u));
    faceAttr[r.face] = (uint16_t)((faceAttr[r.face] & 0x1Fu) | ((faceNM[r.face] >> 4) ? MDMC_FACE_NON_MANIFOLD : 0u));
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
// blocks of `bs` threads covering n elements
static inline int nb(int64_t n, int bs) { return (int)std::max<int64_t>((n + bs - 1) / bs, 1); }

void launchSplitCopy(const int* nmFaces, int n, const int4* he, const int* faceFirst, const uint16_t* faceAttr,
                     const float* pos, const float* nrm, const SplitWork& w, uint32_t* status, cudaStream_t s) {
    countLaunch(2);
    kCopyOut<<<nb(n, 256), 256, 0, s>>>(nmFaces, n, he, faceFirst, faceAttr, pos, nrm, w, status);
    kUpdateRefs<<<nb(4 * (int64_t)n, 256), 256, 0, s>>>(n, w, status);
}
void launchSplitMarkNM(const int4* nmList, const DevCounters* ctr, const SplitWork& w,
                       uint32_t* status, cudaStream_t s) {
    countLaunch();
    kMarkNM<<<152 * 8, 256, 0, s>>>(nmList, ctr, w, status);
}
void launchSplitSubdivide(int n, const SplitWork& w, uint32_t* status, cudaStream_t s) {
    countLaunch();
    kSubdivide<<<nb(n, 128), 128, 0, s>>>(n, w, status);
}
void launchSplitCollapse(const SplitWork& w, uint32_t* status, cudaStream_t s) {
    countLaunch(3);
    kCollapse<<<nb(w.nh, 256), 256, 0, s>>>(w, status);
    kSortPartners<<<nb(w.nv, 256), 256, 0, s>>>(w.vNum, w.vSlots, w.nv);
    kSortPartners<<<nb(w.nh, 256), 256, 0, s>>>(w.hNum, w.hSlots, w.nh);
}
void launchSplitMerge(const SplitWork& w, uint32_t* status, cudaStream_t s) {
    if (w.cornerLimit < w.nv) {  // subdivided: nv = 8n, corners below 4n
        countLaunch();
        kMergeInner<<<nb(w.cornerLimit, 128), 128, 0, s>>>(w, w.cornerLimit / 4, status);
    }
    // the general passes (they return at once after kMergeInner did the work)
    countLaunch(2);
    kMergeVertices<<<std::min(nb(w.nv, 128), 152 * 16), 128, 0, s>>>(w, status);
    kUpdateOrigins<<<std::min(nb(w.nh, 128), 152 * 16), 128, 0, s>>>(w, status);
}
void launchSplitMergeHalfedges(const SplitWork& w, uint32_t* status, cudaStream_t s) {
    countLaunch(2);
    cudaMemsetAsync(w.hTwinBest, 0, sizeof(unsigned long long) * (size_t)w.nh, s);
    kMergeHalfedges<<<nb(w.nh, 128), 128, 0, s>>>(w, status);
    kApplyMergedTwins<<<std::min(nb(w.nh, 256), 152 * 16), 256, 0, s>>>(w);
}
void launchSplitMove(const GridDesc& g, float iso, const SplitWork& w, cudaStream_t s) {
    countLaunch();
    if (g.refined) kMoveVertices<RefinedView><<<nb(w.nv, 128), 128, 0, s>>>(g.ref, iso, w);
    else kMoveVertices<PlainView><<<nb(w.nv, 128), 128, 0, s>>>(g.plain, iso, w);
}
void launchSplitCopyBack(const SplitWork& w, const int* appV, const int* appH, const int* appF, int V2, int H2, int F2,
                         float* pos, float* nrm, int4* he, int* faceFirst, uint16_t* faceAttr, uint32_t* status,
                         cudaStream_t s) {
    countLaunch(3);
    kCopyBackVertices<<<nb(w.nv, 256), 256, 0, s>>>(w, appV, V2, pos, nrm, status);
    kCopyBackFaces<<<nb(w.nf, 256), 256, 0, s>>>(w, appF, H2, F2, faceFirst, faceAttr, status);
    kCopyBackHalfedges<<<nb(w.nh, 256), 256, 0, s>>>(w, V2, H2, F2, he, status);
}
void launchSplitResetMaps(int n, const int* nmFaces, const SplitWork& w, cudaStream_t s) {
    countLaunch();
    kResetMaps<<<nb(4 * (int64_t)n, 256), 256, 0, s>>>(n, nmFaces, w);
}

void launchCensusCountOld(const SplitWork& w, int n, const int* rowStart, const int2* adj, const int4* he, int* out,
                          cudaStream_t s) {
    if (n <= 0) return;
    countLaunch();
    kCensusCountOld<<<nb(4 * (int64_t)n, 256), 256, 0, s>>>(w, n, rowStart, adj, he, out);
}
void launchCensusCollectOld(const SplitWork& w, int n, const int* rowStart, const int2* adj, const int4* he,
                            CensusRec* oldRecs, CensusRec* newRecs, int* fill, int capOld, int capNew, uint32_t* status,
                            cudaStream_t s) {
    if (n <= 0) return;
    countLaunch();
    kCensusCollectOld<<<nb(4 * (int64_t)n, 256), 256, 0, s>>>(w, n, rowStart, adj, he, oldRecs, newRecs, fill,
                                                               make_int2(capOld, capNew), status);
}
void launchCensusCollectNew(const SplitWork& w, const int4* he, MeshDims md, CensusRec* newRecs, int* fill, int capNew,
                            uint32_t* status, cudaStream_t s) {
    if (w.nh <= 0) return;
    countLaunch();
    kCensusCollectNew<<<nb(w.nh, 256), 256, 0, s>>>(w, he, md, newRecs, fill, capNew, status);
}
void launchCensusApply(CensusRec* recs, const int* fill, int cap, const CensusTable& t, int sign, uint32_t* vcount,
                       uint8_t* faceNM, int4* nmList, int nmCapacity, DevCounters* ctr, cudaStream_t s) {
    if (cap <= 0) return;
    countLaunch(2);
    kCensusInsert<<<nb(cap, 256), 256, 0, s>>>(recs, fill, cap, t, &ctr->status);
    kCensusApply<<<nb(cap, 256), 256, 0, s>>>(recs, fill, cap, t, sign, vcount, faceNM, nmList, nmCapacity, ctr);
}
void launchCensusFinish(const CensusRec* recs, const int* fill, int cap, const uint32_t* vcount, const uint8_t* faceNM,
                        uint8_t* vflags, uint16_t* faceAttr, cudaStream_t s) {
    if (cap <= 0) return;
    countLaunch();
    kCensusFinish<<<nb(cap, 256), 256, 0, s>>>(recs, fill, cap, vcount, faceNM, vflags, faceAttr);
}

}  // namespace mdmc
