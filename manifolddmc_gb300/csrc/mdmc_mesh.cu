// Halfedge-mesh kernels: edge-table finishing (twins and flags), the
// asymptotic-decider twin repair, face-fan detection and the output pass.
//
// Reference: connectHalfedgeTwins and refresh*Flags
// (D/Halfedges/HalfedgeMesh.cu:92-291), reconnectHalfedges
// (D/PostProcesses/ManifoldCreator.cu:39-312), detectNonManifoldVertices
// (D/PostProcesses/ManifoldCreator.cu:319-536) and the statistics getters
// (D/Halfedges/HalfedgeMesh.cu:1164-1239).
//
// The reference's bucket order is the order of atomic inserts; here the ids
// of a bucket are sorted first, which makes every per-bucket decision (twin
// pairing of 3- and 4-face edges, wall-side ties in the repair) deterministic.
#include <cuda_runtime.h>

#include <algorithm>

#include "mdmc_device.cuh"
#include "mdmc_kernels.h"

namespace mdmc {

__device__ __forceinline__ void setTwin(int4* he, int h, int t) { reinterpret_cast<int*>(he)[4 * (int64_t)h + 3] = t; }

// face attributes: clearPatternFlags + unsetNonManifoldFlag (HalfedgeMesh.cu:1050-1055)
__global__ void kResetFaceFlags(uint16_t* attr, int numFaces) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f < numFaces) attr[f] = (uint16_t)(attr[f] & 0x1F);
}
void launchResetFaceFlags(uint16_t* attr, int numFaces, cudaStream_t s) {
    if (numFaces > 0) {
        countLaunch();
        kResetFaceFlags<<<(numFaces + 255) / 256, 256, 0, s>>>(attr, numFaces);
    }
}

// ---------------------------------------------------------------------------
// Edge buckets without a hash table.  Every halfedge is listed in the row of
// the smaller of its two end vertices as (larger end, id), the larger end
// stored as ~end when the halfedge leaves it; all halfedges of the vertex
// pair {a, b} then sit in one row.  A warp takes 32 consecutive vertices,
// whose rows are one contiguous span: it stages the span in shared memory
// with coalesced loads and each lane settles the buckets of its own row.
// Same buckets, counts and flags as the edge table of refreshHashTable /
// connectHalfedgeTwins (D/Halfedges/HalfedgeMesh.cu:62-291, :1063-1100); a
// bucket keeps its 4 smallest ids.
// ---------------------------------------------------------------------------

// the end vertices of halfedge h, false (and a status bit) when an id is out of range
__device__ __forceinline__ bool edgeEnds(const int4* __restrict__ he, MeshDims md, int h, int& a, int& b,
                                         uint32_t* status) {
    const int4 e = he[h];
    a = e.x;
    b = (inb(e.z, md.H) && inb(a, md.V)) ? he[e.z].x : -1;
    if (!inb(b, md.V)) {
        atomicOr(status, kStatusBadIndex);
        return false;
    }
    return true;
}

// row sizes; rank[h] = the halfedge's place in its row (the count before it,
// in atomic order), -1 for a halfedge with an id out of range
__global__ void kEdgeRowDegree(const int4* __restrict__ he, MeshDims md, int* __restrict__ deg, int* __restrict__ rank,
                               uint32_t* status) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= md.H) return;
    int a, b;
    rank[h] = edgeEnds(he, md, h, a, b, status) ? atomicAdd(&deg[min(a, b)], 1) : -1;
}

__global__ void kEdgeRowScatter(const int4* __restrict__ he, MeshDims md, const int* __restrict__ rowStart,
                                const int* __restrict__ rank, int2* __restrict__ adj) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= md.H) return;
    const int k = rank[h];
    if (k < 0) return;
    const int a = he[h].x, b = he[he[h].z].x;  // in range (checked by the degree pass)
    const int m = min(a, b), o = max(a, b);
    adj[rowStart[m] + k] = make_int2(a == m ? o : ~o, h);
}

// the 4 smallest ids of a bucket, ascending, with their origins
__device__ __forceinline__ void keepSmallest(int ids[4], int org[4], int g, int go) {
    if (g >= ids[3]) return;
    int k = 3;
    while (k > 0 && ids[k - 1] > g) {
        ids[k] = ids[k - 1];
        org[k] = org[k - 1];
        --k;
    }
    ids[k] = g;
    org[k] = go;
}

constexpr int kBucketWarps = 8;
constexpr int kBucketStage = 512;  // row entries of 32 vertices staged per warp (longer spans: global memory)

// One warp per tile of 32 consecutive vertices (grid-stride over tiles).  The
// tile's rows form one contiguous span of the row array; it is staged in
// shared memory, each entry's larger end vertex and row (lane) beside it.
// Then one lane per entry counts the entries of its own row with the same
// end vertex (its bucket) and those before it: the bucket's first entry
// counts the bucket.  Only an entry of a bucket of other than two halfedges
// (or, with connectTwins, any entry) goes on: it collects the bucket's four
// smallest ids and acts for its own halfedge: the vertex flag of its origin
// (non-manifold / weird / boundary by the bucket's size; with vcount, also
// counted per vertex), the non-manifold face flag and the per-face counts of
// edges with more than two and with four halfedges (faceNM, zeroed by the
// caller), its twin by the rules of
// connectHalfedgeTwins (with connectTwins), and the first entry of a 4-face
// bucket lists it.  The counters take one addition per block.
__global__ void __launch_bounds__(32 * kBucketWarps) kEdgeBuckets(int4* __restrict__ he, MeshDims md,
                                                                  const int* __restrict__ rowStart,
                                                                  const int2* __restrict__ adj, int connectTwins,
                                                                  uint16_t* faceAttr, uint8_t* vflags, uint8_t* faceNM,
                                                                  uint32_t* vcount, int4* __restrict__ nmList,
                                                                  DevCounters* ctr) {
    __shared__ int2 stage[kBucketWarps][kBucketStage];
    __shared__ int stageEnd[kBucketWarps][kBucketStage];
    __shared__ uint8_t stageRow[kBucketWarps][kBucketStage];
    __shared__ int rowBegin[kBucketWarps][33];
    __shared__ unsigned long long part[3][kBucketWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned long long nE = 0, nE3 = 0, nE4 = 0;
    const int tiles = (md.V + 31) / 32;
    for (int tile = blockIdx.x * kBucketWarps + warp; tile < tiles; tile += gridDim.x * kBucketWarps) {
        const int m0 = tile * 32;
        const int myStart = rowStart[min(m0 + lane, md.V)];
        const int s0 = __shfl_sync(0xffffffffu, myStart, 0);
        const int s1 = rowStart[min(m0 + 32, md.V)];
        const int span = s1 - s0;
        const bool staged = span <= kBucketStage;
        __syncwarp();
        rowBegin[warp][lane] = myStart - s0;
        if (lane == 0) rowBegin[warp][32] = span;
        if (staged)
            for (int k = lane; k < span; k += 32) {
                const int2 r = adj[s0 + k];
                stage[warp][k] = r;
                stageEnd[warp][k] = r.x >= 0 ? r.x : ~r.x;
            }
        __syncwarp();
        if (staged) {  // each lane tags its row's entries
            const int b = rowBegin[warp][lane], e = rowBegin[warp][lane + 1];
            for (int k = b; k < e; ++k) stageRow[warp][k] = (uint8_t)lane;
        }
        __syncwarp();
        for (int k = lane; k < span; k += 32) {
            int row;
            int2 mine;
            if (staged) {
                row = stageRow[warp][k];
                mine = stage[warp][k];
            } else {  // a long span: the row by bisection over the 33 bounds
                int lo = 0, hi = 32;
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (rowBegin[warp][mid] <= k) lo = mid;
                    else hi = mid;
                }
                row = lo;
                mine = adj[s0 + k];
            }
            const int r0 = rowBegin[warp][row], r1 = rowBegin[warp][row + 1];
            const int oe = mine.x >= 0 ? mine.x : ~mine.x;
            int cnt = 0, before = 0;
            if (staged) {
                for (int j = r0; j < r1; ++j) {
                    const int same = stageEnd[warp][j] == oe ? 1 : 0;
                    cnt += same;
                    before += j < k ? same : 0;
                }
            } else {
                for (int j = r0; j < r1; ++j) {
                    const int x = adj[s0 + j].x;
                    const int same = (x >= 0 ? x : ~x) == oe ? 1 : 0;
                    cnt += same;
                    before += j < k ? same : 0;
                }
            }
            if (before == 0) {
                ++nE;
                nE3 += cnt == 3 ? 1 : 0;
                nE4 += cnt == 4 ? 1 : 0;
            }
            if (cnt == 2 && !connectTwins) continue;
            // the rare path: the bucket's four smallest ids and their origins
            const int m = m0 + row;
            int ids[4] = {0x7FFFFFFF, 0x7FFFFFFF, 0x7FFFFFFF, 0x7FFFFFFF}, org[4] = {-1, -1, -1, -1};
            for (int j = r0; j < r1; ++j) {
                const int2 r = staged ? stage[warp][j] : adj[s0 + j];
                if ((r.x >= 0 ? r.x : ~r.x) == oe) keepSmallest(ids, org, r.y, r.x >= 0 ? m : oe);
            }
            if (before == 0) {
                if (cnt > 4) atomicOr(&ctr->status, kStatusBucketOverflow);
                if (cnt >= 4) {
                    const unsigned long long slot = atomicAdd(&ctr->nmBuckets, 1ULL);
                    if (slot < (unsigned long long)(md.H / 4 + 1))
                        nmList[slot] = make_int4(ids[0], ids[1], ids[2], ids[3]);
                    else atomicOr(&ctr->status, kStatusBadIndex);
                }
            }
            const int h = mine.y, origin = mine.x >= 0 ? m : oe;
            if (connectTwins && cnt >= 2 && cnt <= 4) {
                int kk = 4;
#pragma unroll
                for (int t = 3; t >= 0; --t)
                    if (ids[t] == h) kk = t;
                if (kk < 4) {
                    int twin;
                    if (cnt == 2) twin = ids[1 - kk];
                    else if (cnt == 3) twin = ids[kk == 2 ? 0 : kk + 1];
                    else  // "HACKY_OLD_WAY", HalfedgeMesh.cu:250-281
                        twin = ids[org[0] != org[1] ? (kk ^ 1) : (org[0] != org[2] ? (kk ^ 2) : 3 - kk)];
                    setTwin(he, h, twin);
                }
            }
            if (cnt == 2) continue;
            if (cnt == 4) orVertexFlag(vflags, origin, MDMC_VERTEX_NON_MANIFOLD);
            else if (cnt == 3) orVertexFlag(vflags, origin, MDMC_VERTEX_WEIRD);
            else if (cnt == 1) orVertexFlag(vflags, origin, MDMC_VERTEX_BOUNDARY);
            if (vcount && cnt <= 4) {
                const int sh = cnt == 1 ? kVCountShiftBoundary : (cnt == 3 ? kVCountShiftWeird : kVCountShiftNM);
                const uint32_t old = atomicAdd(vcount + origin, 1u << sh);
                if (((old >> sh) & 0x3FFu) >= 1000u) atomicOr(&ctr->status, kStatusCountOverflow);
            }
            if (cnt > 2) {
                const int f = he[h].y;
                if (inb(f, md.F)) {
                    atomicAdd(reinterpret_cast<uint32_t*>(faceNM) + (f >> 2), (cnt == 4 ? 0x11u : 0x01u) << ((f & 3) * 8));
                    if (cnt == 4) orFaceAttr(faceAttr, f, MDMC_FACE_NON_MANIFOLD);
                } else {
                    atomicOr(&ctr->status, kStatusBadIndex);
                }
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        nE += __shfl_down_sync(0xffffffffu, nE, o);
        nE3 += __shfl_down_sync(0xffffffffu, nE3, o);
        nE4 += __shfl_down_sync(0xffffffffu, nE4, o);
    }
    if (lane == 0) {
        part[0][warp] = nE;
        part[1][warp] = nE3;
        part[2][warp] = nE4;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        unsigned long long t = 0;
#pragma unroll
        for (int w = 0; w < kBucketWarps; ++w) t += part[threadIdx.x][w];
        if (t) atomicAdd(threadIdx.x == 0 ? &ctr->edges : (threadIdx.x == 1 ? &ctr->edges3 : &ctr->edges4), t);
    }
}

void launchEdgeRowDegree(const int4* he, MeshDims md, int* deg, int* rank, uint32_t* status, cudaStream_t s) {
    if (md.H <= 0) return;
    countLaunch();
    kEdgeRowDegree<<<(md.H + 255) / 256, 256, 0, s>>>(he, md, deg, rank, status);
}

void launchEdgeBuckets(int4* he, MeshDims md, const int* rowStart, const int* rank, int2* adj, int connectTwins,
                       uint16_t* faceAttr, uint8_t* vflags, uint8_t* faceNM, uint32_t* vcount, int4* nmList,
                       DevCounters* ctr, cudaStream_t s) {
    if (md.H <= 0) return;
    countLaunch(2);
    kEdgeRowScatter<<<(md.H + 255) / 256, 256, 0, s>>>(he, md, rowStart, rank, adj);
    const int64_t tiles = ((int64_t)md.V + 31) / 32;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((tiles + kBucketWarps - 1) / kBucketWarps, 152 * 8));
    kEdgeBuckets<<<blocks, 32 * kBucketWarps, 0, s>>>(he, md, rowStart, adj, connectTwins, faceAttr, vflags, faceNM,
                                                      vcount, nmList, ctr);
}

// ---------------------------------------------------------------------------
// reconnectHalfedges, D/PostProcesses/ManifoldCreator.cu:39-312
// ---------------------------------------------------------------------------
__device__ __forceinline__ F3 nudge(int it) {
    F3 r = f3((it & 1) ? 1.f : 0.f, (it & 2) ? 1.f : 0.f, (it & 4) ? 1.f : 0.f);
    if (it & 8) r.x = -r.x;
    if (it & 16) r.y = -r.y;
    if (it & 32) r.z = -r.z;
    return r * kEpsilon;
}

__device__ __forceinline__ F3 loadP(const float* pos, int v) {
    return f3(pos[3 * (int64_t)v], pos[3 * (int64_t)v + 1], pos[3 * (int64_t)v + 2]);
}

template <class View>
__global__ void kReconnect(View g, float iso, const int4* __restrict__ nmList,
                           const DevCounters* ctr, int4* he, const float* __restrict__ pos, MeshDims md,
                           uint32_t* status) {
    const int count = min((int)ctr->nmBuckets, md.H / 4 + 1);
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < count; w += gridDim.x * blockDim.x) {
        const NMIds b(nmList[w]);
        // every id, its next, next.next and their origins must be in range
        bool ok = true;
        for (int k = 0; k < 4 && ok; ++k) {
            int h = b.ids[k];
            for (int d = 0; d < 3 && ok; ++d) {
                ok = inb(h, md.H) && inb(he[h].x, md.V);
                if (ok) h = he[h].z;
            }
        }
        if (!ok) {
            atomicOr(status, kStatusBadIndex);
            continue;
        }
        const int4 h0 = he[b.ids[0]];
        const int n0 = h0.x, n1 = he[h0.z].x;
        F3 p0 = loadP(pos, n0), p1 = loadP(pos, n1);
        int c0[3], c1[3];
        g.cellOf(p0, c0);
        g.cellOf(p1, c1);
        // nudge both vertices until their cells are face neighbours (:87-108)
        for (int i = 0; i < 0x40; ++i) {
            const F3 o0 = nudge(i);
            F3 o1 = o0;
            int finalK = -1;
            for (int k = 0; k < 0x40; ++k) {
                o1 = nudge(k);
                int a[3], bb[3];
                g.cellOf(p0 + o0, a);
                g.cellOf(p1 + o1, bb);
                int sum = abs(a[0] - bb[0]) + abs(a[1] - bb[1]) + abs(a[2] - bb[2]);
                if (sum == 1) { finalK = k; break; }
            }
            if (finalK != -1) {
                p0 = p0 + o0;
                g.cellOf(p0, c0);
                p1 = p1 + o1;
                g.cellOf(p1, c1);
                break;
            }
        }
        const int64_t lin0 = ((int64_t)c0[2] * g.Y + c0[1]) * g.X + c0[0];
        const int64_t lin1 = ((int64_t)c1[2] * g.Y + c1[1]) * g.X + c1[0];
        int A[3], B[3];
        for (int a = 0; a < 3; ++a) {
            A[a] = lin0 < lin1 ? c0[a] : c1[a];
            B[a] = lin0 < lin1 ? c1[a] : c0[a];
        }
        int nr[3], mn[3];
        for (int a = 0; a < 3; ++a) {
            nr[a] = max(A[a], B[a]) - min(A[a], B[a]);
            mn[a] = max(A[a], B[a]);
        }
        int xo[3] = {0, 0, 0}, yo[3] = {0, 0, 0};
        if (nr[0] == 0) {
            xo[0] = 1;
            if (nr[1] == 0) yo[1] = 1;
            else yo[2] = 1;
        } else {
            xo[1] = 1;
            yo[2] = 1;
        }
        if (mn[0] < 0 || mn[1] < 0 || mn[2] < 0 || mn[0] + 1 >= g.X || mn[1] + 1 >= g.Y || mn[2] + 1 >= g.Z)
            atomicOr(status, kStatusWallOutOfGrid);
        const float w0 = atClamped(g, mn[0], mn[1], mn[2]);
        const float w1 = atClamped(g, mn[0] + xo[0], mn[1] + xo[1], mn[2] + xo[2]);
        const float w2 = atClamped(g, mn[0] + xo[0] + yo[0], mn[1] + xo[1] + yo[1], mn[2] + xo[2] + yo[2]);
        const float w3 = atClamped(g, mn[0] + yo[0], mn[1] + yo[1], mn[2] + yo[2]);
        const F3 corner0 = g.origin() + g.deltas() * f3((float)mn[0], (float)mn[1], (float)mn[2]);
        const F3 corner2 = g.origin() + g.deltas() * f3((float)(mn[0] + xo[0] + yo[0]), (float)(mn[1] + xo[1] + yo[1]),
                                                        (float)(mn[2] + xo[2] + yo[2]));
        const bool omitX = xo[0] == 0 && yo[0] == 0;
        const bool omitY = xo[1] == 0 && yo[1] == 0;
        auto down = [&](F3 p, float& u, float& v) {
            if (omitX) { u = p.y; v = p.z; }
            else if (omitY) { u = p.x; v = p.z; }
            else { u = p.x; v = p.y; }
        };
        float minU, minV, maxU, maxV;
        down(corner0, minU, minV);
        down(corner2, maxU, maxV);
        int sorted[4] = {-1, -1, -1, -1};
        for (int i = 0; i < 4; ++i) {
            const int hid = b.ids[i];
            const int opp = he[he[he[hid].z].z].x;
            float u, v;
            down(loadP(pos, opp), u, v);
            const float mnU = u - minU, mnV = v - minV, mxU = u - maxU, mxV = v - maxV;
            if (mnV < 0.f) sorted[0] = hid;
            if (mxU > 0.f) sorted[1] = hid;
            if (mxV > 0.f) sorted[2] = hid;
            if (mnU < 0.f) sorted[3] = hid;
        }
        if (sorted[0] < 0 || sorted[1] < 0 || sorted[2] < 0 || sorted[3] < 0) continue;
        // AsymptoticDecider2D::quadrant0BelongsTogether, D/Utils/AsymptoticDecider.h:119-164
        const float m00 = w0, m10 = w1, m11 = w2, m01 = w3;
        float C = m00 - m10;
        C = C - m01;
        C = C + m11;
        const float delta = (m00 * m11 - m10 * m01) / C;
        const bool together = (m00 < iso && delta >= iso) || (m00 >= iso && delta < iso);
        if (!together) {
            setTwin(he, sorted[0], sorted[1]); setTwin(he, sorted[1], sorted[0]);
            setTwin(he, sorted[2], sorted[3]); setTwin(he, sorted[3], sorted[2]);
        } else {
            setTwin(he, sorted[0], sorted[3]); setTwin(he, sorted[3], sorted[0]);
            setTwin(he, sorted[1], sorted[2]); setTwin(he, sorted[2], sorted[1]);
        }
    }
}

void launchReconnect(const GridDesc& g, float iso, const int4* nmList, const DevCounters* ctr,
                     int4* he, const float* pos, MeshDims md, uint32_t* status, cudaStream_t s) {
    countLaunch();
    if (g.refined) kReconnect<RefinedView><<<152 * 2, 128, 0, s>>>(g.ref, iso, nmList, ctr, he, pos, md, status);
    else kReconnect<PlainView><<<152 * 2, 128, 0, s>>>(g.plain, iso, nmList, ctr, he, pos, md, status);
}

// ---------------------------------------------------------------------------
// detectNonManifoldVertices, D/PostProcesses/ManifoldCreator.cu:319-536
// ---------------------------------------------------------------------------
// stepping around a vertex; any id outside the arrays ends the walk
__device__ __forceinline__ int stepCW(const int4* he, int h, int H) {
    const int t = he[h].w;
    if (t == -1) return -1;
    if (!inb(t, H)) return -2;
    const int n = he[t].z;
    return inb(n, H) ? n : -2;
}
__device__ __forceinline__ int stepCCW(const int4* he, int h, int H) {
    int p = h;
    for (int i = 0; i < 3; ++i) {
        p = he[p].z;
        if (!inb(p, H)) return -2;
    }
    const int t = he[p].w;
    if (t == -1) return -1;
    return inb(t, H) ? t : -2;
}
__device__ __forceinline__ int fanWalk(const int4* he, int start, bool cw, int H, uint32_t* status) {
    const int origin = he[start].x;
    int result = start;
    int cur = cw ? stepCW(he, start, H) : stepCCW(he, start, H);
    int guard = 0;
    while (cur >= 0) {
        if (cur == result) break;
        if (origin != he[cur].x) break;
        if (cur < result) result = cur;
        cur = cw ? stepCW(he, cur, H) : stepCCW(he, cur, H);
        if (++guard > 4096) {
            atomicOr(status, kStatusWalkLimit);
            break;
        }
    }
    if (cur == -2) atomicOr(status, kStatusBadIndex);
    return result;
}

// One walk per vertex.  When the walks from the vertex's smallest outgoing
// halfedge visit exactly all of the vertex's outgoing halfedges through
// symmetric twin pairs (faces are 4-cycles) -- clockwise back to the start
// (a closed fan), or clockwise to a boundary and counter-clockwise to the
// other boundary (an open fan) -- the counter-clockwise step is the inverse of
// the clockwise one on that fan: every outgoing halfedge's own walks cover the
// same fan, its key is the fan's smallest id, and the vertex has one fan with
// no limit hit.  Every other vertex (non-manifold, asymmetric twins) takes the
// per-halfedge walks and is counted.  Also turns "no outgoing halfedge" into -1.
//
// With the vertex pass's degrees (the DMC mesh after the twin repair), a
// positive degree needs no walk.  It says that every edge of the vertex's
// contour has a quad and that no face of its cell has four crossing edges.
// The vertex's faces are then the quads of its contour's edges; two
// consecutive ones share the mesh edge to the vertex of the neighbour across
// the cell face of their contour segment, that face has no other crossing
// edge, so exactly these two halfedges hold the vertex pair (the pairs the
// twin repair changes have four) and they are twins: the faces form one
// closed fan.  After the splitter the same holds for every DMC vertex it
// did not touch (no corner of a copied face): its faces, and the twins of
// their halfedges at it, are those the vertex pass saw.
__global__ void kFanFast(const int4* __restrict__ he, MeshDims md, int* __restrict__ vertexHE,
                         const int* __restrict__ deg, bool vertexPassDegrees, int* __restrict__ fans,
                         uint8_t* __restrict__ slow, uint8_t* __restrict__ vflags, unsigned long long* slowCount,
                         const unsigned long long* gate, const int* __restrict__ dmcDeg,
                         const uint8_t* __restrict__ touched, int dmcV) {
    if (gate && *gate != 0) return;  // a speculative pass whose mesh the splitter will change
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    bool isSlow = false;
    if (v < md.V) {
        // a DMC vertex the splitter did not touch has the out-degree the vertex
        // pass counted (the output pass left its star alone)
        const bool kept = dmcDeg && v < dmcV && !touched[v];
        const int ds = kept ? dmcDeg[v] : deg[v];
        const int d = ds < 0 ? -ds : ds;
        if (d == 0) {
            vertexHE[v] = -1;
            fans[v] = 0;
            slow[v] = 0;
            vflags[v] &= (uint8_t)~MDMC_VERTEX_MULTIPLE_FANS;
        } else if ((vertexPassDegrees || kept) && ds > 0) {
            fans[v] = 1;
            slow[v] = 0;
            vflags[v] &= (uint8_t)~MDMC_VERTEX_MULTIPLE_FANS;
        } else {
            const int start = vertexHE[v];
            bool ok = inb(start, md.H) && d <= 1024;
            bool open = false;
            int x = start, visited = 1;
            while (ok) {  // clockwise: next(twin(x))
                const int4 hx = he[x];
                if (hx.x != v) {
                    ok = false;
                    break;
                }
                if (hx.w == -1) {
                    open = true;
                    break;
                }
                if (!inb(hx.w, md.H)) {
                    ok = false;
                    break;
                }
                const int4 ht = he[hx.w];
                if (ht.w != x || !inb(ht.z, md.H)) {
                    ok = false;
                    break;
                }
                x = ht.z;
                if (x == start) break;
                if (++visited > d) ok = false;
            }
            x = start;
            while (ok && open) {  // counter-clockwise: twin(next^3(x)), up to the other boundary
                int p = x;
                for (int k = 0; k < 3 && ok; ++k) {
                    p = he[p].z;
                    ok = inb(p, md.H);
                }
                if (!ok) break;
                const int t = he[p].w;
                if (t == -1) break;
                if (!inb(t, md.H)) {
                    ok = false;
                    break;
                }
                const int4 htt = he[t];
                if (htt.w != p || htt.x != v) {
                    ok = false;
                    break;
                }
                x = t;
                if (x == start || ++visited > d) ok = false;
            }
            ok = ok && visited == d;
            fans[v] = ok ? 1 : 0;
            slow[v] = ok ? 0 : 1;
            isSlow = !ok;
            // one fan: not a non-manifold vertex (the slow ones are flagged by kFanFlags)
            if (ok) vflags[v] &= (uint8_t)~MDMC_VERTEX_MULTIPLE_FANS;
        }
    }
    const unsigned b = __ballot_sync(0xffffffffu, isSlow);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(slowCount, (unsigned long long)__popc(b));
}

// A fan key is the smallest halfedge id of the fan and has the origin of the
// halfedge it was found from, so "distinct (origin, key) pairs per origin"
// (the reference's sort + unique) equals "halfedges named as key by some
// halfedge, per origin".  No sort is needed.  Only the halfedges of vertices
// the single walk did not settle.
// (a grid-stride loop over a fixed grid: when no vertex is unsettled, which
// is the common case, each block reads the counter once and leaves)
// isKey[h] == mark: h is a fan key in this detection pass (the caller gives
// every pass its own mark, so that the marks of earlier passes need no clearing)
__global__ void kFanKeys(const int4* __restrict__ he, MeshDims md, const uint8_t* __restrict__ slow,
                         const unsigned long long* slowCount, uint8_t* __restrict__ isKey, uint8_t mark,
                         uint32_t* status) {
    if (*slowCount == 0) return;
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < md.H; h += gridDim.x * blockDim.x) {
        const int v = he[h].x;
        if (!inb(v, md.V) || !slow[v]) continue;
        const int k = min(h, min(fanWalk(he, h, true, md.H, status), fanWalk(he, h, false, md.H, status)));
        isKey[k] = mark;
    }
}

// (the marks are read 16 at a time and compared four at a time; few match)
__device__ __forceinline__ void countFanKey(const int4* __restrict__ he, MeshDims md, const uint8_t* __restrict__ slow,
                                            int h, int* __restrict__ fans, uint32_t* status) {
    const int v = he[h].x;
    if (inb(v, md.V)) {
        if (slow[v]) atomicAdd(&fans[v], 1);
    } else {
        atomicOr(status, kStatusBadIndex);
    }
}
__global__ void kFanCount(const int4* __restrict__ he, MeshDims md, const uint8_t* __restrict__ slow,
                          const unsigned long long* slowCount, const uint8_t* __restrict__ isKey, uint8_t mark,
                          int* __restrict__ fans, uint32_t* status) {
    if (*slowCount == 0) return;
    const uint32_t marks = 0x01010101u * mark;
    const int chunks = md.H >> 4;  // whole 16-byte chunks (isKey is 256-byte aligned)
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < chunks; c += gridDim.x * blockDim.x) {
        const uint4 k = reinterpret_cast<const uint4*>(isKey)[c];
        const uint32_t words[4] = {k.x, k.y, k.z, k.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            uint32_t eq = __vcmpeq4(words[q], marks);  // 0xFF in every byte that holds the mark
            while (eq) {
                const int b = (__ffs(eq) - 1) >> 3;
                eq &= ~(0xFFu << (8 * b));
                countFanKey(he, md, slow, 16 * c + 4 * q + b, fans, status);
            }
        }
    }
    // the last H mod 16 marks, one each
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int h = 16 * chunks + t;
    if (t < 16 && h < md.H && isKey[h] == mark) countFanKey(he, md, slow, h, fans, status);
}

// the vertices the single walk did not settle (kFanFast flagged the others;
// a grid-stride loop that leaves at once when there are none)
__global__ void kFanFlags(const int* __restrict__ fans, const uint8_t* __restrict__ slow, uint8_t* __restrict__ vflags,
                          int numVertices, DevCounters* ctr) {
    if (ctr->slowFans == 0) return;
    int nm = 0;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < numVertices; v += gridDim.x * blockDim.x) {
        if (!slow[v]) continue;
        uint8_t f = vflags[v];
        if (fans[v] > 1) {
            f |= MDMC_VERTEX_MULTIPLE_FANS;
            ++nm;
        } else {
            f &= (uint8_t)~MDMC_VERTEX_MULTIPLE_FANS;
        }
        vflags[v] = f;
    }
    blockAddTo(&ctr->nmVertices, nm);
}

void launchDetectFans(const int4* he, MeshDims md, int* vertexHE, const int* deg, bool vertexPassDegrees,
                      uint8_t* slow, uint8_t* isKey, uint8_t keyMark, int* fans, uint8_t* vflags, DevCounters* ctr,
                      uint32_t* status, const unsigned long long* gate, const int* dmcDeg, const uint8_t* touched,
                      int dmcV, cudaStream_t s) {
    if (md.V > 0) {
        countLaunch();
        kFanFast<<<(md.V + 255) / 256, 256, 0, s>>>(he, md, vertexHE, deg, vertexPassDegrees, fans, slow, vflags,
                                                    &ctr->slowFans, gate, dmcDeg, touched, dmcV);
    }
    if (md.H > 0) {
        countLaunch();
        const int blocks = std::min((md.H + 255) / 256, 152 * 8);
        kFanKeys<<<blocks, 256, 0, s>>>(he, md, slow, &ctr->slowFans, isKey, keyMark, status);
        countLaunch();
        kFanCount<<<blocks, 256, 0, s>>>(he, md, slow, &ctr->slowFans, isKey, keyMark, fans, status);
    }
    if (md.V > 0) {
        countLaunch();
        kFanFlags<<<std::min((md.V + 255) / 256, 152 * 8), 256, 0, s>>>(fans, slow, vflags, md.V, ctr);
    }
}

// ---------------------------------------------------------------------------
// output pass: face vertex quads, getNumQuadsWithNonManifoldEdges, and the
// smallest outgoing halfedge of every vertex
// ---------------------------------------------------------------------------
// (edge sizes: faceNM, one count per face, when given; else heValence, the
// quad pass's size of every halfedge's bucket)
__global__ void kFaceOutput(const int4* __restrict__ he, const int* __restrict__ faceFirst, MeshDims md,
                            const uint8_t* __restrict__ heValence, const uint8_t* __restrict__ faceNM,
                            int4* __restrict__ quads, int* vertexHE, int* deg, const uint8_t* __restrict__ touched,
                            int dmcV, DevCounters* ctr) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    int cnt = -1;
    if (f < md.F) {
        int h = faceFirst[f];
        int q[4] = {-1, -1, -1, -1}, hs[4] = {-1, -1, -1, -1};
        bool ok = true;
        // most faces (DMC quads, and the inner quads the splitter leaves in
        // their slots) hold halfedges h..h+3 in walk order: load those four
        // together and walk only when the links say otherwise
        bool direct = (h & 3) == 0 && inb(h + 3, md.H);
        if (direct) {
            int4 e[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) e[i] = he[h + i];
#pragma unroll
            for (int i = 0; i < 4; ++i) direct = direct && e[i].z == h + ((i + 1) & 3);
            if (direct)
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    q[i] = e[i].x;
                    hs[i] = h + i;
                }
        }
        for (int i = 0; i < 4 && ok && !direct; ++i) {
            ok = inb(h, md.H);
            if (ok) {
                const int4 e = he[h];
                q[i] = e.x;
                hs[i] = h;
                h = e.z;
            }
        }
        quads[f] = make_int4(q[0], q[1], q[2], q[3]);
        // the vertex stars (smallest outgoing halfedge, out-degree) from the
        // same four records: every halfedge lies in exactly one face.  (With
        // touched: a DMC vertex the splitter did not touch keeps the star the
        // quad pass gave it, since none of its outgoing halfedges changed.)
        if (ok && vertexHE)
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if (inb(q[i], md.V) && !(touched && q[i] < dmcV && !touched[q[i]])) {
                    atomicMin(&vertexHE[q[i]], hs[i]);
                    if (deg) atomicAdd(&deg[q[i]], 1);
                }
        if (ok) {
            cnt = 0;
            if (faceNM) cnt = faceNM[f] & kFaceNMCount;
            else
                for (int i = 0; i < 4; ++i)
                    if (heValence[hs[i]] > 2) ++cnt;
        } else {
            atomicOr(&ctr->status, kStatusBadIndex);
        }
    }
    // quads with 1..4 edges of more than two faces, 16 bits each
    blockAddPacked(cnt >= 1 && cnt <= 4 ? 1ull << (16 * (cnt - 1)) : 0ull, [&](unsigned long long t) {
#pragma unroll
        for (int k = 1; k <= 4; ++k)
            if ((t >> (16 * (k - 1))) & 0xFFFFu) atomicAdd(&ctr->quadsNM[k], (t >> (16 * (k - 1))) & 0xFFFFu);
    });
}

__global__ void kVertexHalfedgeFix(int* vertexHE, int numVertices) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < numVertices && vertexHE[v] == 0x7F7F7F7F) vertexHE[v] = -1;
}

void launchVertexHalfedgeFix(int* vertexHE, int numVertices, cudaStream_t s) {
    if (numVertices <= 0) return;
    countLaunch();
    kVertexHalfedgeFix<<<(numVertices + 255) / 256, 256, 0, s>>>(vertexHE, numVertices);
}

// the stars the output pass recomputes start from "none" (0x7F7F7F7F; atomicMin
// lowers it) and degree 0: every vertex's, or with touched only those of the
// touched DMC vertices and of the vertices appended after them
__global__ void kResetStars(int* vertexHE, int* deg, const uint8_t* __restrict__ touched, int dmcV, int numVertices) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < numVertices; v += gridDim.x * blockDim.x) {
        if (v < dmcV && !touched[v]) continue;
        vertexHE[v] = 0x7F7F7F7F;
        if (deg) deg[v] = 0;
    }
}

void launchOutput(const int4* he, const int* faceFirst, MeshDims md, const uint8_t* heValence, const uint8_t* faceNM,
                  int4* quads, int* vertexHE, int* deg, const uint8_t* touched, int dmcV, DevCounters* ctr,
                  uint32_t* status, cudaStream_t s) {
    (void)status;
    if (!touched) dmcV = 0;
    if (md.V > 0 && vertexHE) {
        if (touched) {
            countLaunch();
            kResetStars<<<std::min((md.V + 255) / 256, 152 * 8), 256, 0, s>>>(vertexHE, deg, touched, dmcV, md.V);
        } else {
            cudaMemsetAsync(vertexHE, 0x7F, sizeof(int) * (size_t)md.V, s);
            if (deg) cudaMemsetAsync(deg, 0, sizeof(int) * (size_t)md.V, s);
        }
    }
    if (md.F > 0) {
        countLaunch();
        kFaceOutput<<<(md.F + 255) / 256, 256, 0, s>>>(he, faceFirst, md, heValence, faceNM, quads, vertexHE, deg,
                                                        touched, dmcV, ctr);
    }
}

// ---------------------------------------------------------------------------
// HalfedgeMesh::toVertexAndIndexBuffer, D/Halfedges/HalfedgeMesh.cu:1102-1146
// (insertVertices :716-760, insertHalfedgeFaceIndices :690-714), with device
// arrays in place of the GL buffers: per vertex {position, normal, rgba}
// coloured by its flags, per quad the triangles (x, y, z) and (z, w, x)
// ---------------------------------------------------------------------------
// LazyEngine::Color::HSVtoRGB (Renderer/Materials/Colors.h:15-57)
__device__ __forceinline__ F3 hsvToRgb(float h, float s, float v) {
    float f = h / 60.0f;
    const float hi = floorf(f);
    f = f - hi;
    const float p = v * (1 - s);
    const float q = v * (1 - s * f);
    const float t = v * (1 - s * (1 - f));
    if (hi == 0.0f || hi == 6.0f) return f3(v, t, p);
    if (hi == 1.0f) return f3(q, v, p);
    if (hi == 2.0f) return f3(p, v, t);
    if (hi == 3.0f) return f3(p, q, v);
    if (hi == 4.0f) return f3(t, p, v);
    return f3(v, p, q);
}

__global__ void kRenderVertices(const float* __restrict__ pos, const float* __restrict__ nrm,
                                const uint8_t* __restrict__ vflags, const int* __restrict__ vertexHE, int numVertices,
                                float* __restrict__ out) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= numVertices) return;
    float* o = out + 10 * (int64_t)v;
    if (vertexHE[v] < 0) {  // no halfedge writes it: the default Vertex (Mesh.h:15-19)
        for (int a = 0; a < 6; ++a) o[a] = __int_as_float(0x7fc00000);
        o[6] = 1.f;
        o[7] = 0.f;
        o[8] = 1.f;
        o[9] = 1.f;
        return;
    }
    const uint32_t fl = vflags[v];
    const bool nm = fl & MDMC_VERTEX_NON_MANIFOLD, weird = fl & MDMC_VERTEX_WEIRD, fans = fl & MDMC_VERTEX_MULTIPLE_FANS;
    float hue = 180.f;
    if (nm) hue = 0.f;
    if (weird) hue = 60.f;
    if (fans) hue = 270.f;
    if (weird && nm) hue = 300.f;
    if (nm && fans) hue = 240.f;
    const F3 c = hsvToRgb(hue, 0.8f, 0.8f);
    for (int a = 0; a < 3; ++a) {
        o[a] = pos[3 * (int64_t)v + a];
        o[3 + a] = nrm[3 * (int64_t)v + a];
    }
    o[6] = c.x;
    o[7] = c.y;
    o[8] = c.z;
    o[9] = 1.f;
}

__global__ void kRenderIndices(const int4* __restrict__ quads, int numFaces, uint32_t* __restrict__ out) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= numFaces) return;
    const int4 q = quads[f];
    uint32_t* o = out + 6 * (int64_t)f;
    o[0] = (uint32_t)q.x;
    o[1] = (uint32_t)q.y;
    o[2] = (uint32_t)q.z;
    o[3] = (uint32_t)q.z;
    o[4] = (uint32_t)q.w;
    o[5] = (uint32_t)q.x;
}

void launchRenderBuffers(const float* pos, const float* nrm, const uint8_t* vflags, const int* vertexHE, int numVertices,
                         const int4* quads, int numFaces, float* vertices, uint32_t* indices, cudaStream_t s) {
    if (vertices && numVertices > 0) {
        countLaunch();
        kRenderVertices<<<(numVertices + 255) / 256, 256, 0, s>>>(pos, nrm, vflags, vertexHE, numVertices, vertices);
    }
    if (indices && numFaces > 0) {
        countLaunch();
        kRenderIndices<<<(numFaces + 255) / 256, 256, 0, s>>>(quads, numFaces, indices);
    }
}

}  // namespace mdmc
