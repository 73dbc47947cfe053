// Kernel launchers of the library (one stream per call, no host syncs).
#pragma once

#include <cuda_runtime.h>

#include "mdmc_device.cuh"
#include "mdmc_types.h"

#include <atomic>

namespace mdmc {

// kernels launched by this library in the process (read per run for stats)
extern std::atomic<long long> g_kernelLaunches;
inline void countLaunch(int n = 1) { g_kernelLaunches.fetch_add(n, std::memory_order_relaxed); }

__device__ __forceinline__ void setTwinOut(int4* he, int h, int t) { reinterpret_cast<int*>(he)[4 * (int64_t)h + 3] = t; }

// packed 16-bit face attributes / 8-bit vertex flags, or-ed through 32-bit words
// (the arrays are padded to a multiple of 4 bytes)
__device__ __forceinline__ void orFaceAttr(uint16_t* attr, int f, uint32_t bits) {
    atomicOr(reinterpret_cast<uint32_t*>(attr) + (f >> 1), bits << ((f & 1) * 16));
}
__device__ __forceinline__ void orVertexFlag(uint8_t* flags, int v, uint32_t bits) {
    atomicOr(reinterpret_cast<uint32_t*>(flags) + (v >> 2), bits << ((v & 3) * 8));
}

// warp-wide sum added to *dst by lane 0 when non-zero (every lane of the warp
// must call it); no block barrier, so warps of uneven length do not wait for
// one another
template <typename T>
__device__ __forceinline__ void warpAddTo(unsigned long long* dst, T v) {
    unsigned long long w = (unsigned long long)v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
    if ((threadIdx.x & 31) == 0 && w) atomicAdd(dst, w);
}

// Counters packed into one word (16 bits each, sums per block below 2^16),
// added over the block with two barriers; thread 0 then passes the block's
// packed total to add(total).  Every thread of the block must call it.
template <class Add>
__device__ __forceinline__ void blockAddPacked(unsigned long long packed, Add add) {
    __shared__ unsigned long long acc;
    if (threadIdx.x == 0) acc = 0;
    __syncthreads();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) packed += __shfl_down_sync(0xffffffffu, packed, o);
    if ((threadIdx.x & 31) == 0 && packed) atomicAdd(&acc, packed);
    __syncthreads();
    if (threadIdx.x == 0 && acc) add(acc);
}

template <typename T>
__device__ __forceinline__ void blockAddTo(unsigned long long* dst, T v) {
    __shared__ unsigned long long acc;
    if (threadIdx.x == 0) acc = 0;
    __syncthreads();
    unsigned long long w = (unsigned long long)v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
    if ((threadIdx.x & 31) == 0 && w) atomicAdd(&acc, w);
    __syncthreads();
    if (threadIdx.x == 0 && acc) atomicAdd(dst, acc);
}

// the grid a run reads: dense, or refined/padded on demand from a coarse grid
struct GridDesc {
    bool refined;
    PlainView plain;
    RefinedView ref;
    const GridGeom& geom() const { return refined ? static_cast<const GridGeom&>(ref) : static_cast<const GridGeom&>(plain); }
};

// the divisors of both views, once their dims are set
inline void setDivisors(GridDesc& d) {
    const FastDiv dx((uint32_t)d.plain.X), dy((uint32_t)d.plain.Y);
    d.plain.divX = d.ref.divX = dx;
    d.plain.divY = d.ref.divY = dy;
    d.ref.divCX1 = FastDiv((uint32_t)(d.ref.cX > 1 ? d.ref.cX - 1 : 1));
    d.ref.divCY1 = FastDiv((uint32_t)(d.ref.cY > 1 ? d.ref.cY - 1 : 1));
}

// the (sorted) ids of one edge bucket with four or more halfedges, as listed
// in the non-manifold edge list
struct NMIds {
    int ids[4];
    __device__ __forceinline__ explicit NMIds(int4 q) {
        ids[0] = q.x;
        ids[1] = q.y;
        ids[2] = q.z;
        ids[3] = q.w;
    }
};

// splitter working copies (device pointers)
struct SplitWork {
    float* pos;
    float* nrm;
    uint32_t* vfl;
    uint32_t* hfl;
    uint32_t* ffl;
    int* vC2O;
    int* hC2O;
    int* fC2O;
    int* vO2C;  // dense over the mesh's vertices, 0x7FFFFFFF = none
    int* hO2C;  // dense over halfedges, -1 = none
    int* fO2C;  // dense over faces, -1 = none
    int* origV;
    int* origH;
    int4* he;
    int* first;
    uint16_t* attr;
    int* vNum;
    int* vSlots;
    int* hNum;
    int* hSlots;
    // sizes: copies (nv, nh, nf) and the mesh (V, H, F)
    int nv, nh, nf;
    int V, H, F;
    // DMC vertex each appended mesh vertex descends from (index o - dmcV)
    int* appParent;
    int dmcV;
    // copies below this id are the faces' corners (4n with subdivision, nv
    // without); flags[0] is set when a merge partner is a corner
    int cornerLimit;
    int* flags;
    // optional: marks the DMC vertices (ids below dmcV) that are corners of
    // a copied face, i.e. whose fans the splitter may change
    uint8_t* touched;
    // per copy halfedge: the last merge pair's twin offer (kMergeHalfedges)
    unsigned long long* hTwinBest;
};

void launchRefine(const float* in, int3 din, float* out, int3 dout, int r, int pad, cudaStream_t s);
void launchCoarseMayCross(const RefinedView& g, float iso, uint32_t* bits, cudaStream_t s);
// also appends the candidate coarse cells to list (count in *listCount)
void launchCoarseMayCross(const RefinedView& g, float iso, uint32_t* bits, uint32_t* list, unsigned long long* listCount,
                          cudaStream_t s);
// The case byte of every cell the mask pass classifies, left for the emit
// pass so that it need not evaluate the corners of cells whose case has a
// table entry.  mode 0: none; 1: a plain grid, p[linear id of the cell's
// corner-0 sample]; 2: a grid refined x4 without padding (standard 4x4x4
// blocks of the block mask), p[coarse cell * 64 + (z & 3) * 16 + (y & 3) * 4 + (x & 3)].
struct CaseBytes {
    uint8_t* p = nullptr;
    int mode = 0;
};
void launchBlockMask(const RefinedView& g, float iso, const uint32_t* list, const unsigned long long* listCount,
                     uint32_t* mask, int W, CaseBytes cases, uint32_t* status, cudaStream_t s);
void launchRowCount(const GridDesc& g, float iso, int4* rowCounts, int numRows, cudaStream_t s);
void launchRowMask(const GridDesc& g, float iso, uint32_t* mask, int numRows, int W, CaseBytes cases, cudaStream_t s);
// exclusive scan of the mask words' popcounts into first (numWords + 1
// entries) that also writes the active cells' ids, the first `capacity` of them
bool scanMaskScatter(const uint32_t* mask, int* first, int64_t numWords, int W, int X, int Y, uint32_t* cellIds,
                     int64_t capacity, int* scratch, cudaStream_t s);
void launchScatterCells(const uint32_t* mask, const int* first, int64_t numWords, int W, int X, int Y, uint32_t* cellIds,
                        int numActive, uint32_t* status, cudaStream_t s);
// numActiveDev != nullptr: the count is read on the device, at most numActive
void launchEmitActive(const GridDesc& g, float iso, const uint32_t* cellIds, ActiveCell* act, int2* counts,
                      int numActive, CaseBytes cases, uint32_t* status, cudaStream_t s,
                      const int* numActiveDev = nullptr);
// exclusive scan of the active cells' (vertex, quad) counts (capA + 1
// entries, the count read from numActiveDev when given) into each record's
// first vertex and quad id, the quad owners (the first capQ) and
// gathered[0..2] = active cells, vertices, quads (-1, -1 for the last two
// when the active cells exceed capA); of counts only counts[n], the total,
// is rewritten
bool scanCellCounts(int2* counts, int64_t capA, const int* numActiveDev, ActiveCell* act, int* quadOwner, int64_t capQ,
                    int* gathered, int* gatheredHost, int2* scratch, cudaStream_t s);
// standard Marching Cubes (edge mask over global edge ids 3 * sample + axis,
// W3 words per sample row)
void launchMCMarkEdges(const GridDesc& g, float iso, const uint32_t* cellIds, int numActive, int W3, uint32_t* edgeMask,
                       uint8_t* cases, int* triCount, uint32_t* status, cudaStream_t s);
void launchMCScatterEdges(const uint32_t* edgeMask, const int* first, int64_t numWords, int W3, int X, uint32_t* edgeIds,
                          int numVertices, uint32_t* status, cudaStream_t s);
void launchMCVertices(const GridDesc& g, float iso, const uint32_t* edgeIds, int numVertices, float* pos, float* nrm,
                      cudaStream_t s);
void launchMCTriangles(const uint32_t* cellIds, const uint8_t* cases, const int* triOffset, int numActive, int X, int Y,
                       int W3, const uint32_t* edgeMask, const int* edgeFirst, int64_t numWords, int* tris,
                       int numTriangles, uint32_t* status, cudaStream_t s);
// Counts a pass reads on the device, for launches made before the host has
// read them back: dev -> {active cells, vertices, quads} (the gathered
// counts), valid only when all three fit the capacities the launch covers.
// A pass given one does nothing when the counts do not fit; the host, which
// reads the same counts, then launches it again at the right size.
struct DeviceCounts {
    const int* dev;
    int capA, capV, capQ;
    __device__ __forceinline__ bool fits(int& a, int& v, int& q) const {
        a = dev[0];
        v = dev[1];
        q = dev[2];
        return a >= 0 && a <= capA && v >= 0 && v <= capV && q >= 0 && q <= capQ;
    }
    bool fits(int64_t a, int64_t v, int64_t q) const {
        return a >= 0 && a <= capA && v >= 0 && v <= capV && q >= 0 && q <= capQ;
    }
};

// degree[v] = the number of quads around DMC vertex v, negated unless every
// edge of its contour has a quad and no face of its cell has four crossing
// edges (then its faces are known to form one fan; see kFanFast)
// flagsInit, starInit (optional): vertex flags set to 0 and smallest
// outgoing halfedges to "none" (0x7F7F7F7F), the quad pass's starting values
void launchVertices(const GridDesc& g, float iso, int surfaceIteration, const ActiveCell* act, int numActive,
                    int numVertices, float* pos, float* nrm, int* degree, uint8_t* flagsInit, int* starInit,
                    uint32_t* status, cudaStream_t s, const DeviceCounts* counts = nullptr);
void launchQuads(const ActiveCell* act, const int* quadOwner, int numActive, const uint32_t* cellMask,
                 const int* cellFirst, int X, int Y, int Z, int W, int4* he, int* faceFirst, uint16_t* faceAttr,
                 uint8_t* vflags, uint8_t* heValence, int4* nmList, int nmCapacity, int numQuads, int numVertices,
                 int4* quadsOut, int* vertexHE, DevCounters* ctr, int qBegin, int qEnd,
                 cudaStream_t s);
void launchVertexHalfedgeFix(int* vertexHE, int numVertices, cudaStream_t s);

// edge buckets: rows of halfedges keyed by their smaller end vertex
// (deg: per vertex, the halfedges whose smaller end it is)
void launchEdgeRowDegree(const int4* he, MeshDims md, int* deg, int* rank, uint32_t* status, cudaStream_t s);
// faceNM (one byte per face): the face's edges with more than two halfedges
// (low nibble) and with exactly four (high nibble).  vcount (optional, one
// word per vertex): how many of the vertex's outgoing halfedges lie on edges
// of one (bits 0-9), three (10-19) and four (20-29) halfedges.
constexpr uint32_t kFaceNMCount = 0x0Fu;
constexpr int kVCountShiftBoundary = 0, kVCountShiftWeird = 10, kVCountShiftNM = 20;
void launchEdgeBuckets(int4* he, MeshDims md, const int* rowStart, const int* rank, int2* adj, int connectTwins,
                       uint16_t* faceAttr, uint8_t* vflags, uint8_t* faceNM, uint32_t* vcount, int4* nmList,
                       DevCounters* ctr, cudaStream_t s);
void launchResetFaceFlags(uint16_t* attr, int numFaces, cudaStream_t s);
void launchReconnect(const GridDesc& g, float iso, const int4* nmList, const DevCounters* ctr,
                     int4* he, const float* pos, MeshDims md, uint32_t* status, cudaStream_t s);
// vertexPassDegrees: deg is the vertex pass's signed degree of the DMC mesh
// (only the twin repair has run since); otherwise non-negative degrees.
// isKey[h] == keyMark marks this pass's fan keys (no other entry may hold it)
// (gate: when given and non-zero, the pass does nothing: the fan-slow count
// stays zero, so the later fan passes do nothing either)
// (dmcDeg, touched, dmcV: optional; after the splitter, a DMC vertex it did
// not touch whose vertex-pass degree was positive still has one closed fan)
void launchDetectFans(const int4* he, MeshDims md, int* vertexHE, const int* deg, bool vertexPassDegrees,
                      uint8_t* slow, uint8_t* isKey, uint8_t keyMark, int* fans, uint8_t* vflags, DevCounters* ctr,
                      uint32_t* status, const unsigned long long* gate, const int* dmcDeg, const uint8_t* touched,
                      int dmcV, cudaStream_t s);
// output quads, quads_with_non_manifold_edges and the vertex stars
// (smallest outgoing halfedge into vertexHE, 0x7F7F7F7F for none; the
// out-degree into deg when given) from one walk per face.  With touched
// (after the splitter): the stars of DMC vertices (below dmcV) it did not
// touch are left as the quad pass wrote them, and their deg is not written.
void launchOutput(const int4* he, const int* faceFirst, MeshDims md, const uint8_t* heValence, const uint8_t* faceNM,
                  int4* quads, int* vertexHE, int* deg, const uint8_t* touched, int dmcV, DevCounters* ctr,
                  uint32_t* status, cudaStream_t s);

// valence-pattern simplifications
void launchValence(const int4* he, MeshDims md, int* val, cudaStream_t s);
void launchSimplify3X3Y(const int4* he, const int* faceFirst, MeshDims md, const int* val, int color, uint16_t* attr,
                        int* count, int4* merge, int* claimA, int* claimC, float* pos, float* nrm, int* type,
                        int* target, uint32_t* status, cudaStream_t s);
void launchSimplify3333(const int4* he, const int* faceFirst, MeshDims md, const int* val, uint16_t* attr, int* type,
                        int* target, cudaStream_t s);
void launchKeepFlags(const int* type, int removedType, int numVertices, int* keepV, const uint16_t* attr, int numFaces,
                     int* keepF, cudaStream_t s);
void launchCompactMesh(const int4* he, const int* faceFirst, MeshDims md, const uint16_t* attr, const int* type,
                       const int* target, int removedType, int remapPattern, const int* vAddr, const int* fAddr,
                       int newVertices, const float* pos, const float* nrm, float* pos2, float* nrm2, int4* quads,
                       uint16_t* attr2, uint32_t* status, cudaStream_t s);
void launchCollectHalfedges(const int4* quads, const uint16_t* attr2, int numFaces, int4* he, int* faceFirst,
                            uint16_t* attr, cudaStream_t s);

// adjoint of the vertex positions (surface iteration off)
void launchGatherParents(const float* dlDpos, int numVertices, int dmcVertices, const int* appParent, float* vertexGrad,
                         cudaStream_t s);
void launchBackwardCells(const GridDesc& g, float iso, const ActiveCell* act, int numActive, const float* vertexGrad,
                         int dmcVertices, float* dlDsamples, uint32_t* status, cudaStream_t s);

void launchRenderBuffers(const float* pos, const float* nrm, const uint8_t* vflags, const int* vertexHE, int numVertices,
                         const int4* quads, int numFaces, float* vertices, uint32_t* indices, cudaStream_t s);

// face coloring 24 -> 5 colors in place (orig: one byte per face of scratch)
void launchColorFaces(const int4* he, const int* faceFirst, uint16_t* attr, uint8_t* orig, int numFaces, int numHalfedges,
                      cudaStream_t s);
// the number of non-manifold faces into offsets[numFaces] (the per-face
// prefixes are not written) and the flagged face ids, ascending, into nmFaces
// (capacity numFaces); false when numFaces is beyond the scan's size
bool scanNMFaces(const uint16_t* attr, int numFaces, int* offsets, int* nmFaces, int* scratch, cudaStream_t s);
// exclusive prefix of "kept and without an original" over count copy
// elements into offsets (count + 1 entries); with assignBase >= 0 instead
// each such element's c2o entry becomes assignBase + its number (the
// halfedges' new ids, before the copy-back) and only offsets[count], the
// total, is written
bool scanAppends(const uint32_t* fl, int* c2o, int count, int* offsets, int* scratch, cudaStream_t s,
                 int assignBase = -1);
void launchFillInt(int* p, int64_t n, int v, cudaStream_t s);
void launchSplitCopy(const int* nmFaces, int n, const int4* he, const int* faceFirst, const uint16_t* faceAttr,
                     const float* pos, const float* nrm, const SplitWork& w, uint32_t* status, cudaStream_t s);
void launchSplitMarkNM(const int4* nmList, const DevCounters* ctr, const SplitWork& w,
                       uint32_t* status, cudaStream_t s);
void launchSplitSubdivide(int n, const SplitWork& w, uint32_t* status, cudaStream_t s);
void launchSplitCollapse(const SplitWork& w, uint32_t* status, cudaStream_t s);
void launchSplitMerge(const SplitWork& w, uint32_t* status, cudaStream_t s);
void launchSplitMergeHalfedges(const SplitWork& w, uint32_t* status, cudaStream_t s);
void launchSplitMove(const GridDesc& g, float iso, const SplitWork& w, cudaStream_t s);
void launchSplitCopyBack(const SplitWork& w, const int* appV, const int* appH, const int* appF, int V2, int H2, int F2,
                         float* pos, float* nrm, int4* he, int* faceFirst, uint16_t* faceAttr, uint32_t* status,
                         cudaStream_t s);
void launchSplitResetMaps(int n, const int* nmFaces, const SplitWork& w, cudaStream_t s);

// Local refresh after a splitter iteration (see mdmc_split.cu).  One record
// per halfedge of an edge whose two ends are in the iteration's vertex set.
struct CensusRec {
    int lo, hi;      // the edge's end vertices, lo < hi
    int h;           // halfedge id
    int origin;      // its origin vertex
    int face;        // its face
    int slot;        // its edge's slot in the census table
};
struct CensusTable {
    unsigned long long* keys;  // lo << 32 | hi, ~0 = empty
    int* count;                // halfedges of the edge
    int* claim;                // set by the record that settles the edge
    int* members;              // the edge's first four halfedge ids
    int capacity;              // a power of two
};
// over the iteration's distinct corners: out[0] += halfedges of the old
// mesh between two vertices of the set, out[1] += those the copy-back keeps
void launchCensusCountOld(const SplitWork& w, int n, const int* rowStart, const int2* adj, const int4* he, int* out,
                          cudaStream_t s);
// their records, into oldRecs and (the kept ones) newRecs; fill[0], fill[1]
// count them (records past a capacity are dropped, the count still grows)
void launchCensusCollectOld(const SplitWork& w, int n, const int* rowStart, const int2* adj, const int4* he,
                            CensusRec* oldRecs, CensusRec* newRecs, int* fill, int capOld, int capNew, uint32_t* status,
                            cudaStream_t s);
// the written-back halfedges' records (after the copy-back), counted by fill[1]
void launchCensusCollectNew(const SplitWork& w, const int4* he, MeshDims md, CensusRec* newRecs, int* fill, int capNew,
                            uint32_t* status, cudaStream_t s);
// counts out (sign -1) or in (+1) the edges of the first min(*fill, cap) records
void launchCensusApply(CensusRec* recs, const int* fill, int cap, const CensusTable& t, int sign, uint32_t* vcount,
                       uint8_t* faceNM, int4* nmList, int nmCapacity, DevCounters* ctr, cudaStream_t s);
// vertex flags and face flags of the records' vertices and faces from their counts
void launchCensusFinish(const CensusRec* recs, const int* fill, int cap, const uint32_t* vcount, const uint8_t* faceNM,
                        uint8_t* vflags, uint16_t* faceAttr, cudaStream_t s);

}  // namespace mdmc
