// C ABI of the library and the host-side orchestration of one run.
//
// Reference: DualMarchingCubes::run and runPostProcesses
// (D/DualMarchingCubes.cu:220-380), ManifoldSplitter::run
// (D/PostProcesses/ManifoldSplitter.cu:96-208), UniformGridHost::readFromFile
// (D/UniformGrid.inl:512-608), Mesh::writeToFile (D/Mesh.cu:446-510).
//
// Buffers are grow-only and owned by the context, so repeated runs on one
// context allocate nothing once the sizes have been seen.  A run reads back
// the row-count totals once (to size its outputs), one count per splitter
// iteration (as the reference's count_if loop does) and the counters at the
// end.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "mdmc.h"
#include "mdmc_kernels.h"
#include "mdmc_scan.cuh"

namespace mdmc {

std::atomic<long long> g_kernelLaunches{0};

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    template <typename T>
    T* as() const {
        return static_cast<T*>(p);
    }
    // grows without keeping the contents
    cudaError_t ensure(size_t need) {
        if (need <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        size_t nb = std::max<size_t>(need + need / 4, 256);
        cudaError_t e = cudaMalloc(&p, nb);
        if (e == cudaSuccess) bytes = nb;
        return e;
    }
    // grows and keeps the first `keep` bytes
    cudaError_t grow(size_t need, size_t keep, cudaStream_t s) {
        if (need <= bytes) return cudaSuccess;
        void* q = nullptr;
        size_t nb = std::max<size_t>(need + need / 2, 256);
        cudaError_t e = cudaMalloc(&q, nb);
        if (e != cudaSuccess) return e;
        if (p && keep) cudaMemcpyAsync(q, p, std::min(keep, bytes), cudaMemcpyDeviceToDevice, s);
        if (p) {
            cudaStreamSynchronize(s);
            cudaFree(p);
        }
        p = q;
        bytes = nb;
        return cudaSuccess;
    }
};

static inline size_t roundUp(size_t x, size_t a) { return (x + a - 1) / a * a; }

// quad ranges of mdmc_run_to_host (each range's arrays are copied out as soon
// as the quad pass has written them).  Each copy costs the link some time of
// its own: on the 512^3-cell headline grid 16 ranges took 1.27 ms end to end,
// 8 ranges 1.22, 4 ranges 1.20 and 2 ranges 1.20.
constexpr int kCopyRanges = 4;

}  // namespace mdmc

using namespace mdmc;

struct mdmc_context {
    mdmc_options opt;
    std::string err;
    // grid preparation
    DevBuf gridBuf, stageBuf, mayCross, candidates;
    // DMC stage
    DevBuf scanScratch, act;
    // mesh
    DevBuf pos, nrm, he, faceFirst, faceAttr, vflags, vertexHE, quads;
    int64_t V = 0, F = 0, H = 0;
    // differentiable path: the last run's grid, iso, DMC vertex and active-cell
    // counts, and the parents of the vertices the splitter appended
    mdmc_grid lastGrid{};
    float lastIso = 0.f;
    int lastSurfaceIteration = 1;
    int64_t dmcV = 0, activeCells = 0;
    DevBuf appParent, vertexGrad;
    bool simplified = false;  // a simplification renumbered the DMC vertices
    // simplification scratch
    DevBuf sVal, sCount, sType, sTarget, sClaimA, sClaimC, sMerge, sKeepV, sKeepF, sPos, sNrm, sQuads, sAttr;
    // edge buckets: per-vertex adjacency rows (destination, halfedge), the
    // 4-face edge list, per-halfedge valence
    DevBuf adjRow, adjRank, adj, nmList, heValence, faceNM;
    DevBuf caseBytes;  // the mask pass's per-cell cases for the emit pass
    int caseMode = 0;  // CaseBytes::mode of the last mask pass
    bool faceNMValid = false;  // faceNM holds the current mesh's per-face counts (else heValence)
    // per-vertex member counts (vcount) and rows that a full refresh left for
    // the current mesh; the splitter's local refresh needs both
    DevBuf vcount;
    bool rowsValid = false;
    // local refresh: records of the old and new edge sets and their tables
    DevBuf censusFill, censusOld, censusNew, censusTabOld, censusTabNew;
    // quad -> owner cell; per-row active-cell mask (32 cells per word) and the
    // index of each word's first active cell; per active cell {contours, quads}
    DevBuf quadOwner, cellMask, cellFirst, cellCounts, cellIds;
    // counters
    DevBuf counters;
    DevCounters* hostCounters = nullptr;  // pinned
    int32_t* hostInts = nullptr;          // pinned scratch for small reads
    int32_t* hostIntsDev = nullptr;       // hostInts as kernels address it (nullptr: not mapped)
    // splitter
    DevBuf nmOffsets, nmFaces;
    DevBuf wPos, wNrm, wVfl, wHfl, wFfl, wVC2O, wHC2O, wFC2O, wOrigV, wOrigH, wHe, wFirst, wAttr, wVNum, wVSlots,
        wHNum, wHSlots;
    DevBuf vO2C, hO2C, fO2C, splitFlags, wHTwin;
    size_t vO2CCount = 0, hO2CCount = 0, fO2CCount = 0;
    DevBuf appV, appH, appF;
    // fan detection
    DevBuf isKey, fans, degree, slowFan;
    // the vertex pass's degrees kept through the splitter, and its marks of
    // the DMC vertices whose fans it may change (fastFans: both valid)
    DevBuf dmcDegree, splitTouched;
    bool fastFans = false;
    uint8_t keyMark = 0;  // the last detection pass's fan-key mark (1..255, 0 = none yet)
    // standard Marching Cubes: edge mask and the index of each word's first
    // edge, per active cell its case and triangle offset, the vertices' edge
    // ids, and the triangle mesh
    DevBuf mcEdgeMask, mcEdgeFirst, mcCases, mcTriOffset, mcEdgeIds, mcPos, mcNrm, mcTris;
    // face coloring scratch
    DevBuf colorOrig;
    // mdmc_run_to_host: the caller's host arrays during the call, a copy
    // stream whose copies overlap the later stages, and which arrays went
    // out early; lateChange = a stage after the quad pass rewrote the mesh
    const mdmc_host_mesh* hostOut = nullptr;
    cudaStream_t copyStream = nullptr;
    cudaEvent_t copyEv[2] = {};
    bool earlyFaces = false, earlyVertices = false, earlyVertexMaps = false, lateChange = false;
    int64_t mcV = 0, mcT = 0;
    // events: start, dmc, halfedge, repair, detect, end
    cudaEvent_t ev[6] = {};
    int evAt[6] = {0, 1, 2, 3, 4, 5};  // the event that marks stage boundary k
    // per-kernel events: refine, count, emit, quads, table, vertices (begin/end each)
    cudaEvent_t kev[12] = {};
    uint32_t kernelTiming = MDMC_TIME_STAGES;  // MDMC_TIME_* bits: what gets event records
    cudaEvent_t countsEv = nullptr;  // the DMC counts have reached the host
    float msRefine = 0.f;
    bool haveMesh = false;
    mdmc_stats stats;
};

namespace {

// stage boundary k (ev[k]); when nothing ran since boundary k - 1 the
// previous boundary's event stands for it (an event record costs ~1.7 us)
inline void markStage(mdmc_context* c, int k, bool ran, cudaStream_t s) {
    if (!(c->kernelTiming & MDMC_TIME_STAGES)) return;
    if (ran || k == 0) {
        cudaEventRecord(c->ev[k], s);
        c->evAt[k] = k;
    } else {
        c->evAt[k] = c->evAt[k - 1];
    }
}

// kev[2k], kev[2k + 1] bracket timed kernel k (bit k of MDMC_TIME_*): an
// event record costs the stream about 1.7 us, so only requested pairs are made
inline void markKernel(mdmc_context* c, int e, cudaStream_t s) {
    if ((c->kernelTiming >> (e >> 1)) & 1u) cudaEventRecord(c->kev[e], s);
}

mdmc_status fail(mdmc_context* c, mdmc_status st, const std::string& msg) {
    if (c) c->err = msg;
    return st;
}

mdmc_status cudaFail(mdmc_context* c, cudaError_t e, const char* where) {
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    return fail(c, e == cudaErrorMemoryAllocation ? MDMC_ERROR_OUT_OF_MEMORY : MDMC_ERROR_CUDA, m);
}

#define MDMC_CHECK(ctx, expr)                              \
    do {                                                   \
        cudaError_t e_ = (expr);                           \
        if (e_ != cudaSuccess) return cudaFail(ctx, e_, #expr); \
    } while (0)

void defaultOptions(mdmc_options* o) {
    o->enable_surface_to_vertex_iteration = 1;
    o->simplify_p3x3y_color = 0;
    o->simplify_p3x3y_old = 0;
    o->simplify_p3333 = 0;
    o->split_non_manifold_halfedges = 1;
    o->detect_non_manifold_vertices = 1;
    o->splitting_step = MDMC_STEP_ALL;
}

std::string statusText(uint32_t s) {
    std::string t;
    auto add = [&](uint32_t bit, const char* name) {
        if (s & bit) t += std::string(t.empty() ? "" : ", ") + name;
    };
    add(kStatusProbeLimit, "edge table probe limit");
    add(kStatusSlotConflict, "quad slot conflict");
    add(kStatusBucketOverflow, "more than four faces on an edge");
    add(kStatusPartnerOverflow, "merge partner overflow");
    add(kStatusWalkLimit, "face-fan walk limit");
    add(kStatusBadTwin, "non-manifold twin outside the working copy");
    add(kStatusIterationCap, "splitter iteration cap");
    add(kStatusWallOutOfGrid, "cell wall outside the grid");
    add(kStatusMissingCell, "quad neighbour cell missing");
    add(kStatusMappingSwap, "unexpected working-copy mapping");
    add(kStatusCountMismatch, "emit pass disagreed with the count pass");
    add(kStatusBadIndex, "element id out of range");
    add(kStatusCountOverflow, "vertex edge-count field overflow");
    return t;
}

template <typename T>
mdmc_status scan(mdmc_context* c, const T* in, T* out, int64_t n, cudaStream_t s) {
    MDMC_CHECK(c, c->scanScratch.ensure(sizeof(int4) * (size_t)scanScratchElems(n)));
    if (!exclusiveScan<T>(in, out, n, c->scanScratch.as<T>(), s))
        return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "prefix sum input too large");
    return MDMC_OK;
}

// index of every mask word's first set bit among all set bits (out has n + 1
// entries, out[n] = all set bits)
mdmc_status scanPopc(mdmc_context* c, const uint32_t* mask, int* out, int64_t n, cudaStream_t s) {
    MDMC_CHECK(c, c->scanScratch.ensure(sizeof(int4) * (size_t)scanScratchElems(n)));
    if (!exclusiveScanPopc(mask, out, n, c->scanScratch.as<int>(), s))
        return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "prefix sum input too large");
    return MDMC_OK;
}

// reads n int32 values from device memory (synchronizes the stream)
mdmc_status readInts(mdmc_context* c, const void* src, int n, cudaStream_t s) {
    MDMC_CHECK(c, cudaMemcpyAsync(c->hostInts, src, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
    MDMC_CHECK(c, cudaStreamSynchronize(s));
    return MDMC_OK;
}


// the view of a grid the kernels read; refined grids get their coarse-cell
// pre-pass for this iso-value (mayCross bits in the context)
mdmc_status makeGridDesc(mdmc_context* c, const mdmc_grid* grid, float iso, GridDesc& d, cudaStream_t s,
                         bool prepass = true) {
    GridGeom geom;
    geom.X = grid->dims[0];
    geom.Y = grid->dims[1];
    geom.Z = grid->dims[2];
    geom.ox = grid->origin[0];
    geom.oy = grid->origin[1];
    geom.oz = grid->origin[2];
    geom.dx = grid->spacing[0];
    geom.dy = grid->spacing[1];
    geom.dz = grid->spacing[2];
    d.refined = grid->coarse_samples != nullptr && (grid->refinement > 0 || grid->add_zero_boundary);
    static_cast<GridGeom&>(d.plain) = geom;
    static_cast<GridGeom&>(d.ref) = geom;
    d.plain.v = grid->samples;
    d.ref.c = grid->coarse_samples;
    d.ref.cX = grid->coarse_dims[0];
    d.ref.cY = grid->coarse_dims[1];
    d.ref.cZ = grid->coarse_dims[2];
    d.ref.r = grid->refinement;
    d.ref.pad = grid->add_zero_boundary ? 1 : 0;
    d.ref.f = (float)(grid->refinement + 1);
    {
        const int f = grid->refinement + 1;
        d.ref.fPow2 = (f & (f - 1)) == 0 ? 1 : 0;
        d.ref.invf = 1.0f / (float)f;
    }
    setDivisors(d);
    d.ref.mayCross = nullptr;
    if (!d.refined) {
        if (!grid->samples) return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "grid has no samples");
        return MDMC_OK;
    }
    const int pad = d.ref.pad;
    for (int a = 0; a < 3; ++a) {
        const int cd = grid->coarse_dims[a];
        if (cd < 1 || grid->refinement < 0 ||
            (int64_t)cd + (int64_t)(cd - 1) * grid->refinement + 2 * pad != grid->dims[a])
            return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "coarse dims do not match the refined dims");
    }
    if (prepass && d.ref.cX >= 2 && d.ref.cY >= 2 && d.ref.cZ >= 2) {
        const int64_t cells = (int64_t)(d.ref.cX - 1) * (d.ref.cY - 1) * (d.ref.cZ - 1);
        MDMC_CHECK(c, c->mayCross.ensure(sizeof(uint32_t) * (size_t)((cells + 31) / 32 + 1)));
        MDMC_CHECK(c, c->candidates.ensure(sizeof(uint32_t) * (size_t)cells));
        d.ref.mayCross = c->mayCross.as<uint32_t>();
        markKernel(c, 0, s);
        launchCoarseMayCross(d.ref, iso, c->mayCross.as<uint32_t>(), c->candidates.as<uint32_t>(),
                             &c->counters.as<DevCounters>()->candidates, s);
        markKernel(c, 1, s);
    }
    return MDMC_OK;
}

SplitWork splitWork(mdmc_context* c, int nv, int nh, int nf) {
    SplitWork w;
    w.nv = nv;
    w.nh = nh;
    w.nf = nf;
    w.V = (int)c->V;
    w.H = (int)c->H;
    w.F = (int)c->F;
    w.pos = c->wPos.as<float>();
    w.nrm = c->wNrm.as<float>();
    w.vfl = c->wVfl.as<uint32_t>();
    w.hfl = c->wHfl.as<uint32_t>();
    w.ffl = c->wFfl.as<uint32_t>();
    w.vC2O = c->wVC2O.as<int>();
    w.hC2O = c->wHC2O.as<int>();
    w.fC2O = c->wFC2O.as<int>();
    w.vO2C = c->vO2C.as<int>();
    w.hO2C = c->hO2C.as<int>();
    w.fO2C = c->fO2C.as<int>();
    w.origV = c->wOrigV.as<int>();
    w.appParent = c->appParent.as<int>();
    w.dmcV = (int)c->dmcV;
    w.cornerLimit = nv;
    w.flags = c->splitFlags.as<int>();
    w.touched = c->fastFans ? c->splitTouched.as<uint8_t>() : nullptr;
    w.hTwinBest = c->wHTwin.as<unsigned long long>();
    w.origH = c->wOrigH.as<int>();
    w.he = c->wHe.as<int4>();
    w.first = c->wFirst.as<int>();
    w.attr = c->wAttr.as<uint16_t>();
    w.vNum = c->wVNum.as<int>();
    w.vSlots = c->wVSlots.as<int>();
    w.hNum = c->wHNum.as<int>();
    w.hSlots = c->wHSlots.as<int>();
    return w;
}

// dense original->copy maps: sized to the mesh, all "none" between iterations
mdmc_status ensureMaps(mdmc_context* c, cudaStream_t s) {
    if ((size_t)c->V > c->vO2CCount) {
        size_t n = (size_t)c->V * 2;
        MDMC_CHECK(c, c->vO2C.ensure(sizeof(int) * n));
        launchFillInt(c->vO2C.as<int>(), (int64_t)(c->vO2C.bytes / sizeof(int)), 0x7FFFFFFF, s);
        c->vO2CCount = c->vO2C.bytes / sizeof(int);
    }
    if ((size_t)c->H > c->hO2CCount) {
        size_t n = (size_t)c->H * 2;
        MDMC_CHECK(c, c->hO2C.ensure(sizeof(int) * n));
        MDMC_CHECK(c, cudaMemsetAsync(c->hO2C.p, 0xFF, c->hO2C.bytes, s));
        c->hO2CCount = c->hO2C.bytes / sizeof(int);
    }
    if ((size_t)c->F > c->fO2CCount) {
        size_t n = (size_t)c->F * 2;
        MDMC_CHECK(c, c->fO2C.ensure(sizeof(int) * n));
        MDMC_CHECK(c, cudaMemsetAsync(c->fO2C.p, 0xFF, c->fO2C.bytes, s));
        c->fO2CCount = c->fO2C.bytes / sizeof(int);
    }
    return MDMC_OK;
}

// Edge buckets of the current mesh from per-vertex adjacency rows: valences,
// vertex and face flags, edge counters, the 4-face edge list, and (connect)
// the twins of connectHalfedgeTwins (D/Halfedges/HalfedgeMesh.cu:92-291)
mdmc_status edgeBuckets(mdmc_context* c, int connect, cudaStream_t s, bool trackCounts = false) {
    DevCounters* ctr = c->counters.as<DevCounters>();
    const MeshDims md{(int)c->V, (int)c->F, (int)c->H};
    MDMC_CHECK(c, c->nmList.ensure(sizeof(int4) * (size_t)(c->H / 4 + 1)));
    MDMC_CHECK(c, c->faceNM.ensure(roundUp((size_t)std::max<int64_t>(c->F, 1), 4)));
    MDMC_CHECK(c, c->adjRow.ensure(sizeof(int) * (size_t)(c->V + 1)));
    MDMC_CHECK(c, c->adjRank.ensure(sizeof(int) * (size_t)std::max<int64_t>(c->H, 1)));
    MDMC_CHECK(c, c->adj.ensure(sizeof(int2) * (size_t)std::max<int64_t>(c->H, 1)));
    MDMC_CHECK(c, cudaMemsetAsync(c->adjRow.p, 0, sizeof(int) * (size_t)c->V, s));
    launchEdgeRowDegree(c->he.as<int4>(), md, c->adjRow.as<int>(), c->adjRank.as<int>(), &ctr->status, s);
    mdmc_status st = scan<int>(c, c->adjRow.as<int>(), c->adjRow.as<int>(), c->V, s);
    if (st != MDMC_OK) return st;
    MDMC_CHECK(c, cudaMemsetAsync(c->vflags.p, 0, roundUp((size_t)std::max<int64_t>(c->V, 1), 4), s));
    MDMC_CHECK(c, cudaMemsetAsync(c->faceNM.p, 0, roundUp((size_t)std::max<int64_t>(c->F, 1), 4), s));
    MDMC_CHECK(c, cudaMemsetAsync((char*)c->counters.p + 8, 0, sizeof(DevCounters) - 8, s));
    if (trackCounts) {
        MDMC_CHECK(c, c->vcount.ensure(sizeof(uint32_t) * (size_t)std::max<int64_t>(c->V, 1)));
        MDMC_CHECK(c, cudaMemsetAsync(c->vcount.p, 0, sizeof(uint32_t) * (size_t)c->V, s));
    }
    launchEdgeBuckets(c->he.as<int4>(), md, c->adjRow.as<int>(), c->adjRank.as<int>(), c->adj.as<int2>(), connect,
                      c->faceAttr.as<uint16_t>(), c->vflags.as<uint8_t>(), c->faceNM.as<uint8_t>(),
                      trackCounts ? c->vcount.as<uint32_t>() : nullptr, c->nmList.as<int4>(), ctr, s);
    c->faceNMValid = true;
    c->rowsValid = trackCounts;
    return MDMC_OK;
}

// HalfedgeMesh::refreshHashTable, D/Halfedges/HalfedgeMesh.cu:1063-1100: the
// face flags are reset and every bucket and flag recomputed (twins kept)
mdmc_status refreshTable(mdmc_context* c, uint32_t* status, cudaStream_t s) {
    (void)status;
    launchResetFaceFlags(c->faceAttr.as<uint16_t>(), (int)c->F, s);
    return edgeBuckets(c, 0, s, true);
}

// Non-manifold vertex detection (detectNonManifoldVertices,
// D/PostProcesses/ManifoldCreator.cu:488-536) and the outputs (quads by face
// walk, getNumQuadsWithNonManifoldEdges, smallest outgoing halfedge per
// vertex).  starsDone: the quad pass already wrote the vertex stars, quads and
// face statistics of this mesh.  gate: a device counter; when it is non-zero
// the detection does nothing (a speculative pass on a mesh about to change).
mdmc_status finishMesh(mdmc_context* c, bool starsDone, uint32_t* status, cudaStream_t s,
                       const unsigned long long* gate = nullptr) {
    DevCounters* ctr = c->counters.as<DevCounters>();
    const bool detect = c->opt.detect_non_manifold_vertices != 0;
    // after the splitter, with the vertex pass's degrees kept: the DMC
    // vertices it did not touch keep the stars the quad pass wrote
    const bool keepStars = !starsDone && c->fastFans && detect;
    MDMC_CHECK(c, c->vertexHE.grow(sizeof(int) * (size_t)std::max<int64_t>(c->V, 1),
                                   keepStars ? sizeof(int) * (size_t)c->dmcV : 0, s));
    MDMC_CHECK(c, c->degree.ensure(sizeof(int) * (size_t)std::max<int64_t>(c->V, 1)));
    MDMC_CHECK(c, c->quads.ensure(sizeof(int4) * (size_t)std::max<int64_t>(c->F, 1)));
    const MeshDims mdF{(int)c->V, (int)c->F, (int)c->H};
    // a changed mesh: output quads, face statistics and vertex stars in one
    // pass over the faces, before the detection that reads the stars (so the
    // stage times count this pass with the detection)
    if (!starsDone)
        launchOutput(c->he.as<int4>(), c->faceFirst.as<int>(), mdF, c->heValence.as<uint8_t>(),
                     c->faceNMValid ? c->faceNM.as<uint8_t>() : nullptr, c->quads.as<int4>(), c->vertexHE.as<int>(),
                     detect ? c->degree.as<int>() : nullptr, keepStars ? c->splitTouched.as<uint8_t>() : nullptr,
                     (int)c->dmcV, ctr, status, s);
    if (detect) {
        // fan keys are marked with this pass's number (1..255); the array is
        // cleared only when it is new or the numbers wrap around.  (A new
        // array is told by its capacity: a reallocation can return the
        // address just freed, holding another array's old marks.)
        const size_t keyBytes = c->isKey.bytes;
        MDMC_CHECK(c, c->isKey.ensure((size_t)std::max<int64_t>(c->H, 1)));
        if (c->isKey.bytes != keyBytes || c->keyMark == 255) {
            MDMC_CHECK(c, cudaMemsetAsync(c->isKey.p, 0, c->isKey.bytes, s));
            c->keyMark = 0;
        }
        ++c->keyMark;
        MDMC_CHECK(c, c->fans.ensure(sizeof(int) * (size_t)std::max<int64_t>(c->V, 1)));
        MDMC_CHECK(c, c->slowFan.ensure((size_t)std::max<int64_t>(c->V, 1)));
        // (the first pass of a run finds the count zeroed with the counters)
        if (!starsDone) MDMC_CHECK(c, cudaMemsetAsync(&ctr->slowFans, 0, sizeof(unsigned long long), s));
        launchDetectFans(c->he.as<int4>(), mdF, c->vertexHE.as<int>(), c->degree.as<int>(), starsDone,
                         c->slowFan.as<uint8_t>(), c->isKey.as<uint8_t>(), c->keyMark, c->fans.as<int>(),
                         c->vflags.as<uint8_t>(), ctr, status, gate,
                         (!starsDone && c->fastFans) ? c->dmcDegree.as<int>() : nullptr, c->splitTouched.as<uint8_t>(),
                         (int)c->dmcV, s);
    }
    markStage(c, 4, detect, s);
    if (!detect) launchVertexHalfedgeFix(c->vertexHE.as<int>(), (int)c->V, s);  // "none" -> -1
    markStage(c, 5, !detect, s);
    MDMC_CHECK(c, cudaGetLastError());
    return MDMC_OK;
}

// simplify3X3Y (kind 0), simplify3X3YOld (kind 1), simplify3333 (kind 2),
// D/Halfedges/HalfedgeMesh.cu:859-1048: mark and merge, compact the vertex
// and quad lists, rebuild the halfedge mesh from the quads (initialize)
mdmc_status runSimplification(mdmc_context* c, int kind, cudaStream_t s) {
    DevCounters* ctr = c->counters.as<DevCounters>();
    uint32_t* status = &ctr->status;
    const int V = (int)c->V, F = (int)c->F;
    const MeshDims md{V, F, (int)c->H};
    if (V <= 0 || F <= 0) return MDMC_OK;
    MDMC_CHECK(c, c->sVal.ensure(sizeof(int) * (size_t)V));
    MDMC_CHECK(c, c->sCount.ensure(sizeof(int) * (size_t)V));
    MDMC_CHECK(c, c->sType.ensure(sizeof(int) * (size_t)V));
    MDMC_CHECK(c, c->sTarget.ensure(sizeof(int) * (size_t)V));
    MDMC_CHECK(c, c->sClaimA.ensure(sizeof(int) * (size_t)V));
    MDMC_CHECK(c, c->sClaimC.ensure(sizeof(int) * (size_t)V));
    MDMC_CHECK(c, c->sMerge.ensure(sizeof(int4) * (size_t)F));
    MDMC_CHECK(c, c->sKeepV.ensure(sizeof(int) * (size_t)(V + 1)));
    MDMC_CHECK(c, c->sKeepF.ensure(sizeof(int) * (size_t)(F + 1)));
    MDMC_CHECK(c, cudaMemsetAsync(c->sVal.p, 0, sizeof(int) * (size_t)V, s));
    MDMC_CHECK(c, cudaMemsetAsync(c->sCount.p, 0, sizeof(int) * (size_t)V, s));
    MDMC_CHECK(c, cudaMemsetAsync(c->sType.p, 0, sizeof(int) * (size_t)V, s));
    MDMC_CHECK(c, cudaMemsetAsync(c->sTarget.p, 0xFF, sizeof(int) * (size_t)V, s));
    MDMC_CHECK(c, cudaMemsetAsync(c->sClaimA.p, 0xFF, sizeof(int) * (size_t)V, s));
    MDMC_CHECK(c, cudaMemsetAsync(c->sClaimC.p, 0xFF, sizeof(int) * (size_t)V, s));
    launchValence(c->he.as<int4>(), md, c->sVal.as<int>(), s);
    if (kind < 2)
        launchSimplify3X3Y(c->he.as<int4>(), c->faceFirst.as<int>(), md, c->sVal.as<int>(), kind == 0 ? 1 : 0,
                           c->faceAttr.as<uint16_t>(), c->sCount.as<int>(), c->sMerge.as<int4>(), c->sClaimA.as<int>(),
                           c->sClaimC.as<int>(), c->pos.as<float>(), c->nrm.as<float>(), c->sType.as<int>(),
                           c->sTarget.as<int>(), status, s);
    else
        launchSimplify3333(c->he.as<int4>(), c->faceFirst.as<int>(), md, c->sVal.as<int>(), c->faceAttr.as<uint16_t>(),
                           c->sType.as<int>(), c->sTarget.as<int>(), s);
    const int removedType = kind < 2 ? 3 : 1;
    launchKeepFlags(c->sType.as<int>(), removedType, V, c->sKeepV.as<int>(), c->faceAttr.as<uint16_t>(), F,
                    c->sKeepF.as<int>(), s);
    mdmc_status st;
    if ((st = scan<int>(c, c->sKeepV.as<int>(), c->sKeepV.as<int>(), V, s)) != MDMC_OK) return st;
    if ((st = scan<int>(c, c->sKeepF.as<int>(), c->sKeepF.as<int>(), F, s)) != MDMC_OK) return st;
    MDMC_CHECK(c, cudaMemcpyAsync(c->hostInts, c->sKeepV.as<int>() + V, sizeof(int), cudaMemcpyDeviceToHost, s));
    MDMC_CHECK(c, cudaMemcpyAsync(c->hostInts + 1, c->sKeepF.as<int>() + F, sizeof(int), cudaMemcpyDeviceToHost, s));
    MDMC_CHECK(c, cudaStreamSynchronize(s));
    MDMC_CHECK(c, cudaGetLastError());
    const int V2 = c->hostInts[0], F2 = c->hostInts[1];
    if (V2 < 0 || V2 > V || F2 < 0 || F2 > F) return fail(c, MDMC_ERROR_CUDA, "inconsistent simplification counts");
    MDMC_CHECK(c, c->sPos.ensure(sizeof(float) * 3 * (size_t)std::max(V2, 1)));
    MDMC_CHECK(c, c->sNrm.ensure(sizeof(float) * 3 * (size_t)std::max(V2, 1)));
    MDMC_CHECK(c, c->sQuads.ensure(sizeof(int4) * (size_t)std::max(F2, 1)));
    MDMC_CHECK(c, c->sAttr.ensure(roundUp(sizeof(uint16_t) * (size_t)std::max(F2, 1), 4)));
    launchCompactMesh(c->he.as<int4>(), c->faceFirst.as<int>(), md, c->faceAttr.as<uint16_t>(), c->sType.as<int>(),
                      c->sTarget.as<int>(), removedType, kind == 2 ? 1 : 0, c->sKeepV.as<int>(), c->sKeepF.as<int>(), V2,
                      c->pos.as<float>(), c->nrm.as<float>(), c->sPos.as<float>(), c->sNrm.as<float>(),
                      c->sQuads.as<int4>(), c->sAttr.as<uint16_t>(), status, s);
    if (V2 > 0) {
        MDMC_CHECK(c, cudaMemcpyAsync(c->pos.p, c->sPos.p, sizeof(float) * 3 * (size_t)V2, cudaMemcpyDeviceToDevice, s));
        MDMC_CHECK(c, cudaMemcpyAsync(c->nrm.p, c->sNrm.p, sizeof(float) * 3 * (size_t)V2, cudaMemcpyDeviceToDevice, s));
    }
    // HalfedgeMesh::initialize from the reduced quads
    c->V = V2;
    c->F = F2;
    c->H = 4 * (int64_t)F2;
    c->simplified = true;
    launchCollectHalfedges(c->sQuads.as<int4>(), c->sAttr.as<uint16_t>(), F2, c->he.as<int4>(), c->faceFirst.as<int>(),
                           c->faceAttr.as<uint16_t>(), s);
    if ((st = edgeBuckets(c, 1, s)) != MDMC_OK) return st;
    MDMC_CHECK(c, cudaGetLastError());
    return MDMC_OK;
}

// The splitter's local refresh (kCensus* in csrc/mdmc_split.cu): record
// buffers and tables sized from the old edge set (nOld records) and the
// kept one (at most capNew); the old records are taken before the copy-back
// overwrites the old halfedges.
struct Census {
    int capOld = 0, capNew = 0;
    CensusTable tOld{}, tNew{};
};

static int censusTableSize(int records) {
    int p = 1024;
    while (p < 2 * records) p *= 2;
    return p;
}

static CensusTable censusTable(DevBuf& b, int capacity) {
    CensusTable t;
    char* p = (char*)b.p;
    t.capacity = capacity;
    t.keys = (unsigned long long*)p;
    t.count = (int*)(p + 8 * (size_t)capacity);
    t.claim = (int*)(p + 12 * (size_t)capacity);
    t.members = (int*)(p + 16 * (size_t)capacity);
    return t;
}

mdmc_status censusBegin(mdmc_context* c, const SplitWork& w, int n, int nOld, int capNew, Census& k, cudaStream_t s) {
    if (nOld > 0x3FFFFFFF || capNew > 0x3FFFFFFF) return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "local refresh too large");
    k.capOld = nOld;
    k.capNew = capNew;
    const int pOld = censusTableSize(nOld), pNew = censusTableSize(capNew);
    MDMC_CHECK(c, c->censusOld.ensure(sizeof(CensusRec) * (size_t)std::max(nOld, 1)));
    MDMC_CHECK(c, c->censusNew.ensure(sizeof(CensusRec) * (size_t)std::max(capNew, 1)));
    MDMC_CHECK(c, c->censusTabOld.ensure(32 * (size_t)pOld));
    MDMC_CHECK(c, c->censusTabNew.ensure(32 * (size_t)pNew));
    k.tOld = censusTable(c->censusTabOld, pOld);
    k.tNew = censusTable(c->censusTabNew, pNew);
    for (const CensusTable* t : {&k.tOld, &k.tNew}) {
        MDMC_CHECK(c, cudaMemsetAsync(t->keys, 0xFF, 8 * (size_t)t->capacity, s));
        MDMC_CHECK(c, cudaMemsetAsync(t->count, 0, 8 * (size_t)t->capacity, s));  // count and claim
    }
    MDMC_CHECK(c, cudaMemsetAsync(c->censusFill.p, 0, sizeof(int) * 4, s));
    launchCensusCollectOld(w, n, c->adjRow.as<int>(), c->adj.as<int2>(), c->he.as<int4>(), c->censusOld.as<CensusRec>(),
                           c->censusNew.as<CensusRec>(), c->censusFill.as<int>(), k.capOld, k.capNew,
                           &c->counters.as<DevCounters>()->status, s);
    return MDMC_OK;
}

// after the copy-back (c->V/H/F already the new sizes; V1, F1 the old ones):
// the kept halfedges' records, the old edge sets counted out and the new ones
// in, then the flags of every vertex and face the records name
mdmc_status censusFinish(mdmc_context* c, const SplitWork& w, const Census& k, int64_t V1, int64_t F1, cudaStream_t s) {
    DevCounters* ctr = c->counters.as<DevCounters>();
    const MeshDims md{(int)c->V, (int)c->F, (int)c->H};
    // the appended vertices and faces start from zero counts and flags
    MDMC_CHECK(c, c->vcount.grow(sizeof(uint32_t) * (size_t)c->V, sizeof(uint32_t) * (size_t)V1, s));
    MDMC_CHECK(c, cudaMemsetAsync(c->vcount.as<uint32_t>() + V1, 0, sizeof(uint32_t) * (size_t)(c->V - V1), s));
    MDMC_CHECK(c, c->faceNM.grow(roundUp((size_t)c->F, 4), (size_t)F1, s));
    MDMC_CHECK(c, cudaMemsetAsync(c->faceNM.as<uint8_t>() + F1, 0, roundUp((size_t)c->F, 4) - (size_t)F1, s));
    MDMC_CHECK(c, cudaMemsetAsync(c->vflags.as<uint8_t>() + V1, 0, roundUp((size_t)c->V, 4) - (size_t)V1, s));
    MDMC_CHECK(c, c->nmList.grow(sizeof(int4) * (size_t)(c->H / 4 + 1), 0, s));
    // the refresh's other counters start from zero, as after a full refresh
    MDMC_CHECK(c, cudaMemsetAsync(&ctr->nmVertices, 0, sizeof(DevCounters) - offsetof(DevCounters, nmVertices), s));
    launchCensusCollectNew(w, c->he.as<int4>(), md, c->censusNew.as<CensusRec>(), c->censusFill.as<int>(), k.capNew,
                           &ctr->status, s);
    const int* fill = c->censusFill.as<int>();
    launchCensusApply(c->censusOld.as<CensusRec>(), fill, k.capOld, k.tOld, -1, c->vcount.as<uint32_t>(),
                      c->faceNM.as<uint8_t>(), c->nmList.as<int4>(), (int)(c->H / 4 + 1), ctr, s);
    launchCensusApply(c->censusNew.as<CensusRec>(), fill + 1, k.capNew, k.tNew, 1, c->vcount.as<uint32_t>(),
                      c->faceNM.as<uint8_t>(), c->nmList.as<int4>(), (int)(c->H / 4 + 1), ctr, s);
    launchCensusFinish(c->censusOld.as<CensusRec>(), fill, k.capOld, c->vcount.as<uint32_t>(), c->faceNM.as<uint8_t>(),
                       c->vflags.as<uint8_t>(), c->faceAttr.as<uint16_t>(), s);
    launchCensusFinish(c->censusNew.as<CensusRec>(), fill + 1, k.capNew, c->vcount.as<uint32_t>(),
                       c->faceNM.as<uint8_t>(), c->vflags.as<uint8_t>(), c->faceAttr.as<uint16_t>(), s);
    // the new record count must fit what was reserved
    MDMC_CHECK(c, cudaMemcpyAsync(c->hostInts, c->censusFill.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    MDMC_CHECK(c, cudaStreamSynchronize(s));
    if (c->hostInts[0] != k.capOld || c->hostInts[1] < 0 || c->hostInts[1] > k.capNew)
        return fail(c, MDMC_ERROR_CUDA, "local refresh record counts disagree with their sizes");
    MDMC_CHECK(c, cudaGetLastError());
    c->faceNMValid = true;
    c->rowsValid = false;
    return MDMC_OK;
}

// ManifoldSplitter::run, D/PostProcesses/ManifoldSplitter.cu:96-208
mdmc_status runSplitter(mdmc_context* c, const GridDesc& g, float iso, int64_t& iterations, cudaStream_t s) {
    DevCounters* ctr = c->counters.as<DevCounters>();
    uint32_t* status = &ctr->status;
    const int step = c->opt.splitting_step;
    iterations = 0;
    // keep the vertex pass's degrees for the fan detection after the splitter
    // (valid for the DMC mesh as the twin repair left it; not after a
    // simplification renumbered it)
    if (c->opt.detect_non_manifold_vertices && !c->simplified && c->dmcV == c->V) {
        std::swap(c->degree.p, c->dmcDegree.p);
        std::swap(c->degree.bytes, c->dmcDegree.bytes);
        MDMC_CHECK(c, c->splitTouched.ensure((size_t)std::max<int64_t>(c->dmcV, 1)));
        MDMC_CHECK(c, cudaMemsetAsync(c->splitTouched.p, 0, (size_t)c->dmcV, s));
        c->fastFans = c->dmcDegree.bytes >= sizeof(int) * (size_t)c->dmcV;
    }
    while (true) {
        // countNonManifoldFaces + the list of non-manifold faces (one scan)
        MDMC_CHECK(c, c->nmOffsets.ensure(sizeof(int) * (size_t)(c->F + 1)));
        MDMC_CHECK(c, c->nmFaces.ensure(sizeof(int) * (size_t)std::max<int64_t>(c->F, 1)));
        MDMC_CHECK(c, c->scanScratch.ensure(sizeof(int4) * (size_t)scanScratchElems(c->F)));
        if (!scanNMFaces(c->faceAttr.as<uint16_t>(), (int)c->F, c->nmOffsets.as<int>(), c->nmFaces.as<int>(),
                         c->scanScratch.as<int>(), s))
            return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "prefix sum input too large");
        mdmc_status st = MDMC_OK;
        MDMC_CHECK(c, cudaGetLastError());
        if ((st = readInts(c, c->nmOffsets.as<int>() + c->F, 1, s)) != MDMC_OK) return st;
        const int n = (int)c->hostInts[0];
        if (n < 0 || n > c->F) return fail(c, MDMC_ERROR_CUDA, "inconsistent non-manifold face count");
        if (n == 0) break;
        if ((int64_t)c->H + 20 * (int64_t)n >= (int64_t)0x7FFFFFFF)
            return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "splitting would exceed 2^31 halfedges");

        const bool doSub = step >= MDMC_STEP_SUBDIVIDE_QUADS;
        const int nv = 4 * n + (doSub ? 4 * n : 0);
        const int nh = 4 * n + (doSub ? 16 * n : 0);
        const int nf = n + (doSub ? 4 * n : 0);
        MDMC_CHECK(c, c->wPos.ensure(sizeof(float) * 3 * (size_t)nv));
        MDMC_CHECK(c, c->wNrm.ensure(sizeof(float) * 3 * (size_t)nv));
        MDMC_CHECK(c, c->wVfl.ensure(sizeof(uint32_t) * (size_t)nv));
        MDMC_CHECK(c, c->wHfl.ensure(sizeof(uint32_t) * (size_t)nh));
        MDMC_CHECK(c, c->wFfl.ensure(sizeof(uint32_t) * (size_t)nf));
        MDMC_CHECK(c, c->wVC2O.ensure(sizeof(int) * (size_t)nv));
        MDMC_CHECK(c, c->wHC2O.ensure(sizeof(int) * (size_t)nh));
        MDMC_CHECK(c, c->wFC2O.ensure(sizeof(int) * (size_t)nf));
        MDMC_CHECK(c, c->wOrigV.ensure(sizeof(int) * (size_t)nv));
        MDMC_CHECK(c, c->wOrigH.ensure(sizeof(int) * 4 * (size_t)n));
        MDMC_CHECK(c, c->wHe.ensure(sizeof(int4) * (size_t)nh));
        MDMC_CHECK(c, c->wFirst.ensure(sizeof(int) * (size_t)nf));
        MDMC_CHECK(c, c->wAttr.ensure(roundUp(sizeof(uint16_t) * (size_t)nf, 4)));
        MDMC_CHECK(c, c->wVNum.ensure(sizeof(int) * (size_t)nv));
        MDMC_CHECK(c, c->wVSlots.ensure(sizeof(int) * 4 * (size_t)nv));
        MDMC_CHECK(c, c->wHNum.ensure(sizeof(int) * (size_t)nh));
        MDMC_CHECK(c, c->wHSlots.ensure(sizeof(int) * 4 * (size_t)nh));
        MDMC_CHECK(c, c->wHTwin.ensure(sizeof(unsigned long long) * (size_t)nh));
        if ((st = ensureMaps(c, s)) != MDMC_OK) return st;
        MDMC_CHECK(c, cudaMemsetAsync(c->wVfl.p, 0, sizeof(uint32_t) * (size_t)nv, s));
        MDMC_CHECK(c, cudaMemsetAsync(c->wOrigV.p, 0xFF, sizeof(int) * (size_t)nv, s));
        MDMC_CHECK(c, cudaMemsetAsync(c->wHfl.p, 0, sizeof(uint32_t) * (size_t)nh, s));
        MDMC_CHECK(c, cudaMemsetAsync(c->wFfl.p, 0, sizeof(uint32_t) * (size_t)nf, s));
        MDMC_CHECK(c, cudaMemsetAsync(c->wVC2O.p, 0xFF, sizeof(int) * (size_t)nv, s));
        MDMC_CHECK(c, cudaMemsetAsync(c->wHC2O.p, 0xFF, sizeof(int) * (size_t)nh, s));
        MDMC_CHECK(c, cudaMemsetAsync(c->wFC2O.p, 0xFF, sizeof(int) * (size_t)nf, s));
        MDMC_CHECK(c, cudaMemsetAsync(c->wHe.p, 0xFF, sizeof(int4) * (size_t)nh, s));
        // (the partner slots need no clearing: an element's count says how
        // many of its slots the collapse wrote, and nothing reads beyond)
        launchFillInt(c->wVNum.as<int>(), nv, 1, s);
        launchFillInt(c->wHNum.as<int>(), nh, 1, s);
        MDMC_CHECK(c, c->splitFlags.ensure(sizeof(int) * 4));
        MDMC_CHECK(c, cudaMemsetAsync(c->splitFlags.p, 0, sizeof(int) * 4, s));
        SplitWork w = splitWork(c, nv, nh, nf);
        if (doSub) w.cornerLimit = 4 * n;

        // createWorkingCopies (:273-301)
        launchSplitCopy(c->nmFaces.as<int>(), n, c->he.as<int4>(), c->faceFirst.as<int>(), c->faceAttr.as<uint16_t>(),
                        c->pos.as<float>(), c->nrm.as<float>(), w, status, s);
        launchSplitMarkNM(c->nmList.as<int4>(), ctr, w, status, s);
        if (doSub) launchSplitSubdivide(n, w, status, s);
        if (step >= MDMC_STEP_COLLAPSE_NON_MANIFOLD_EDGES) {
            launchSplitCollapse(w, status, s);
            if (step >= MDMC_STEP_MERGE_VERTICES) launchSplitMerge(w, status, s);
            if (step >= MDMC_STEP_UPDATE_HALFEDGE_TWINS) launchSplitMergeHalfedges(w, status, s);
        }
        if (step >= MDMC_STEP_MOVE_VERTICES_TO_SURFACE) launchSplitMove(g, iso, w, s);

        // copyWorkingCopiesBack (:1297-1387): kept elements without an
        // original are appended in working-copy order
        MDMC_CHECK(c, c->appV.ensure(sizeof(int) * (size_t)(nv + 1)));
        MDMC_CHECK(c, c->appH.ensure(sizeof(int) * (size_t)(nh + 1)));
        MDMC_CHECK(c, c->appF.ensure(sizeof(int) * (size_t)(nf + 1)));
        MDMC_CHECK(c, c->scanScratch.ensure(sizeof(int4) * (size_t)scanScratchElems(nh)));
        if (!scanAppends(w.vfl, w.vC2O, nv, c->appV.as<int>(), c->scanScratch.as<int>(), s) ||
            !scanAppends(w.hfl, w.hC2O, nh, c->appH.as<int>(), c->scanScratch.as<int>(), s, (int)c->H) ||
            !scanAppends(w.ffl, w.fC2O, nf, c->appF.as<int>(), c->scanScratch.as<int>(), s))
            return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "prefix sum input too large");
        // a small iteration after a full refresh gets the local refresh: the
        // sizes of its old and kept edge sets come back with the append counts
        const bool local = c->rowsValid && doSub && (int64_t)nh * 16 <= c->H;
        if (local) {
            MDMC_CHECK(c, c->censusFill.ensure(sizeof(int) * 4));
            MDMC_CHECK(c, cudaMemsetAsync(c->censusFill.p, 0, sizeof(int) * 4, s));
            launchCensusCountOld(w, n, c->adjRow.as<int>(), c->adj.as<int2>(), c->he.as<int4>(), c->censusFill.as<int>(),
                                 s);
            MDMC_CHECK(c, cudaMemcpyAsync(c->hostInts + 3, c->censusFill.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
        }
        MDMC_CHECK(c, cudaMemcpyAsync(c->hostInts, c->appV.as<int>() + nv, sizeof(int), cudaMemcpyDeviceToHost, s));
        MDMC_CHECK(c, cudaMemcpyAsync(c->hostInts + 1, c->appH.as<int>() + nh, sizeof(int), cudaMemcpyDeviceToHost, s));
        MDMC_CHECK(c, cudaMemcpyAsync(c->hostInts + 2, c->appF.as<int>() + nf, sizeof(int), cudaMemcpyDeviceToHost, s));
        MDMC_CHECK(c, cudaStreamSynchronize(s));
        MDMC_CHECK(c, cudaGetLastError());
        const int64_t addV = c->hostInts[0], addH = c->hostInts[1], addF = c->hostInts[2];
        if (addV < 0 || addV > nv || addH < 0 || addH > nh || addF < 0 || addF > nf)
            return fail(c, MDMC_ERROR_CUDA, "inconsistent working-copy append counts");
        const int64_t V2 = c->V + addV, H2 = c->H + addH, F2 = c->F + addF;
        Census census;
        if (local) {
            const int64_t nOld = c->hostInts[3], nSame = c->hostInts[4];
            if (nOld < 0 || nSame < 0 || nSame > nOld || nOld > c->H)
                return fail(c, MDMC_ERROR_CUDA, "inconsistent local-refresh sizes");
            if ((st = censusBegin(c, w, n, (int)nOld, (int)(nSame + nh), census, s)) != MDMC_OK) return st;
        }
        MDMC_CHECK(c, c->pos.grow(sizeof(float) * 3 * (size_t)V2, sizeof(float) * 3 * (size_t)c->V, s));
        MDMC_CHECK(c, c->nrm.grow(sizeof(float) * 3 * (size_t)V2, sizeof(float) * 3 * (size_t)c->V, s));
        MDMC_CHECK(c, c->vflags.grow(roundUp((size_t)V2, 4), (size_t)c->V, s));
        MDMC_CHECK(c, c->appParent.grow(sizeof(int) * (size_t)std::max<int64_t>(V2 - c->dmcV, 1),
                                        sizeof(int) * (size_t)std::max<int64_t>(c->V - c->dmcV, 0), s));
        SplitWork wb = w;
        wb.appParent = c->appParent.as<int>();
        MDMC_CHECK(c, c->he.grow(sizeof(int4) * (size_t)H2, sizeof(int4) * (size_t)c->H, s));
        MDMC_CHECK(c, c->faceFirst.grow(sizeof(int) * (size_t)F2, sizeof(int) * (size_t)c->F, s));
        MDMC_CHECK(c, c->faceAttr.grow(roundUp(sizeof(uint16_t) * (size_t)F2, 4), sizeof(uint16_t) * (size_t)c->F, s));
        launchSplitCopyBack(wb, c->appV.as<int>(), c->appH.as<int>(), c->appF.as<int>(), (int)V2, (int)H2, (int)F2,
                            c->pos.as<float>(), c->nrm.as<float>(), c->he.as<int4>(), c->faceFirst.as<int>(),
                            c->faceAttr.as<uint16_t>(), status, s);
        launchSplitResetMaps(n, c->nmFaces.as<int>(), w, s);
        const int64_t V1 = c->V, F1 = c->F;
        c->V = V2;
        c->H = H2;
        c->F = F2;
        if (local) st = censusFinish(c, wb, census, V1, F1, s);
        else st = refreshTable(c, status, s);
        if (st != MDMC_OK) return st;
        MDMC_CHECK(c, cudaGetLastError());
        ++iterations;
        if (step < MDMC_STEP_ENABLE_ITERATIVE_REFINEMENT) break;
        if (iterations >= 64) {  // the reference loops without a cap
            uint32_t bit = kStatusIterationCap;
            MDMC_CHECK(c, cudaMemcpyAsync(c->hostInts, status, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
            MDMC_CHECK(c, cudaStreamSynchronize(s));
            bit |= (uint32_t)c->hostInts[0];
            MDMC_CHECK(c, cudaMemcpyAsync(status, &bit, sizeof(uint32_t), cudaMemcpyHostToDevice, s));
            MDMC_CHECK(c, cudaStreamSynchronize(s));
            break;
        }
    }
    return MDMC_OK;
}

// mdmc_run_to_host: as soon as the quad pass has written a range of quads
// (their halfedges, quads and face arrays) or the vertex pass the positions
// and normals, copy them to the caller's host arrays on the copy stream while
// the run goes on.  Only when the whole mesh fits the host arrays; the end of
// the call copies again whatever a later stage rewrote.
bool earlyFits(const mdmc_context* c) {
    const mdmc_host_mesh* h = c->hostOut;
    return h && c->V <= h->capacity_vertices && c->F <= h->capacity_faces;
}

mdmc_status copyAfter(mdmc_context* c, int k, cudaStream_t s) {
    MDMC_CHECK(c, cudaEventRecord(c->copyEv[k], s));
    MDMC_CHECK(c, cudaStreamWaitEvent(c->copyStream, c->copyEv[k], 0));
    return MDMC_OK;
}

cudaError_t copyOut(mdmc_context* c, void* dst, const void* src, size_t bytes) {
    if (!dst || bytes == 0) return cudaSuccess;
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->copyStream);
}

// the halfedges and output quads of quads [q0, q1); with faces also the face
// first halfedges and attributes of quads [0, q1) (small arrays, copied once
// after the last range: every copy costs the link time of its own)
mdmc_status earlyCopyFaces(mdmc_context* c, int64_t q0, int64_t q1, bool faces, cudaStream_t s) {
    const mdmc_host_mesh* h = c->hostOut;
    mdmc_status st = copyAfter(c, 0, s);
    if (st != MDMC_OK) return st;
    const size_t n = (size_t)(q1 - q0);
    MDMC_CHECK(c, copyOut(c, h->halfedges ? h->halfedges + 16 * q0 : nullptr, c->he.as<int4>() + 4 * q0, 4 * sizeof(int4) * n));
    MDMC_CHECK(c, copyOut(c, h->quads ? h->quads + 4 * q0 : nullptr, c->quads.as<int4>() + q0, sizeof(int4) * n));
    if (faces) {
        MDMC_CHECK(c, copyOut(c, h->face_first_halfedge, c->faceFirst.as<int>(), sizeof(int) * (size_t)q1));
        MDMC_CHECK(c, copyOut(c, h->face_attributes, c->faceAttr.as<uint16_t>(), sizeof(uint16_t) * (size_t)q1));
    }
    return MDMC_OK;
}

// the vertex halfedges and flags, final once the fan detection has run
mdmc_status earlyCopyVertexMaps(mdmc_context* c, cudaStream_t s) {
    const mdmc_host_mesh* h = c->hostOut;
    mdmc_status st = copyAfter(c, 0, s);
    if (st != MDMC_OK) return st;
    MDMC_CHECK(c, copyOut(c, h->vertex_halfedge, c->vertexHE.p, sizeof(int) * (size_t)c->V));
    MDMC_CHECK(c, copyOut(c, h->vertex_flags, c->vflags.p, (size_t)c->V));
    c->earlyVertexMaps = true;
    return MDMC_OK;
}

mdmc_status earlyCopyVertices(mdmc_context* c, cudaStream_t s) {
    const mdmc_host_mesh* h = c->hostOut;
    mdmc_status st = copyAfter(c, 1, s);
    if (st != MDMC_OK) return st;
    MDMC_CHECK(c, copyOut(c, h->positions, c->pos.p, sizeof(float) * 3 * (size_t)c->V));
    MDMC_CHECK(c, copyOut(c, h->normals, c->nrm.p, sizeof(float) * 3 * (size_t)c->V));
    c->earlyVertices = true;
    return MDMC_OK;
}

// The DMC front end: the active-cell mask per x-row of cells (W words per
// row, numWords in all) and the index of every word's first active cell
// (cellFirst, the cell index the quad pass reads too); A = active cells.
// The mask and its scan, without reading the count back: the scan lists the
// active cells' ids as far as the list holds (idsCapacity); cellFirst[numWords]
// is the count.
mdmc_status markActive(mdmc_context* c, const GridDesc& g, float iso, int& W, int64_t& numWords, int64_t& idsCapacity,
                       cudaStream_t s) {
    const GridGeom& geom = g.geom();
    const int X = geom.X, Y = geom.Y, Z = geom.Z;
    uint32_t* status = &c->counters.as<DevCounters>()->status;
    const int64_t numRows = (X > 1 && Y > 1 && Z > 1) ? (int64_t)(Y - 1) * (Z - 1) : 0;
    W = (X - 1 + 31) / 32;
    numWords = numRows * (int64_t)W;
    MDMC_CHECK(c, c->cellMask.ensure(sizeof(uint32_t) * (size_t)std::max<int64_t>(numWords, 1)));
    MDMC_CHECK(c, c->cellFirst.ensure(sizeof(int) * (size_t)(numWords + 1)));
    markKernel(c, 2, s);
    if (g.refined && numWords > 0) MDMC_CHECK(c, cudaMemsetAsync(c->cellMask.p, 0, sizeof(uint32_t) * (size_t)numWords, s));
    const bool blockMask = g.refined && g.ref.mayCross && 2 * (g.ref.r + 4) * (g.ref.r + 4) <= 512 && numWords > 0;
    // per-cell cases for the emit pass: every cell of a plain grid, the
    // standard blocks of a x4 refinement without padding
    CaseBytes cases;
    if (!g.refined && numWords > 0) {
        MDMC_CHECK(c, c->caseBytes.ensure((size_t)X * Y * Z));
        cases = CaseBytes{c->caseBytes.as<uint8_t>(), 1};
    } else if (blockMask && g.ref.r == 3 && !g.ref.pad) {
        const int64_t coarseCells = (int64_t)(g.ref.cX - 1) * (g.ref.cY - 1) * (g.ref.cZ - 1);
        MDMC_CHECK(c, c->caseBytes.ensure((size_t)coarseCells * 64));
        cases = CaseBytes{c->caseBytes.as<uint8_t>(), 2};
    }
    c->caseMode = cases.mode;
    if (blockMask)
        launchBlockMask(g.ref, iso, c->candidates.as<uint32_t>(), &c->counters.as<DevCounters>()->candidates,
                        c->cellMask.as<uint32_t>(), W, cases, status, s);
    else
        launchRowMask(g, iso, c->cellMask.as<uint32_t>(), (int)numRows, W, cases, s);
    // the scan also lists the active cells' ids, as many as the list holds
    // already (all of them when the grid is like the last one)
    MDMC_CHECK(c, c->scanScratch.ensure(sizeof(int4) * (size_t)scanScratchElems(numWords)));
    idsCapacity = (int64_t)(c->cellIds.bytes / sizeof(uint32_t));
    if (!scanMaskScatter(c->cellMask.as<uint32_t>(), c->cellFirst.as<int>(), numWords, W, X, Y,
                         c->cellIds.as<uint32_t>(), idsCapacity, c->scanScratch.as<int>(), s))
        return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "prefix sum input too large");
    markKernel(c, 3, s);
    MDMC_CHECK(c, cudaGetLastError());
    return MDMC_OK;
}

// With the count A known: checks it and lists the ids the scan had no room for.
mdmc_status finishActive(mdmc_context* c, const GridDesc& g, int W, int64_t numWords, int64_t A, int64_t idsCapacity,
                         cudaStream_t s) {
    const GridGeom& geom = g.geom();
    const int X = geom.X, Y = geom.Y, Z = geom.Z;
    const int64_t cells = (X > 1 && Y > 1 && Z > 1) ? (int64_t)(X - 1) * (Y - 1) * (Z - 1) : 0;
    if (A < 0 || A > cells) return fail(c, MDMC_ERROR_CUDA, "inconsistent cell count from the mask pass");
    if (A > 0x7FFFFFFF) return fail(c, MDMC_ERROR_LIMIT, "more than 2^31 active cells");
    if (A > idsCapacity) {
        MDMC_CHECK(c, c->cellIds.ensure(sizeof(uint32_t) * (size_t)A));
        launchScatterCells(c->cellMask.as<uint32_t>(), c->cellFirst.as<int>(), numWords, W, X, Y,
                           c->cellIds.as<uint32_t>(), (int)A, &c->counters.as<DevCounters>()->status, s);
    }
    return MDMC_OK;
}

// The DMC front end with the count read back: mask, scan and the ids of all
// active cells.
mdmc_status activeCells(mdmc_context* c, const GridDesc& g, float iso, int& W, int64_t& numWords, int64_t& A,
                        cudaStream_t s) {
    int64_t idsCapacity = 0;
    mdmc_status st = markActive(c, g, iso, W, numWords, idsCapacity, s);
    if (st != MDMC_OK) return st;
    if ((st = readInts(c, c->cellFirst.as<int>() + numWords, 1, s)) != MDMC_OK) return st;
    A = c->hostInts[0];
    return finishActive(c, g, W, numWords, A, idsCapacity, s);
}

}  // namespace

extern "C" {

void mdmc_default_options(mdmc_options* options) {
    if (options) defaultOptions(options);
}

mdmc_status mdmc_create(mdmc_context** context, const mdmc_options* options) {
    if (!context) return MDMC_ERROR_INVALID_ARGUMENT;
    *context = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return MDMC_ERROR_NO_DEVICE;
    if (cudaFree(nullptr) != cudaSuccess) return MDMC_ERROR_CUDA;  // context unusable
    mdmc_context* c = new mdmc_context();
    if (options) c->opt = *options;
    else defaultOptions(&c->opt);
    std::memset(&c->stats, 0, sizeof c->stats);
    if (cudaMallocHost(&c->hostCounters, sizeof(DevCounters)) != cudaSuccess ||
        cudaMallocHost(&c->hostInts, 64 * sizeof(int32_t)) != cudaSuccess || c->counters.ensure(sizeof(DevCounters)) != cudaSuccess) {
        mdmc_destroy(c);
        return MDMC_ERROR_OUT_OF_MEMORY;
    }
    void* mapped = nullptr;
    if (cudaHostGetDevicePointer(&mapped, c->hostInts, 0) == cudaSuccess) c->hostIntsDev = static_cast<int32_t*>(mapped);
    else (void)cudaGetLastError();
    for (auto& e : c->ev) cudaEventCreate(&e);
    for (auto& e : c->kev) cudaEventCreate(&e);
    for (auto& e : c->copyEv) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    if (cudaEventCreateWithFlags(&c->countsEv, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->copyStream, cudaStreamNonBlocking) != cudaSuccess) {
        mdmc_destroy(c);
        return MDMC_ERROR_CUDA;
    }
    // record every event once so that elapsed-time queries of stages a run
    // skips (e.g. no refinement on this context) return 0 instead of failing
    for (auto& e : c->ev) cudaEventRecord(e, 0);
    for (auto& e : c->kev) cudaEventRecord(e, 0);
    if (cudaDeviceSynchronize() != cudaSuccess) {
        mdmc_destroy(c);
        return MDMC_ERROR_CUDA;
    }
    *context = c;
    return MDMC_OK;
}

void mdmc_destroy(mdmc_context* c) {
    if (!c) return;
    for (auto& e : c->ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : c->kev)
        if (e) cudaEventDestroy(e);
    for (auto& e : c->copyEv)
        if (e) cudaEventDestroy(e);
    if (c->countsEv) cudaEventDestroy(c->countsEv);
    if (c->copyStream) cudaStreamDestroy(c->copyStream);
    if (c->hostCounters) cudaFreeHost(c->hostCounters);
    if (c->hostInts) cudaFreeHost(c->hostInts);
    delete c;
}

mdmc_status mdmc_set_kernel_timing(mdmc_context* c, uint32_t kernels) {
    if (!c || (kernels & ~(uint32_t)MDMC_TIME_ALL)) return MDMC_ERROR_INVALID_ARGUMENT;
    c->kernelTiming = kernels;
    return MDMC_OK;
}

mdmc_status mdmc_set_options(mdmc_context* c, const mdmc_options* options) {
    if (!c || !options) return MDMC_ERROR_INVALID_ARGUMENT;
    c->opt = *options;
    return MDMC_OK;
}

mdmc_status mdmc_get_options(const mdmc_context* c, mdmc_options* options) {
    if (!c || !options) return MDMC_ERROR_INVALID_ARGUMENT;
    *options = c->opt;
    return MDMC_OK;
}

mdmc_status mdmc_read_bin(const char* path, int32_t dims[3], float spacing[3], float origin[3], float* host_samples) {
    if (!path || !dims || !spacing || !origin) return MDMC_ERROR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "rb");
    if (!f) return MDMC_ERROR_IO;
    bool ok = std::fread(dims, sizeof(int32_t), 3, f) == 3 && std::fread(spacing, sizeof(float), 3, f) == 3;
    if (!ok || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) {
        std::fclose(f);
        return MDMC_ERROR_IO;
    }
    for (int a = 0; a < 3; ++a) origin[a] = (-0.5f * (float)(dims[a] - 1)) * spacing[a];
    if (host_samples) {
        const size_t n = (size_t)dims[0] * dims[1] * dims[2];
        std::vector<uint16_t> raw(n);
        if (std::fread(raw.data(), sizeof(uint16_t), n, f) != n) {
            std::fclose(f);
            return MDMC_ERROR_IO;
        }
        for (size_t i = 0; i < n; ++i) host_samples[i] = (float)raw[i];
    }
    std::fclose(f);
    return MDMC_OK;
}

mdmc_status mdmc_prepare_grid(mdmc_context* c, const float* samples, int samples_on_host, const int32_t dims[3],
                              const float origin[3], const float spacing[3], int32_t refinement,
                              int32_t add_zero_boundary, mdmc_grid* out, void* stream) {
    if (!c || !samples || !dims || !origin || !spacing || !out) return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "null argument");
    if (refinement < 0 || dims[0] < 1 || dims[1] < 1 || dims[2] < 1)
        return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "invalid dims or refinement");
    (void)cudaGetLastError();  // errors of earlier, unrelated runtime calls are not ours
    cudaStream_t s = (cudaStream_t)stream;
    const int pad = add_zero_boundary ? 1 : 0;
    int32_t od[3];
    float osp[3], oor[3];
    size_t outN = 1, inN = 1;
    for (int a = 0; a < 3; ++a) {
        // D/UniformGrid.inl:585-598
        const int64_t d = (int64_t)dims[a] + (int64_t)(dims[a] - 1) * refinement + 2 * pad;
        if (d > (1 << 30)) return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "refined grid too large");
        od[a] = (int32_t)d;
        osp[a] = (spacing[a] * 1.f) / ((float)refinement + 1.f);
        oor[a] = origin[a];
        if (pad) oor[a] = oor[a] - osp[a];
        outN *= (size_t)od[a];
        inN *= (size_t)dims[a];
    }
    if (outN >= 0xFFFFFFFFull) return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "grid has 2^32 samples or more");
    const float* src = samples;
    out->coarse_samples = nullptr;
    out->coarse_dims[0] = out->coarse_dims[1] = out->coarse_dims[2] = 0;
    out->refinement = refinement;
    out->add_zero_boundary = pad;
    if (refinement == 0 && !pad) {
        if (samples_on_host) {
            MDMC_CHECK(c, c->gridBuf.ensure(sizeof(float) * outN));
            MDMC_CHECK(c, cudaMemcpyAsync(c->gridBuf.p, samples, sizeof(float) * outN, cudaMemcpyHostToDevice, s));
            src = c->gridBuf.as<float>();
        }
        out->samples = src;
    } else {
        // refined on demand from the coarse grid by the kernels that read it
        if (samples_on_host) {
            MDMC_CHECK(c, c->stageBuf.ensure(sizeof(float) * inN));
            MDMC_CHECK(c, cudaMemcpyAsync(c->stageBuf.p, samples, sizeof(float) * inN, cudaMemcpyHostToDevice, s));
            src = c->stageBuf.as<float>();
        }
        out->samples = nullptr;
        out->coarse_samples = src;
        for (int a = 0; a < 3; ++a) out->coarse_dims[a] = dims[a];
    }
    for (int a = 0; a < 3; ++a) {
        out->dims[a] = od[a];
        out->origin[a] = oor[a];
        out->spacing[a] = osp[a];
    }
    return MDMC_OK;
}

mdmc_status mdmc_materialize_grid(mdmc_context* c, const mdmc_grid* grid, float* out, void* stream) {
    if (!c || !grid || !out) return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "null argument");
    (void)cudaGetLastError();
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = (size_t)grid->dims[0] * grid->dims[1] * grid->dims[2];
    if (grid->coarse_samples && (grid->refinement > 0 || grid->add_zero_boundary)) {
        launchRefine(grid->coarse_samples, make_int3(grid->coarse_dims[0], grid->coarse_dims[1], grid->coarse_dims[2]),
                     out, make_int3(grid->dims[0], grid->dims[1], grid->dims[2]), grid->refinement,
                     grid->add_zero_boundary ? 1 : 0, s);
        MDMC_CHECK(c, cudaGetLastError());
    } else {
        if (!grid->samples) return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "grid has no samples");
        MDMC_CHECK(c, cudaMemcpyAsync(out, grid->samples, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
    }
    return MDMC_OK;
}

mdmc_status mdmc_run(mdmc_context* c, const mdmc_grid* grid, float iso, mdmc_mesh* mesh, mdmc_stats* stats,
                     void* stream) {
    if (!c || !grid) return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "null argument");
    c->err.clear();
    (void)cudaGetLastError();  // errors of earlier, unrelated runtime calls are not ours
    const int X = grid->dims[0], Y = grid->dims[1], Z = grid->dims[2];
    if (X < 1 || Y < 1 || Z < 1) return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "invalid grid dims");
    if ((uint64_t)X * Y * Z >= 0xFFFFFFFFull) return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "grid has 2^32 samples or more");
    cudaStream_t s = (cudaStream_t)stream;
    c->haveMesh = false;
    c->lastGrid = *grid;
    c->lastIso = iso;
    c->lastSurfaceIteration = c->opt.enable_surface_to_vertex_iteration;
    c->dmcV = c->activeCells = 0;
    c->simplified = false;
    c->earlyFaces = c->earlyVertices = c->earlyVertexMaps = c->lateChange = false;
    c->rowsValid = false;
    c->fastFans = false;
    std::memset(&c->stats, 0, sizeof c->stats);
    DevCounters* ctr = c->counters.as<DevCounters>();
    uint32_t* status = &ctr->status;
    MDMC_CHECK(c, cudaMemsetAsync(ctr, 0, sizeof(DevCounters), s));
    const long long launches0 = g_kernelLaunches.load();
    markStage(c, 0, true, s);
    markKernel(c, 0, s);
    markKernel(c, 1, s);
    GridDesc g;
    mdmc_status st0 = makeGridDesc(c, grid, iso, g, s);
    if (st0 != MDMC_OK) return st0;

    // ---- DMC (performDualMarchingCubes) -----------------------------------------
    int64_t numWords = 0, idsCapacity = 0;
    int W = 0;
    mdmc_status st = markActive(c, g, iso, W, numWords, idsCapacity, s);
    if (st != MDMC_OK) return st;

    // The active cells' records, their contour and quad counts, and in the
    // scan of the counts their offsets and the quad owners.  Without reading
    // the active-cell count back first: the records are made for as many cells
    // as the lists hold (all of them when the grid is like the last one), the
    // count read on the device, and one read-back brings the cell, vertex and
    // quad counts; only when the lists were too short is the pass repeated at
    // the right size.
    const int* numActiveDev = c->cellFirst.as<int>() + numWords;
    MDMC_CHECK(c, c->cellCounts.ensure(sizeof(int2)));
    int64_t capA = std::min<int64_t>(idsCapacity, (int64_t)(c->act.bytes / sizeof(ActiveCell)));
    capA = std::min<int64_t>(capA, (int64_t)(c->cellCounts.bytes / sizeof(int2)) - 1);
    capA = std::max<int64_t>(std::min<int64_t>(capA, 0x7FFFFFFF), 0);
    const int64_t capQ = std::min<int64_t>((int64_t)(c->quadOwner.bytes / sizeof(int)), 0x7FFFFFFF);
    markKernel(c, 4, s);
    MDMC_CHECK(c, c->scanScratch.ensure(sizeof(int4) * (size_t)scanScratchElems(capA)));
    launchEmitActive(g, iso, c->cellIds.as<uint32_t>(), c->act.as<ActiveCell>(), c->cellCounts.as<int2>(), (int)capA,
                     CaseBytes{c->caseBytes.as<uint8_t>(), c->caseMode}, status, s, numActiveDev);
    // the scan's last block writes the counts straight into the pinned host
    // scratch when the device can address it (no copy on the stream)
    if (!scanCellCounts(c->cellCounts.as<int2>(), capA, numActiveDev, c->act.as<ActiveCell>(), c->quadOwner.as<int>(),
                        capQ, ctr->gathered, c->hostIntsDev, c->scanScratch.as<int2>(), s))
        return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "prefix sum input too large");
    markKernel(c, 5, s);
    if (!c->hostIntsDev)
        MDMC_CHECK(c, cudaMemcpyAsync(c->hostInts, ctr->gathered, 3 * sizeof(int), cudaMemcpyDeviceToHost, s));
    MDMC_CHECK(c, cudaEventRecord(c->countsEv, s));
    // Before the counts reach the host: when the arrays of an earlier run are
    // large enough, the vertex pass runs on the device's counts, so that the
    // device works while the host waits for them.  Not for runs into host
    // arrays, whose quad pass goes first to start the copies.
    DeviceCounts spec{ctr->gathered, 0, 0, 0};
    bool speculated = false;
    if (!c->hostOut && capA > 0 && capQ > 0) {
        const int64_t capV = std::min<int64_t>(
            std::min<int64_t>(std::min(c->pos.bytes, c->nrm.bytes) / (3 * sizeof(float)),
                              (int64_t)(std::min(c->degree.bytes, c->vertexHE.bytes) / sizeof(int))),
            (int64_t)(c->vflags.bytes & ~(size_t)3));  // (the flags are kept in whole words)
        if (capV > 0) {
            spec.capA = (int)capA;
            spec.capV = (int)std::min<int64_t>(capV, 0x7FFFFFFF);
            spec.capQ = (int)capQ;
            markKernel(c, 10, s);
            launchVertices(g, iso, c->opt.enable_surface_to_vertex_iteration, c->act.as<ActiveCell>(), spec.capA,
                           spec.capV, c->pos.as<float>(), c->nrm.as<float>(), c->degree.as<int>(),
                           c->vflags.as<uint8_t>(), c->vertexHE.as<int>(), status, s, &spec);
            markKernel(c, 11, s);
            speculated = true;
        }
    }
    MDMC_CHECK(c, cudaGetLastError());
    MDMC_CHECK(c, cudaEventSynchronize(c->countsEv));  // the counts, not the passes behind them
    const int64_t A = c->hostInts[0];
    int64_t Vd = c->hostInts[1], Q = c->hostInts[2];
    // the records and quad owners, and the vertex pass's vertices, are
    // complete exactly when the counts fit what the passes covered
    const bool emitDone = A >= 0 && A <= capA && Q >= 0 && Q <= capQ;
    const bool aheadDone = speculated && spec.fits(A, Vd, Q);
    if ((st = finishActive(c, g, W, numWords, A, idsCapacity, s)) != MDMC_OK) return st;
    c->stats.num_active_cells = A;
    if (!emitDone) {
        MDMC_CHECK(c, c->act.ensure(sizeof(ActiveCell) * (size_t)std::max<int64_t>(A, 1)));
        MDMC_CHECK(c, c->cellCounts.ensure(sizeof(int2) * (size_t)(A + 1)));
        const int64_t needQ = A <= capA && Q >= 0 ? Q : 3 * A;  // a cell owns at most three quads
        if (needQ >= (int64_t)0x7FFFFFFF) return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "more than 2^31 quads");
        MDMC_CHECK(c, c->quadOwner.ensure(sizeof(int) * (size_t)std::max<int64_t>(needQ, 1)));
        MDMC_CHECK(c, c->scanScratch.ensure(sizeof(int4) * (size_t)scanScratchElems(A)));
        launchEmitActive(g, iso, c->cellIds.as<uint32_t>(), c->act.as<ActiveCell>(), c->cellCounts.as<int2>(), (int)A,
                         CaseBytes{c->caseBytes.as<uint8_t>(), c->caseMode}, status, s);
        if (!scanCellCounts(c->cellCounts.as<int2>(), A, nullptr, c->act.as<ActiveCell>(), c->quadOwner.as<int>(),
                            needQ, ctr->gathered, nullptr, c->scanScratch.as<int2>(), s))
            return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "prefix sum input too large");
        MDMC_CHECK(c, cudaGetLastError());
        if (A > 0) {
            if ((st = readInts(c, ctr->gathered, 3, s)) != MDMC_OK) return st;
            Vd = c->hostInts[1];
            Q = c->hostInts[2];
        } else {
            Vd = Q = 0;
        }
    }
    if (Vd < A || Vd > 4 * A || Q < 0 || Q > 3 * A)
        return fail(c, MDMC_ERROR_CUDA, "inconsistent vertex or quad count from the emit pass");
    c->stats.num_dmc_vertices = Vd;
    c->stats.num_dmc_quads = Q;
    if (4 * Q >= (int64_t)0x7FFFFFFF) return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "more than 2^31 halfedges");
    if (Vd == 0) {
        // "DMC: No Vertices have been produced!" (D/DualMarchingCubes.cu:256-261)
        c->V = c->F = c->H = 0;
        c->stats.num_edges = c->stats.num_edges3 = c->stats.num_edges4 = -1;
        c->stats.num_non_manifold_vertices = -1;
        for (int k = 0; k < 4; ++k) c->stats.quads_with_non_manifold_edges[k] = -1;
        c->haveMesh = true;
        if (mesh) mdmc_get_mesh(c, mesh);
        if (stats) *stats = c->stats;
        return MDMC_OK;
    }
    c->V = Vd;
    c->F = Q;
    c->H = 4 * Q;
    c->dmcV = Vd;
    c->activeCells = A;
    MDMC_CHECK(c, c->quadOwner.ensure(sizeof(int) * (size_t)std::max<int64_t>(Q, 1)));
    MDMC_CHECK(c, c->pos.ensure(sizeof(float) * 3 * (size_t)Vd));
    MDMC_CHECK(c, c->nrm.ensure(sizeof(float) * 3 * (size_t)Vd));
    MDMC_CHECK(c, c->vflags.ensure(roundUp((size_t)Vd, 4)));
    MDMC_CHECK(c, c->he.ensure(sizeof(int4) * 4 * (size_t)std::max<int64_t>(Q, 1)));
    MDMC_CHECK(c, c->faceFirst.ensure(sizeof(int) * (size_t)std::max<int64_t>(Q, 1)));
    MDMC_CHECK(c, c->faceAttr.ensure(roundUp(sizeof(uint16_t) * (size_t)std::max<int64_t>(Q, 1), 4)));
    MDMC_CHECK(c, c->nmList.ensure(sizeof(int4) * (size_t)(Q + 1)));
    MDMC_CHECK(c, c->heValence.ensure((size_t)std::max<int64_t>(4 * Q, 1)));
    // (the vertex pass run ahead set the flags and stars' starting values)
    if (!aheadDone) MDMC_CHECK(c, cudaMemsetAsync(c->vflags.p, 0, roundUp((size_t)Vd, 4), s));
    MDMC_CHECK(c, c->quads.ensure(sizeof(int4) * (size_t)std::max<int64_t>(Q, 1)));
    MDMC_CHECK(c, c->vertexHE.ensure(sizeof(int) * (size_t)Vd));
    MDMC_CHECK(c, c->degree.ensure(sizeof(int) * (size_t)Vd));
    if (!aheadDone) MDMC_CHECK(c, cudaMemsetAsync(c->vertexHE.p, 0x7F, sizeof(int) * (size_t)Vd, s));

    // mapQuadrilaterals + collectHalfedgeElements, and the halfedge mesh's
    // twins and flags (HalfedgeMesh::initialize) in the same pass
    markKernel(c, 6, s);
    // with host arrays to fill, the quads go in ranges, each copied out as
    // soon as it is written, so that the copies start early
    const bool early = earlyFits(c);
    const int ranges = early ? kCopyRanges : 1;
    for (int k = 0; k < ranges; ++k) {
        const int64_t q0 = Q * k / ranges, q1 = Q * (k + 1) / ranges;
        launchQuads(c->act.as<ActiveCell>(), c->quadOwner.as<int>(), (int)A, c->cellMask.as<uint32_t>(),
                    c->cellFirst.as<int>(), X, Y, Z, W, c->he.as<int4>(), c->faceFirst.as<int>(),
                    c->faceAttr.as<uint16_t>(), c->vflags.as<uint8_t>(), c->heValence.as<uint8_t>(),
                    c->nmList.as<int4>(), (int)(Q + 1), (int)Q, (int)Vd, c->quads.as<int4>(), c->vertexHE.as<int>(),
                    ctr, (int)q0, (int)q1, s);
        if (early && (st = earlyCopyFaces(c, q0, q1, k == ranges - 1, s)) != MDMC_OK) return st;
    }
    c->earlyFaces = early;
    c->faceNMValid = false;  // the quad pass wrote heValence
    markKernel(c, 7, s);
    // vertex positions and normals (sliceP's vertex part)
    if (!aheadDone) {
        markKernel(c, 10, s);
        launchVertices(g, iso, c->opt.enable_surface_to_vertex_iteration, c->act.as<ActiveCell>(), (int)A, (int)Vd,
                       c->pos.as<float>(), c->nrm.as<float>(), c->degree.as<int>(), nullptr, nullptr, status, s);
        markKernel(c, 11, s);
    }
    if (early && (st = earlyCopyVertices(c, s)) != MDMC_OK) return st;
    MDMC_CHECK(c, cudaGetLastError());
    markStage(c, 1, true, s);
    markKernel(c, 8, s);
    // runPostProcesses, D/DualMarchingCubes.cu:335-380: simplifications first
    if (c->opt.simplify_p3x3y_color && (st = runSimplification(c, 0, s)) != MDMC_OK) return st;
    if (c->opt.simplify_p3x3y_old && (st = runSimplification(c, 1, s)) != MDMC_OK) return st;
    if (c->opt.simplify_p3333 && (st = runSimplification(c, 2, s)) != MDMC_OK) return st;
    const MeshDims md0{(int)c->V, (int)c->F, (int)c->H};
    markKernel(c, 9, s);
    markStage(c, 2, c->opt.simplify_p3x3y_color || c->opt.simplify_p3x3y_old || c->opt.simplify_p3333, s);

    // ---- repair: fixManifoldTwins, then the splitter ---------------------------
    launchReconnect(g, iso, c->nmList.as<int4>(), ctr, c->he.as<int4>(), c->pos.as<float>(), md0,
                    status, s);
    MDMC_CHECK(c, cudaGetLastError());
    int64_t iterations = 0;
    // When no face is non-manifold the splitter does nothing and the mesh is
    // final here, with its vertex stars, output quads and face statistics
    // already written by the quad pass: detection and output run at once and
    // one read-back decides.  Their status bits go to a side word, kept only if
    // the splitter turns out not to run.
    bool finished = false;
    if (!c->simplified) {
        markStage(c, 3, true, s);
        // (on the device the detection is skipped when the splitter will run)
        if ((st = finishMesh(c, true, &ctr->specStatus, s, c->opt.split_non_manifold_halfedges ? &ctr->nmBuckets : nullptr)) !=
            MDMC_OK)
            return st;
        if (early && (st = earlyCopyVertexMaps(c, s)) != MDMC_OK) return st;
        MDMC_CHECK(c, cudaMemcpyAsync(c->hostCounters, ctr, sizeof(DevCounters), cudaMemcpyDeviceToHost, s));
        MDMC_CHECK(c, cudaStreamSynchronize(s));
        finished = !(c->opt.split_non_manifold_halfedges && c->hostCounters->nmBuckets > 0);
        c->lateChange = c->hostCounters->nmBuckets > 0;  // fixManifoldTwins rewrote twins
        if (finished) c->hostCounters->status |= c->hostCounters->specStatus;
    }
    if (!finished) {
        c->lateChange = true;
        if (c->opt.split_non_manifold_halfedges) {
            if ((st = runSplitter(c, g, iso, iterations, s)) != MDMC_OK) return st;
        }
        markStage(c, 3, true, s);
        // the splitter's refresh reset the edge counters; detection and the
        // face statistics start from zero again
        MDMC_CHECK(c, cudaMemsetAsync(&ctr->nmVertices, 0, sizeof(unsigned long long), s));
        MDMC_CHECK(c, cudaMemsetAsync(&ctr->quadsNM[0], 0, sizeof(ctr->quadsNM), s));
        if ((st = finishMesh(c, false, status, s)) != MDMC_OK) return st;
        MDMC_CHECK(c, cudaMemcpyAsync(c->hostCounters, ctr, sizeof(DevCounters), cudaMemcpyDeviceToHost, s));
        MDMC_CHECK(c, cudaStreamSynchronize(s));
    }

    const DevCounters& hc = *c->hostCounters;
    c->stats.num_edges = (int64_t)hc.edges;
    c->stats.num_edges3 = (int64_t)hc.edges3;
    c->stats.num_edges4 = (int64_t)hc.edges4;
    c->stats.num_non_manifold_vertices = c->opt.detect_non_manifold_vertices ? (int64_t)hc.nmVertices : -1;
    for (int k = 0; k < 4; ++k) c->stats.quads_with_non_manifold_edges[k] = (int64_t)hc.quadsNM[k + 1];
    c->stats.split_iterations = iterations;
    c->stats.anomalies = (int64_t)hc.status;
    float ms[5] = {0, 0, 0, 0, 0};
    if (c->kernelTiming & MDMC_TIME_STAGES) {
        for (int k = 0; k < 4; ++k)
            if (cudaEventElapsedTime(&ms[k], c->ev[c->evAt[k]], c->ev[c->evAt[k + 1]]) != cudaSuccess) ms[k] = 0.f;
        if (cudaEventElapsedTime(&ms[4], c->ev[c->evAt[0]], c->ev[c->evAt[5]]) != cudaSuccess) ms[4] = 0.f;
    }
    c->stats.ms_dmc = ms[0];
    c->stats.ms_halfedge = ms[1];
    c->stats.ms_repair = ms[2];
    c->stats.ms_detect = ms[3];
    c->stats.ms_total = ms[4];
    float km[6] = {0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 6; ++k)
        if (((c->kernelTiming >> k) & 1u) &&
            cudaEventElapsedTime(&km[k], c->kev[2 * k], c->kev[2 * k + 1]) != cudaSuccess)
            km[k] = 0.f;
    (void)cudaGetLastError();  // elapsed-time queries leave no error behind
    c->stats.ms_refine = km[0];
    c->stats.ms_count = km[1];
    c->stats.ms_emit = km[2];
    c->stats.ms_quads = km[3];
    c->stats.ms_table = km[4];
    c->stats.ms_vertices = km[5];
    c->stats.kernel_launches = (int64_t)(g_kernelLaunches.load() - launches0);
    c->haveMesh = true;
    if (mesh) mdmc_get_mesh(c, mesh);
    if (stats) *stats = c->stats;
    if (hc.status) {
        c->err = "device limits hit: " + statusText(hc.status);
        if (hc.status & (kStatusProbeLimit | kStatusMissingCell)) return MDMC_ERROR_LIMIT;
    }
    return MDMC_OK;
}

mdmc_status mdmc_run_standard_mc(mdmc_context* c, const mdmc_grid* grid, float iso, mdmc_triangle_mesh* mesh,
                                 void* stream) {
    if (!c || !grid) return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "null argument");
    c->err.clear();
    (void)cudaGetLastError();
    const int X = grid->dims[0], Y = grid->dims[1], Z = grid->dims[2];
    if (X < 1 || Y < 1 || Z < 1) return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "invalid grid dims");
    if (3 * (uint64_t)X * Y * Z >= 0xFFFFFFFFull)
        return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "grid has 2^32 edges or more");
    cudaStream_t s = (cudaStream_t)stream;
    c->mcV = c->mcT = 0;
    if (mesh) std::memset(mesh, 0, sizeof *mesh);
    DevCounters* ctr = c->counters.as<DevCounters>();
    uint32_t* status = &ctr->status;
    MDMC_CHECK(c, cudaMemsetAsync(ctr, 0, sizeof(DevCounters), s));
    GridDesc g;
    mdmc_status st = makeGridDesc(c, grid, iso, g, s);
    if (st != MDMC_OK) return st;
    int64_t numWords = 0, A = 0;
    int W = 0;
    if ((st = activeCells(c, g, iso, W, numWords, A, s)) != MDMC_OK) return st;
    if (A > 0) {
        // intersected edges: bit 3x + axis of the words of sample row (y, z)
        const int W3 = (3 * X + 31) / 32;
        const int64_t nE = (int64_t)Y * Z * W3;
        MDMC_CHECK(c, c->mcEdgeMask.ensure(sizeof(uint32_t) * (size_t)nE));
        MDMC_CHECK(c, c->mcEdgeFirst.ensure(sizeof(int) * (size_t)(nE + 1)));
        MDMC_CHECK(c, c->mcCases.ensure((size_t)A));
        MDMC_CHECK(c, c->mcTriOffset.ensure(sizeof(int) * (size_t)(A + 1)));
        MDMC_CHECK(c, cudaMemsetAsync(c->mcEdgeMask.p, 0, sizeof(uint32_t) * (size_t)nE, s));
        launchMCMarkEdges(g, iso, c->cellIds.as<uint32_t>(), (int)A, W3, c->mcEdgeMask.as<uint32_t>(),
                          c->mcCases.as<uint8_t>(), c->mcTriOffset.as<int>(), status, s);
        if ((st = scanPopc(c, c->mcEdgeMask.as<uint32_t>(), c->mcEdgeFirst.as<int>(), nE, s)) != MDMC_OK) return st;
        if ((st = scan<int>(c, c->mcTriOffset.as<int>(), c->mcTriOffset.as<int>(), A, s)) != MDMC_OK) return st;
        MDMC_CHECK(c, cudaGetLastError());
        if ((st = readInts(c, c->mcEdgeFirst.as<int>() + nE, 1, s)) != MDMC_OK) return st;
        const int64_t V = c->hostInts[0];
        if ((st = readInts(c, c->mcTriOffset.as<int>() + A, 1, s)) != MDMC_OK) return st;
        const int64_t T = c->hostInts[0];
        if (V < 3 || V > 12 * A || T < 1 || T > 5 * A)
            return fail(c, MDMC_ERROR_CUDA, "inconsistent vertex or triangle count from the edge pass");
        MDMC_CHECK(c, c->mcEdgeIds.ensure(sizeof(uint32_t) * (size_t)V));
        MDMC_CHECK(c, c->mcPos.ensure(sizeof(float) * 3 * (size_t)V));
        MDMC_CHECK(c, c->mcNrm.ensure(sizeof(float) * 3 * (size_t)V));
        MDMC_CHECK(c, c->mcTris.ensure(sizeof(int) * 3 * (size_t)T));
        launchMCScatterEdges(c->mcEdgeMask.as<uint32_t>(), c->mcEdgeFirst.as<int>(), nE, W3, X,
                             c->mcEdgeIds.as<uint32_t>(), (int)V, status, s);
        launchMCVertices(g, iso, c->mcEdgeIds.as<uint32_t>(), (int)V, c->mcPos.as<float>(), c->mcNrm.as<float>(), s);
        launchMCTriangles(c->cellIds.as<uint32_t>(), c->mcCases.as<uint8_t>(), c->mcTriOffset.as<int>(), (int)A, X, Y, W3,
                          c->mcEdgeMask.as<uint32_t>(), c->mcEdgeFirst.as<int>(), nE, c->mcTris.as<int>(), (int)T, status,
                          s);
        MDMC_CHECK(c, cudaGetLastError());
        c->mcV = V;
        c->mcT = T;
    }
    MDMC_CHECK(c, cudaMemcpyAsync(c->hostCounters, ctr, sizeof(DevCounters), cudaMemcpyDeviceToHost, s));
    MDMC_CHECK(c, cudaStreamSynchronize(s));
    if (mesh) {
        mesh->num_vertices = c->mcV;
        mesh->num_triangles = c->mcT;
        mesh->positions = c->mcPos.as<float>();
        mesh->normals = c->mcNrm.as<float>();
        mesh->triangles = c->mcTris.as<int32_t>();
    }
    const uint32_t hs = c->hostCounters->status;
    if (hs) {
        c->err = "device limits hit: " + statusText(hs);
        return MDMC_ERROR_LIMIT;
    }
    return MDMC_OK;
}

mdmc_status mdmc_download_triangle_mesh(mdmc_context* c, float* positions, float* normals, int32_t* triangles,
                                        void* stream) {
    if (!c) return MDMC_ERROR_INVALID_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    if (positions && c->mcV)
        MDMC_CHECK(c, cudaMemcpyAsync(positions, c->mcPos.p, sizeof(float) * 3 * (size_t)c->mcV, cudaMemcpyDeviceToHost, s));
    if (normals && c->mcV)
        MDMC_CHECK(c, cudaMemcpyAsync(normals, c->mcNrm.p, sizeof(float) * 3 * (size_t)c->mcV, cudaMemcpyDeviceToHost, s));
    if (triangles && c->mcT)
        MDMC_CHECK(c, cudaMemcpyAsync(triangles, c->mcTris.p, sizeof(int) * 3 * (size_t)c->mcT, cudaMemcpyDeviceToHost, s));
    MDMC_CHECK(c, cudaStreamSynchronize(s));
    return MDMC_OK;
}

mdmc_status mdmc_get_mesh(const mdmc_context* c, mdmc_mesh* m) {
    if (!c || !m) return MDMC_ERROR_INVALID_ARGUMENT;
    std::memset(m, 0, sizeof *m);
    if (!c->haveMesh) return MDMC_ERROR_INVALID_ARGUMENT;
    m->num_vertices = c->V;
    m->num_faces = c->F;
    m->num_halfedges = c->H;
    m->positions = c->pos.as<float>();
    m->normals = c->nrm.as<float>();
    m->quads = c->quads.as<int32_t>();
    m->halfedges = c->he.as<int32_t>();
    m->face_first_halfedge = c->faceFirst.as<int32_t>();
    m->face_attributes = c->faceAttr.as<uint16_t>();
    m->vertex_halfedge = c->vertexHE.as<int32_t>();
    m->vertex_flags = c->vflags.as<uint8_t>();
    return MDMC_OK;
}

mdmc_status mdmc_get_stats(const mdmc_context* c, mdmc_stats* stats) {
    if (!c || !stats) return MDMC_ERROR_INVALID_ARGUMENT;
    *stats = c->stats;
    return MDMC_OK;
}

mdmc_status mdmc_download_mesh(mdmc_context* c, float* positions, float* normals, int32_t* quads, int32_t* halfedges,
                               int32_t* face_first_halfedge, uint16_t* face_attributes, int32_t* vertex_halfedge,
                               uint8_t* vertex_flags, void* stream) {
    if (!c || !c->haveMesh) return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "no mesh");
    cudaStream_t s = (cudaStream_t)stream;
    auto cp = [&](void* dst, const DevBuf& b, size_t bytes) -> cudaError_t {
        if (!dst || bytes == 0) return cudaSuccess;
        return cudaMemcpyAsync(dst, b.p, bytes, cudaMemcpyDeviceToHost, s);
    };
    MDMC_CHECK(c, cp(positions, c->pos, sizeof(float) * 3 * (size_t)c->V));
    MDMC_CHECK(c, cp(normals, c->nrm, sizeof(float) * 3 * (size_t)c->V));
    MDMC_CHECK(c, cp(quads, c->quads, sizeof(int4) * (size_t)c->F));
    MDMC_CHECK(c, cp(halfedges, c->he, sizeof(int4) * (size_t)c->H));
    MDMC_CHECK(c, cp(face_first_halfedge, c->faceFirst, sizeof(int) * (size_t)c->F));
    MDMC_CHECK(c, cp(face_attributes, c->faceAttr, sizeof(uint16_t) * (size_t)c->F));
    MDMC_CHECK(c, cp(vertex_halfedge, c->vertexHE, sizeof(int) * (size_t)c->V));
    MDMC_CHECK(c, cp(vertex_flags, c->vflags, (size_t)c->V));
    MDMC_CHECK(c, cudaStreamSynchronize(s));
    return MDMC_OK;
}

mdmc_status mdmc_run_to_host(mdmc_context* c, const mdmc_grid* grid, float iso, const mdmc_host_mesh* out,
                             mdmc_mesh* mesh, mdmc_stats* stats, void* stream) {
    if (!c || !grid || !out || out->capacity_vertices < 0 || out->capacity_faces < 0)
        return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "null argument or negative capacity");
    cudaStream_t s = (cudaStream_t)stream;
    c->hostOut = out;
    const mdmc_status st = mdmc_run(c, grid, iso, mesh, stats, stream);
    c->hostOut = nullptr;
    // the early copies write the caller's arrays: they end before this call does
    const cudaError_t ce = cudaStreamSynchronize(c->copyStream);
    if (st != MDMC_OK && st != MDMC_ERROR_LIMIT) return st;
    if (ce != cudaSuccess) return cudaFail(c, ce, "early copies");
    const std::string runMessage = c->err;
    if (c->V > out->capacity_vertices || c->F > out->capacity_faces) {
        char text[200];
        std::snprintf(text, sizeof text, "the mesh has %lld vertices and %lld faces; the host arrays hold %lld and %lld",
                      (long long)c->V, (long long)c->F, (long long)out->capacity_vertices,
                      (long long)out->capacity_faces);
        return fail(c, MDMC_ERROR_LIMIT, text);
    }
    auto cp = [&](void* dst, const DevBuf& b, size_t bytes) -> cudaError_t {
        if (!dst || bytes == 0) return cudaSuccess;
        return cudaMemcpyAsync(dst, b.p, bytes, cudaMemcpyDeviceToHost, s);
    };
    if (!c->earlyFaces || c->lateChange || c->simplified) {
        MDMC_CHECK(c, cp(out->halfedges, c->he, sizeof(int4) * (size_t)c->H));
        MDMC_CHECK(c, cp(out->quads, c->quads, sizeof(int4) * (size_t)c->F));
        MDMC_CHECK(c, cp(out->face_first_halfedge, c->faceFirst, sizeof(int) * (size_t)c->F));
        MDMC_CHECK(c, cp(out->face_attributes, c->faceAttr, sizeof(uint16_t) * (size_t)c->F));
    }
    if (!c->earlyVertices || c->lateChange || c->simplified) {
        MDMC_CHECK(c, cp(out->positions, c->pos, sizeof(float) * 3 * (size_t)c->V));
        MDMC_CHECK(c, cp(out->normals, c->nrm, sizeof(float) * 3 * (size_t)c->V));
    }
    if (!c->earlyVertexMaps || c->lateChange || c->simplified) {
        MDMC_CHECK(c, cp(out->vertex_halfedge, c->vertexHE, sizeof(int) * (size_t)c->V));
        MDMC_CHECK(c, cp(out->vertex_flags, c->vflags, (size_t)c->V));
    }
    MDMC_CHECK(c, cudaStreamSynchronize(s));
    c->err = runMessage;
    return st;
}

mdmc_status mdmc_backward(mdmc_context* c, const float* dl_dpositions, float* dl_dsamples, int accumulate,
                          void* stream) {
    if (!c || !dl_dsamples || (!dl_dpositions && c->V > 0)) return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "null argument");
    c->err.clear();
    (void)cudaGetLastError();
    if (!c->haveMesh) return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "no forward run to differentiate");
    if (c->lastSurfaceIteration)
        return fail(c, MDMC_ERROR_INVALID_ARGUMENT,
                    "the adjoint needs a forward run with enable_surface_to_vertex_iteration = 0");
    if (c->simplified)
        return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "the adjoint is not defined after a simplification pass");
    cudaStream_t s = (cudaStream_t)stream;
    const mdmc_grid& grid = c->lastGrid;
    GridDesc g;
    mdmc_status st = makeGridDesc(c, &grid, c->lastIso, g, s, false);
    if (st != MDMC_OK) return st;
    const int64_t outCount = g.refined ? (int64_t)grid.coarse_dims[0] * grid.coarse_dims[1] * grid.coarse_dims[2]
                                       : (int64_t)grid.dims[0] * grid.dims[1] * grid.dims[2];
    if (!accumulate) MDMC_CHECK(c, cudaMemsetAsync(dl_dsamples, 0, sizeof(float) * (size_t)outCount, s));
    if (c->dmcV == 0) return MDMC_OK;
    MDMC_CHECK(c, c->vertexGrad.ensure(sizeof(float) * 3 * (size_t)c->dmcV));
    MDMC_CHECK(c, cudaMemcpyAsync(c->vertexGrad.p, dl_dpositions, sizeof(float) * 3 * (size_t)c->dmcV,
                                  cudaMemcpyDeviceToDevice, s));
    launchGatherParents(dl_dpositions, (int)c->V, (int)c->dmcV, c->appParent.as<int>(), c->vertexGrad.as<float>(), s);
    DevCounters* ctr = c->counters.as<DevCounters>();
    MDMC_CHECK(c, cudaMemsetAsync(&ctr->status, 0, sizeof(uint32_t), s));
    launchBackwardCells(g, c->lastIso, c->act.as<ActiveCell>(), (int)c->activeCells, c->vertexGrad.as<float>(),
                        (int)c->dmcV, dl_dsamples, &ctr->status, s);
    MDMC_CHECK(c, cudaGetLastError());
    return MDMC_OK;
}

mdmc_status mdmc_render_buffers(mdmc_context* c, float* vertices, uint32_t* indices, void* stream) {
    if (!c) return MDMC_ERROR_INVALID_ARGUMENT;
    c->err.clear();
    (void)cudaGetLastError();
    if (!c->haveMesh) return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "no mesh: run first");
    launchRenderBuffers(c->pos.as<float>(), c->nrm.as<float>(), c->vflags.as<uint8_t>(), c->vertexHE.as<int>(),
                        (int)c->V, c->quads.as<int4>(), (int)c->F, vertices, indices, (cudaStream_t)stream);
    MDMC_CHECK(c, cudaGetLastError());
    return MDMC_OK;
}

mdmc_status mdmc_color_faces(mdmc_context* c, void* stream) {
    if (!c) return MDMC_ERROR_INVALID_ARGUMENT;
    c->err.clear();
    (void)cudaGetLastError();
    if (!c->haveMesh) return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "no mesh: run first");
    if (c->F == 0) return MDMC_OK;
    MDMC_CHECK(c, c->colorOrig.ensure((size_t)c->F));
    launchColorFaces(c->he.as<int4>(), c->faceFirst.as<int>(), c->faceAttr.as<uint16_t>(), c->colorOrig.as<uint8_t>(),
                     (int)c->F, (int)c->H, (cudaStream_t)stream);
    MDMC_CHECK(c, cudaGetLastError());
    return MDMC_OK;
}

mdmc_status mdmc_write_bin(const char* path, const int32_t dims[3], const float spacing[3], const float* host_samples) {
    if (!path || !dims || !spacing || !host_samples || dims[0] < 1 || dims[1] < 1 || dims[2] < 1)
        return MDMC_ERROR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "wb");
    if (!f) return MDMC_ERROR_IO;
    bool ok = std::fwrite(dims, sizeof(int32_t), 3, f) == 3 && std::fwrite(spacing, sizeof(float), 3, f) == 3;
    const size_t n = (size_t)dims[0] * dims[1] * dims[2];
    std::vector<uint16_t> buf(std::min<size_t>(n, (size_t)1 << 20));
    for (size_t i = 0; ok && i < n; i += buf.size()) {
        const size_t m = std::min(buf.size(), n - i);
        for (size_t k = 0; k < m; ++k) {
            // static_cast<unsigned short>(float): truncation; out-of-range values clamp here
            const float v = host_samples[i + k];
            buf[k] = v != v || v <= 0.f ? 0 : (v >= 65535.f ? 65535 : (uint16_t)v);
        }
        ok = std::fwrite(buf.data(), sizeof(uint16_t), m, f) == m;
    }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? MDMC_OK : MDMC_ERROR_IO;
}

mdmc_status mdmc_write_obj(mdmc_context* c, const char* path) {
    if (!c || !path || !c->haveMesh) return fail(c, MDMC_ERROR_INVALID_ARGUMENT, "no mesh or path");
    std::vector<float> p(3 * (size_t)c->V), n(3 * (size_t)c->V);
    std::vector<int32_t> q(4 * (size_t)c->F);
    mdmc_status st = mdmc_download_mesh(c, p.data(), n.data(), q.data(), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    if (st != MDMC_OK) return st;
    FILE* f = std::fopen(path, "w");
    if (!f) return fail(c, MDMC_ERROR_IO, std::string("cannot open ") + path);
    // iostream's default float output: %g with 6 significant digits
    for (int64_t v = 0; v < c->V; ++v) std::fprintf(f, "v %g %g %g\n", p[3 * v], p[3 * v + 1], p[3 * v + 2]);
    for (int64_t v = 0; v < c->V; ++v) std::fprintf(f, "vn %g %g %g\n", n[3 * v], n[3 * v + 1], n[3 * v + 2]);
    for (int64_t i = 0; i < c->F; ++i) {
        const int a = q[4 * i] + 1, b = q[4 * i + 1] + 1, d = q[4 * i + 2] + 1, e = q[4 * i + 3] + 1;
        std::fprintf(f, "f %d//%d %d//%d %d//%d %d//%d\n", a, a, b, b, d, d, e, e);
    }
    std::fclose(f);
    return MDMC_OK;
}

const char* mdmc_last_error(const mdmc_context* c) { return c ? c->err.c_str() : "null context"; }

void mdmc_case_tables(uint64_t contour_words[256], uint8_t ambiguous[256]) {
    for (int i = 0; i < 256; ++i) {
        if (contour_words) contour_words[i] = kContourTableHost[i];
        if (ambiguous) ambiguous[i] = caseIsAmbiguous(i) ? 1 : 0;
    }
}

}  // extern "C"
