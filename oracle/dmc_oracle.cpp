// CPU oracle for the Dual Marching Cubes + manifold repair path.
//
// TEST INFRASTRUCTURE ONLY: a sequential restatement of the reference's
// algorithm (PhiliGuertler/ManifoldDMC, MarchingCubes/VisualDMC/src/DMC/) used
// by the tests, the smoke test and the CPU-baseline leg of bench.py to check
// the CUDA path.  Every function cites the reference lines it follows.
// Compiled with -ffp-contract=off so that each float operation is rounded as
// written; the CUDA path is built with -fmad=false and the same operation
// order, so the two agree bit for bit.
//
// Parity pin: checked against the reference's golden meshes in
// tests/test_oracle_golden.py.

#include "dmc_oracle.h"
#include "mc_contour_table_oracle.h"
#include "mc_triangle_table_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <unordered_map>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <vector>

namespace oracle {

// The arithmetic type of the restatement: float (the default, bit for bit
// the CUDA path's operations) or, with -DMDMC_ORACLE_REAL=double, the FP64
// form of the same algorithm that is timed as the CPU baseline.  Input
// samples and the C API stay float in both.
#ifndef MDMC_ORACLE_REAL
#define MDMC_ORACLE_REAL float
#endif
typedef MDMC_ORACLE_REAL Real;

// ------------------------------------------------------------------------ //
// small float vector helpers, each operation rounded once (glm semantics)
// ------------------------------------------------------------------------ //
struct V3 {
    Real x, y, z;
};
static inline V3 v3(Real x, Real y, Real z) { return {x, y, z}; }
static inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 mul(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
static inline V3 muls(V3 a, Real s) { return {a.x * s, a.y * s, a.z * s}; }
static inline V3 smul(Real s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
static inline V3 divv(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
static inline V3 divs(V3 a, Real s) { return {a.x / s, a.y / s, a.z / s}; }
static inline Real gmin(Real x, Real y) { return (y < x) ? y : x; }  // glm::min
static inline Real gmax(Real x, Real y) { return (x < y) ? y : x; }  // glm::max
static inline Real gclamp(Real x, Real lo, Real hi) { return gmin(gmax(x, lo), hi); }
// glm::normalize: v * (1 / sqrt(dot(v, v))), dot = (x*x + y*y) + z*z
static inline V3 normalize(V3 v) {
    Real d = v.x * v.x + v.y * v.y;
    d = d + v.z * v.z;
    Real inv = 1.0f / std::sqrt(d);
    return muls(v, inv);
}

static const Real kEpsilon = 0.0001f;  // LazyEngine::Constants::EPSILON

// ------------------------------------------------------------------------ //
// Grid, D/UniformGrid.h:44-130
// ------------------------------------------------------------------------ //
struct Grid {
    int d[3];
    Real origin[3];
    Real deltas[3];
    const Real* v;
    inline Real at(int x, int y, int z) const {
        return v[(size_t)z * d[0] * d[1] + (size_t)y * d[0] + x];
    }
    inline Real atClamped(int x, int y, int z) const {
        x = x < 0 ? 0 : (x > d[0] - 1 ? d[0] - 1 : x);
        y = y < 0 ? 0 : (y > d[1] - 1 ? d[1] - 1 : y);
        z = z < 0 ? 0 : (z > d[2] - 1 ? d[2] - 1 : z);
        return at(x, y, z);
    }
    V3 o() const { return v3(origin[0], origin[1], origin[2]); }
    V3 dl() const { return v3(deltas[0], deltas[1], deltas[2]); }
};

// Interpolation<float>::interpolateTrilinearly, D/Utils/Interpolation.inl:76-84
static inline Real trilinear(const Real s[8], V3 p) {
    Real a = s[0] + p.x * (s[1] - s[0]);
    Real b = s[2] + p.x * (s[3] - s[2]);
    Real c = s[4] + p.x * (s[5] - s[4]);
    Real e = s[6] + p.x * (s[7] - s[6]);
    Real lo = (1.f - p.y) * a + p.y * b;
    Real hi = (1.f - p.y) * c + p.y * e;
    return (1.f - p.z) * lo + p.z * hi;
}
static inline V3 trilinear3(const V3 s[8], V3 p) {
    Real xs[8], ys[8], zs[8];
    for (int i = 0; i < 8; ++i) { xs[i] = s[i].x; ys[i] = s[i].y; zs[i] = s[i].z; }
    return v3(trilinear(xs, p), trilinear(ys, p), trilinear(zs, p));
}

// UniformGrid::evaluateCellCornerValues, D/UniformGrid.inl:414-427
static inline void cornerValues(const Grid& g, int x, int y, int z, Real s[8]) {
    for (int i = 0; i < 8; ++i) s[i] = g.atClamped(x + (i & 1), y + ((i >> 1) & 1), z + ((i >> 2) & 1));
}

// ------------------------------------------------------------------------ //
// refineGrid, D/UniformGrid.inl:279-319 (+ host geometry :575-608)
// ------------------------------------------------------------------------ //
static void refine(const Grid& in, int r, bool pad, std::vector<Real>& out, int od[3], Real oo[3],
                   Real odl[3]) {
    for (int a = 0; a < 3; ++a) {
        od[a] = in.d[a] + (in.d[a] - 1) * r + (pad ? 2 : 0);
        odl[a] = (in.deltas[a] * 1.f) / ((Real)r + 1.f);
        oo[a] = in.origin[a];
        if (pad) oo[a] = oo[a] - odl[a];
    }
    out.assign((size_t)od[0] * od[1] * od[2], 0.f);
    const Real f = (Real)(r + 1);
#pragma omp parallel for schedule(static)
    for (int z = 0; z < od[2]; ++z)
        for (int y = 0; y < od[1]; ++y)
            for (int x = 0; x < od[0]; ++x) {
                int ix = x, iy = y, iz = z;
                if (pad) {
                    ix = std::min(std::max(ix, 1), od[0] - 2) - 1;
                    iy = std::min(std::max(iy, 1), od[1] - 2) - 1;
                    iz = std::min(std::max(iz, 1), od[2] - 2) - 1;
                }
                Real qx = (Real)ix / f, qy = (Real)iy / f, qz = (Real)iz / f;
                int mx = (int)std::floor(qx), my = (int)std::floor(qy), mz = (int)std::floor(qz);
                V3 diff = v3(qx - (Real)mx, qy - (Real)my, qz - (Real)mz);
                Real s[8];
                cornerValues(in, mx, my, mz, s);
                out[(size_t)z * od[0] * od[1] + (size_t)y * od[0] + x] = trilinear(s, diff);
            }
}

// ------------------------------------------------------------------------ //
// Cell intersection, D/CellIntersection.{h,inl}
// ------------------------------------------------------------------------ //
// corner pair of each cell edge (EdgeVertices table, D/CellIntersection.inl:383)
static const int kEdgeV0[12] = {0, 1, 2, 0, 4, 5, 6, 4, 0, 1, 3, 2};
static const int kEdgeV1[12] = {1, 3, 3, 2, 5, 7, 7, 6, 4, 5, 7, 6};
// axis of each edge: 0 = x, 1 = y, 2 = z (computeGlobalIndex's offs)
static const int kEdgeAxis[12] = {0, 1, 0, 1, 0, 1, 0, 1, 2, 2, 2, 2};

static inline int nib(uint64_t w, int i) { return (int)((w >> (4 * i)) & 0xF); }
static inline int contourSize(uint64_t c, int t) { return nib(c, t); }
static inline int contourEdgeBit(uint64_t c, int t, int pos) {
    int before = 0;
    for (int k = 0; k < t; ++k) before += nib(c, k);
    return 16 + 4 * (before + pos);
}
static inline int contourEdge(uint64_t c, int t, int pos) {
    return (int)((c >> contourEdgeBit(c, t, pos)) & 0xF);
}
static inline void setContourEdge(uint64_t& c, int t, int pos, int e) {
    int b = contourEdgeBit(c, t, pos);
    c &= ~(0xFULL << b);
    c |= (uint64_t)e << b;
}
static inline void setContourSize(uint64_t& c, int t, int n) {
    c &= ~(0xFULL << (4 * t));
    c |= (uint64_t)n << (4 * t);
}

// faces of the cell: edges and corners in the flattened orientation
// (D/CellIntersection.inl:290-292)
static const unsigned short kFaceEdges[6] = {0x0123, 0x4765, 0x4908, 0x2A6B, 0x83B7, 0x95A1};
static const unsigned short kFaceCorners[6] = {0x3120, 0x6475, 0x1504, 0x7362, 0x2064, 0x7531};

// Whether a case takes the asymptotic-decider path: the reference marks a
// case MC_AMBIGUOUS (D/DualMarchingCubes.cpp:301) exactly when one of its
// faces has the diagonal sign pattern, or when its only two (or six) inside
// corners are opposite ends of a cell diagonal.
bool caseIsAmbiguous(int c) {
    for (int f = 0; f < 6; ++f) {
        int fc = 0;
        for (int i = 0; i < 4; ++i) fc |= ((c >> nib(kFaceCorners[f], i)) & 1) << i;
        if (fc == 6 || fc == 9) return true;
    }
    for (int i = 0; i < 4; ++i) {
        int pair = (1 << i) | (1 << (7 - i));
        if (c == pair || c == (255 ^ pair)) return true;
    }
    return false;
}

// marchingCubesAsymptoticPolygon, D/CellIntersection.inl:202-338
static uint64_t asymptoticContours(const Real s[8], Real iso, int& numContours) {
    unsigned char seg[12];
    for (int i = 0; i < 12; ++i) seg[i] = 0xFF;
    auto connect = [&](int in, int out) {
        seg[in] = (unsigned char)((seg[in] & 0xF0) | (out & 0xF));
        seg[out] = (unsigned char)((seg[out] & 0x0F) | (in << 4));
    };
    for (int f = 0; f < 6; ++f) {
        int e[4];
        Real val[4];
        unsigned fc = 0;
        for (int i = 0; i < 4; ++i) {
            int v = nib(kFaceCorners[f], i);
            e[i] = nib(kFaceEdges[f], i);
            val[i] = s[v];
            fc |= (unsigned)(val[i] >= iso) << i;
        }
        switch (fc) {
            case 1: connect(e[0], e[3]); break;
            case 2: connect(e[1], e[0]); break;
            case 3: connect(e[1], e[3]); break;
            case 4: connect(e[3], e[2]); break;
            case 5: connect(e[0], e[2]); break;
            case 7: connect(e[1], e[2]); break;
            case 8: connect(e[2], e[1]); break;
            case 10: connect(e[2], e[0]); break;
            case 11: connect(e[2], e[3]); break;
            case 12: connect(e[3], e[1]); break;
            case 13: connect(e[0], e[1]); break;
            case 14: connect(e[3], e[0]); break;
            case 6:
            case 9: {
                // (a*d - b*c) / (a + d - b - c)
                Real num = val[0] * val[3] - val[1] * val[2];
                Real den = val[0] + val[3];
                den = den - val[1];
                den = den - val[2];
                Real decision = num / den;
                if (fc == 6) {
                    if (decision >= iso) { connect(e[3], e[0]); connect(e[1], e[2]); }
                    else { connect(e[1], e[0]); connect(e[3], e[2]); }
                } else {
                    if (decision >= iso) { connect(e[0], e[1]); connect(e[2], e[3]); }
                    else { connect(e[0], e[3]); connect(e[2], e[1]); }
                }
            } break;
            default: break;
        }
    }
    uint64_t c = 0xFFFFFFFFFFFF0000ULL;
    int n = 0;
    for (int edge = 0; edge < 12; ++edge) {
        if (seg[edge] == 0xFF) continue;
        int start = edge;
        int out = seg[edge] & 0xF;
        int pos = 0;
        setContourEdge(c, n, pos, start);
        int guard = 0;
        while (out != start && guard < 12) {  // a closed contour has <= 12 edges
            ++pos;
            setContourEdge(c, n, pos, out);
            int in = out;
            out = (in < 12) ? (seg[in] & 0xF) : start;
            if (in < 12) seg[in] = 0xFF;
            ++guard;
        }
        setContourSize(c, n, pos + 1);
        ++n;
    }
    numContours = n;
    return c;
}

static uint64_t cellContours(int cs, const Real s[8], Real iso, int& n) {
    if (caseIsAmbiguous(cs)) return asymptoticContours(s, iso, n);
    uint64_t c = kContourTable[cs];
    n = 0;
    for (int t = 0; t < 4; ++t) if (nib(c, t) > 0) n = t + 1;
    return c;
}

// UniformGrid::computeGradients, D/UniformGrid.inl:325-379
static void cornerGradients(const Grid& g, int x, int y, int z, const Real s[8], V3 out[8]) {
    auto cl = [](int dim, int ii) { return ii < 0 ? 0 : (ii >= dim ? dim - 1 : ii); };
    const int X = g.d[0], Y = g.d[1], Z = g.d[2];
    V3 gr[8];
    gr[0] = v3(s[1] - g.at(cl(X, x - 1), y, z), s[2] - g.at(x, cl(Y, y - 1), z), s[4] - g.at(x, y, cl(Z, z - 1)));
    gr[1] = v3(g.at(cl(X, x + 2), y, z) - s[0], s[3] - g.at(x + 1, cl(Y, y - 1), z),
               s[5] - g.at(x + 1, y, cl(Z, z - 1)));
    gr[2] = v3(s[3] - g.at(cl(X, x - 1), y + 1, z), g.at(x, cl(Y, y + 2), z) - s[0],
               s[6] - g.at(x, y + 1, cl(Z, z - 1)));
    gr[3] = v3(g.at(cl(X, x + 2), y + 1, z) - s[2], g.at(x + 1, cl(Y, y + 2), z) - s[1],
               s[7] - g.at(x + 1, y + 1, cl(Z, z - 1)));
    gr[4] = v3(s[5] - g.at(cl(X, x - 1), y, z + 1), s[6] - g.at(x, cl(Y, y - 1), z + 1),
               g.at(x, y, cl(Z, z + 2)) - s[0]);
    gr[5] = v3(g.at(cl(X, x + 2), y, z + 1) - s[4], s[7] - g.at(x + 1, cl(Y, y - 1), z + 1),
               g.at(x + 1, y, cl(Z, z + 2)) - s[1]);
    gr[6] = v3(s[7] - g.at(cl(X, x - 1), y + 1, z + 1), g.at(x, cl(Y, y + 2), z + 1) - s[4],
               g.at(x, y + 1, cl(Z, z + 2)) - s[2]);
    gr[7] = v3(g.at(cl(X, x + 2), y + 1, z + 1) - s[6], g.at(x + 1, cl(Y, y + 2), z + 1) - s[5],
               g.at(x + 1, y + 1, cl(Z, z + 2)) - s[3]);
    V3 dl = g.dl();
    for (int i = 0; i < 8; ++i) out[i] = divv(smul(0.5f, gr[i]), dl);
}

// VertexToSurfaceIterator, D/CellIntersection.inl:12-122
struct SurfaceIterator {
    const Real* s;
    Real iso;
    Real step = 0.05f;
    int maxIter = 30;

    V3 gradient(V3 p) const {
        Real gx = (1 - p.z) * ((1 - p.y) * (s[1] - s[0]) + p.y * (s[3] - s[2])) +
                   p.z * ((1 - p.y) * (s[5] - s[4]) + p.y * (s[7] - s[6]));
        Real gy = (1 - p.z) * ((1 - p.x) * (s[2] - s[0]) + p.x * (s[3] - s[1])) +
                   p.z * ((1 - p.x) * (s[6] - s[4]) + p.x * (s[7] - s[5]));
        Real gz = (1 - p.y) * ((1 - p.x) * (s[4] - s[0]) + p.x * (s[5] - s[1])) +
                   p.y * ((1 - p.x) * (s[6] - s[2]) + p.x * (s[7] - s[3]));
        return v3(gx, gy, gz);
    }
    // updateGradient, :83-122; returns breakNow, sets clamp flags
    bool update(V3& point, V3& grad, const V3& in1, V3& in2, Real v1, Real& v2, bool clamped[3]) const {
        grad = normalize(grad);
        in2 = add(in1, smul(step, grad));
        clamped[0] = in2.x <= 0.f || in2.x >= 1.f;
        clamped[1] = in2.y <= 0.f || in2.y >= 1.f;
        clamped[2] = in2.z <= 0.f || in2.z >= 1.f;
        in2 = v3(gclamp(in2.x, 0.f, 1.f), gclamp(in2.y, 0.f, 1.f), gclamp(in2.z, 0.f, 1.f));
        v2 = trilinear(s, in2);
        if ((v1 <= iso && iso <= v2) || (v2 <= iso && iso <= v1)) {
            Real e = v1;
            if (v1 != v2) e = (iso - v1) / (v2 - v1);
            point = add(in1, smul(e, sub(in2, in1)));
            return true;
        }
        return false;
    }
    void move(V3& point) const {
        V3 in1 = point;
        Real v1 = trilinear(s, in1);
        Real v2 = 0.f;
        for (int i = 0; i < maxIter; ++i) {
            V3 g = gradient(in1);
            if (v1 > iso) g = v3(-g.x, -g.y, -g.z);
            V3 in2 = in1;
            bool cl[3];
            if (update(point, g, in1, in2, v1, v2, cl)) break;
            if (cl[0] || cl[1] || cl[2]) {
                if (cl[0]) g.x = 0.f;
                else if (cl[1]) g.y = 0.f;
                else g.z = 0.f;
                bool cl2[3];
                if (update(point, g, in1, in2, v1, v2, cl2)) break;
            }
            in1 = in2;
            v1 = v2;
        }
        const Real lo = kEpsilon, hi = 1.f - kEpsilon;
        point = v3(gclamp(point.x, lo, hi), gclamp(point.y, lo, hi), gclamp(point.z, lo, hi));
    }
};

// computeVertexPosition, D/CellIntersection.inl:361-366
static inline int quadSlot(int e, int edgyBit) {
    const unsigned long long t = 240177437832960ULL;
    return (int)((t >> (4 * e + 2 * edgyBit)) & 3);
}

// ------------------------------------------------------------------------ //
// Halfedge mesh
// ------------------------------------------------------------------------ //
struct HE {
    int origin, face, next, twin;
};

// QuadrilateralAttribute bits, D/DeviceVectors.h:334-450
static const uint16_t kAttrInvalidColor = 0x1F;
static const uint16_t kAttrNonManifold = 0x20;
// vertex Flags bits, D/Halfedges/Halfedge.h:14-111
static const uint8_t kFlagNonManifold = 1, kFlagBoundary = 2, kFlagWeird = 4, kFlagMultiFan = 8,
                     kFlagRemove = 16;

// anomaly bits (same meaning and values as the CUDA path's status word)
enum : uint32_t {
    kSSlot = 1u << 1, kSBucket = 1u << 2, kSPartner = 1u << 3, kSWalk = 1u << 4, kSBadTwin = 1u << 5,
    kSIterCap = 1u << 6, kSWall = 1u << 7, kSMapping = 1u << 9
};

struct Bucket {
    int count = 0;
    int ids[4] = {-1, -1, -1, -1};
};

// concatenateKeys, D/Utils/Utilities.h:15-22
static inline uint64_t edgeKey(int a, int b) {
    if (a < b) return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b;
    return ((uint64_t)(uint32_t)b << 32) | (uint32_t)a;
}

struct Result {
    // DMC stage
    std::vector<Real> dmcPos, dmcNrm;
    std::vector<int> dmcQuads;
    std::vector<uint16_t> dmcAttr;
    // per DMC vertex: its cell (3 ints) and the cell edges of its contour (12-bit mask)
    std::vector<int> dmcCell;
    std::vector<uint16_t> dmcEdges;
    // per final vertex: the DMC vertex it descends from (-1: none)
    std::vector<int> parent;
    // final mesh
    std::vector<Real> pos, nrm;  // 3 per vertex
    std::vector<HE> he;
    std::vector<int> faceFirst;
    std::vector<uint16_t> faceAttr;
    std::vector<uint8_t> vflags;
    std::vector<int> vertexHE;
    int64_t stats[MDMC_ORC_NUM_STATS];
};

struct EdgeTable {
    std::unordered_map<uint64_t, Bucket> map;
    uint32_t anomalies = 0;
    // keeps the 4 smallest ids of a bucket (the reference keeps the first 4
    // inserted, in atomic order); more than 4 faces on one edge is an anomaly
    void insert(int a, int b, int h) {
        Bucket& bk = map[edgeKey(a, b)];
        if (bk.count < 4) {
            bk.ids[bk.count] = h;
        } else {
            anomalies |= kSBucket;
            int* mx = std::max_element(bk.ids, bk.ids + 4);
            if (h < *mx) *mx = h;
        }
        ++bk.count;
    }
    void finish() {
        for (auto& kv : map) {
            int n = std::min(kv.second.count, 4);
            std::sort(kv.second.ids, kv.second.ids + n);
        }
    }
    int valence(int a, int b) const {
        auto it = map.find(edgeKey(a, b));
        return it == map.end() ? -1 : it->second.count;
    }
};

struct Mesh {
    std::vector<Real> pos, nrm;
    std::vector<HE> he;
    std::vector<int> faceFirst;
    std::vector<uint16_t> faceAttr;
    std::vector<uint8_t> vflags;
    std::vector<int> parent;  // DMC vertex each vertex descends from
    EdgeTable table;
    uint32_t anomalies = 0;

    int numV() const { return (int)(pos.size() / 3); }
    V3 P(int v) const { return v3(pos[3 * v], pos[3 * v + 1], pos[3 * v + 2]); }

    // refreshHashTableGPU, D/Halfedges/HalfedgeMesh.cu:62-90 (and the edge part
    // of collectHalfedgeElements, :55-59)
    void buildTable() {
        table = EdgeTable();
        for (size_t f = 0; f < faceFirst.size(); ++f) {
            int h = faceFirst[f];
            int q[4], hs[4];
            for (int i = 0; i < 4; ++i) {
                q[i] = he[h].origin;
                hs[i] = h;
                h = he[h].next;
            }
            for (int i = 0; i < 4; ++i) table.insert(q[i], q[(i + 1) & 3], hs[i]);
        }
        table.finish();
    }
    // refresh{NonManifold,Weird,Boundary}Flags, :92-148
    void vertexFlagsFromTable() {
        for (auto& kv : table.map) {
            const Bucket& b = kv.second;
            if (b.count == 4)
                for (int i = 0; i < 4; ++i) vflags[he[b.ids[i]].origin] |= kFlagNonManifold;
            if (b.count == 3)
                for (int i = 0; i < 3; ++i) vflags[he[b.ids[i]].origin] |= kFlagWeird;
            if (b.count == 1) vflags[he[b.ids[0]].origin] |= kFlagBoundary;
        }
    }
    // refreshFaceFlagsGPU, :150-171
    void faceFlagsFromTable() {
        for (auto& kv : table.map) {
            const Bucket& b = kv.second;
            if (b.count != 4) continue;
            for (int i = 0; i < 4; ++i) faceAttr[he[b.ids[i]].face] |= kAttrNonManifold;
        }
    }
    // connectHalfedgeTwins, :173-291
    void connectTwins() {
        for (auto& kv : table.map) {
            const Bucket& b = kv.second;
            const int* e = b.ids;
            switch (b.count) {
                case 2:
                    he[e[0]].twin = e[1];
                    he[e[1]].twin = e[0];
                    break;
                case 3:
                    he[e[0]].twin = e[1];
                    he[e[1]].twin = e[2];
                    he[e[2]].twin = e[0];
                    break;
                case 4: {
                    int v0 = he[e[0]].origin, v1 = he[e[1]].origin, v2 = he[e[2]].origin;
                    if (v0 != v1) {
                        he[e[0]].twin = e[1]; he[e[1]].twin = e[0];
                        he[e[2]].twin = e[3]; he[e[3]].twin = e[2];
                    } else if (v0 != v2) {
                        he[e[0]].twin = e[2]; he[e[2]].twin = e[0];
                        he[e[1]].twin = e[3]; he[e[3]].twin = e[1];
                    } else {
                        he[e[0]].twin = e[3]; he[e[3]].twin = e[0];
                        he[e[1]].twin = e[2]; he[e[2]].twin = e[1];
                    }
                    for (int i = 0; i < 4; ++i) faceAttr[he[e[i]].face] |= kAttrNonManifold;
                } break;
                default: break;
            }
        }
    }
    // HalfedgeMesh::refreshHashTable, :1063-1100
    void refresh() {
        buildTable();
        for (auto& a : faceAttr) a = (uint16_t)(a & 0x1F);  // clearPatternFlags + unset NM
        std::fill(vflags.begin(), vflags.end(), 0);
        vertexFlagsFromTable();
        faceFlagsFromTable();
    }
};

// ------------------------------------------------------------------------ //
// DMC stage: performDualMarchingCubes + mapQuadrilaterals,
// D/DualMarchingCubes.cu:38-85, sliceP D/CellIntersection.inl:368-439
// ------------------------------------------------------------------------ //
struct QuadEntry {
    int slot[4] = {-1, -1, -1, -1};
    int color = (int)kAttrInvalidColor;
};

// One z-slab of cells [z0, z1): vertices numbered from 0 within the slab,
// quad slots keyed by the global edge key.
struct SlabDMC {
    std::vector<Real> pos, nrm;
    std::vector<int> cells;
    std::vector<uint16_t> edgeMasks;
    std::unordered_map<uint64_t, QuadEntry> table;
    uint32_t anomalies = 0;
};

static void runDMCSlab(const Grid& g, Real iso, bool surfaceIteration, int z0, int z1, SlabDMC& out) {
    const int X = g.d[0], Y = g.d[1];
    V3 origin = g.o(), dl = g.dl();
    for (int z = z0; z < z1; ++z)
        for (int y = 0; y + 1 < Y; ++y)
            for (int x = 0; x + 1 < X; ++x) {
                Real s[8];
                cornerValues(g, x, y, z, s);
                int cs = 0;
                for (int i = 0; i < 8; ++i) cs |= (s[i] >= iso ? 1 : 0) << i;
                if (cs == 0 || cs == 255) continue;
                int n = 0;
                uint64_t c = cellContours(cs, s, iso, n);
                V3 normals[8];
                cornerGradients(g, x, y, z, s, normals);
                unsigned edgy = 0;
                for (int t = 0; t < n; ++t) {
                    int sz = contourSize(c, t);
                    V3 p = v3(0.f, 0.f, 0.f);
                    for (int i = 0; i < sz; ++i) {
                        int e = contourEdge(c, t, i);
                        int a0 = kEdgeV0[e], a1 = kEdgeV1[e];
                        Real w = (iso - s[a0]) / (s[a1] - s[a0]);
                        // computeLocalCoordinateOffset, :176-200: the edge's own
                        // axis gets the crossing, the others corner a0's coordinate
                        Real c0[3] = {(Real)(a0 & 1), (Real)((a0 >> 1) & 1), (Real)((a0 >> 2) & 1)};
                        c0[kEdgeAxis[e]] = w;
                        p = add(p, v3(c0[0], c0[1], c0[2]));
                        if (s[a0] < iso) edgy |= 1u << e;
                    }
                    p = divs(p, (Real)sz);
                    if (surfaceIteration) {
                        SurfaceIterator it{s, iso};
                        it.move(p);
                    }
                    V3 nm = normalize(trilinear3(normals, p));
                    V3 wp = add(origin, mul(add(v3((Real)x, (Real)y, (Real)z), p), dl));
                    int vid = (int)(out.pos.size() / 3);
                    out.pos.push_back(wp.x); out.pos.push_back(wp.y); out.pos.push_back(wp.z);
                    out.nrm.push_back(nm.x); out.nrm.push_back(nm.y); out.nrm.push_back(nm.z);
                    out.cells.push_back(x); out.cells.push_back(y); out.cells.push_back(z);
                    uint16_t mask = 0;
                    for (int i = 0; i < sz; ++i) mask |= (uint16_t)(1u << contourEdge(c, t, i));
                    out.edgeMasks.push_back(mask);
                    for (int i = 0; i < sz; ++i) {
                        int e = contourEdge(c, t, i);
                        int a0 = kEdgeV0[e];
                        int sx = x + (a0 & 1), sy = y + ((a0 >> 1) & 1), sz2 = z + ((a0 >> 2) & 1);
                        uint64_t key = 3ULL * ((uint64_t)sz2 * X * Y + (uint64_t)sy * X + sx) + kEdgeAxis[e];
                        int slot = quadSlot(e, (edgy >> e) & 1);
                        QuadEntry& q = out.table[key];
                        if (q.slot[slot] != -1) out.anomalies |= kSSlot;
                        q.slot[slot] = vid;
                        int base = (x & 1) | ((y & 1) << 1) | ((z & 1) << 2);
                        if (e == 0) q.color = 3 * base;
                        if (e == 3) q.color = 3 * base + 1;
                        if (e == 8) q.color = 3 * base + 2;
                    }
                }
            }
}

// performDualMarchingCubes + mapQuadrilaterals (D/DualMarchingCubes.cu:38-85):
// z-slabs in parallel (OpenMP), joined in slab order, so vertex ids follow
// the cells' (z, y, x) order as in a single pass
static void runDMC(const Grid& g, Real iso, bool surfaceIteration, std::vector<Real>& pos,
                   std::vector<Real>& nrm, std::vector<int>& quads, std::vector<uint16_t>& attr,
                   std::vector<int>& cells, std::vector<uint16_t>& edgeMasks, uint32_t& anomalies) {
    const int Zc = std::max(g.d[2] - 1, 0);
    int slabs = 1;
#ifdef _OPENMP
    slabs = std::max(1, std::min(Zc, 4 * omp_get_max_threads()));
#endif
    std::vector<SlabDMC> part(slabs);
#pragma omp parallel for schedule(dynamic, 1)
    for (int k = 0; k < slabs; ++k)
        runDMCSlab(g, iso, surfaceIteration, (int)((int64_t)Zc * k / slabs), (int)((int64_t)Zc * (k + 1) / slabs),
                   part[k]);
    std::unordered_map<uint64_t, QuadEntry> table;
    int base = 0;
    for (int k = 0; k < slabs; ++k) {
        SlabDMC& sd = part[k];
        anomalies |= sd.anomalies;
        pos.insert(pos.end(), sd.pos.begin(), sd.pos.end());
        nrm.insert(nrm.end(), sd.nrm.begin(), sd.nrm.end());
        cells.insert(cells.end(), sd.cells.begin(), sd.cells.end());
        edgeMasks.insert(edgeMasks.end(), sd.edgeMasks.begin(), sd.edgeMasks.end());
        for (auto& kv : sd.table) {
            QuadEntry& q = table[kv.first];
            for (int i = 0; i < 4; ++i) {
                if (kv.second.slot[i] == -1) continue;
                if (q.slot[i] != -1) anomalies |= kSSlot;
                q.slot[i] = kv.second.slot[i] + base;
            }
            if (kv.second.color != (int)kAttrInvalidColor) q.color = kv.second.color;
        }
        base += (int)(sd.pos.size() / 3);
        SlabDMC().table.swap(sd.table);
    }
    std::vector<uint64_t> keys;
    keys.reserve(table.size());
    for (auto& kv : table)
        if (kv.second.slot[0] >= 0 && kv.second.slot[1] >= 0 && kv.second.slot[2] >= 0 && kv.second.slot[3] >= 0)
            keys.push_back(kv.first);
    std::sort(keys.begin(), keys.end());
    for (uint64_t k : keys) {
        const QuadEntry& q = table[k];
        for (int i = 0; i < 4; ++i) quads.push_back(q.slot[i]);
        attr.push_back((uint16_t)((kAttrInvalidColor & 0xE0) | q.color));
    }
}

// ------------------------------------------------------------------------ //
// reconnectHalfedges, D/PostProcesses/ManifoldCreator.cu:39-312
// ------------------------------------------------------------------------ //
static inline void cellOf(const Grid& g, V3 p, int c[3]) {
    V3 off = divv(sub(p, g.o()), g.dl());
    c[0] = (int)std::floor(off.x);
    c[1] = (int)std::floor(off.y);
    c[2] = (int)std::floor(off.z);
}
static inline V3 nudge(int it) {
    V3 r = v3((it & 1) ? 1.f : 0.f, (it & 2) ? 1.f : 0.f, (it & 4) ? 1.f : 0.f);
    if (it & 8) r.x = -r.x;
    if (it & 16) r.y = -r.y;
    if (it & 32) r.z = -r.z;
    return muls(r, kEpsilon);
}
static inline int gridIndex(const Grid& g, const int c[3]) {
    return c[2] * g.d[0] * g.d[1] + c[1] * g.d[0] + c[0];
}

static void reconnect(Mesh& m, const Grid& g, Real iso) {
    for (auto& kv : m.table.map) {
        const Bucket& b = kv.second;
        if (b.count < 4) continue;  // isHashTableEntryNonManifold: all 4 ids set
        const HE h0 = m.he[b.ids[0]];
        int n0 = h0.origin, n1 = m.he[h0.next].origin;
        V3 p0 = m.P(n0), p1 = m.P(n1);
        int c0[3], c1[3];
        cellOf(g, p0, c0);
        cellOf(g, p1, c1);
        for (int i = 0; i < 0x40; ++i) {
            V3 o0 = nudge(i), o1 = o0;
            int finalK = -1;
            for (int k = 0; k < 0x40; ++k) {
                o1 = nudge(k);
                int a[3], bb[3];
                cellOf(g, add(p0, o0), a);
                cellOf(g, add(p1, o1), bb);
                int sum = std::abs(a[0] - bb[0]) + std::abs(a[1] - bb[1]) + std::abs(a[2] - bb[2]);
                if (sum == 1) { finalK = k; break; }
            }
            if (finalK != -1) {
                p0 = add(p0, o0);
                cellOf(g, p0, c0);
                p1 = add(p1, o1);
                cellOf(g, p1, c1);
                break;
            }
        }
        int A[3], B[3];
        if (gridIndex(g, c0) < gridIndex(g, c1)) {
            std::memcpy(A, c0, sizeof A); std::memcpy(B, c1, sizeof B);
        } else {
            std::memcpy(A, c1, sizeof A); std::memcpy(B, c0, sizeof B);
        }
        // computeOffsetDirections
        int nrmv[3];
        for (int a = 0; a < 3; ++a) nrmv[a] = std::max(A[a], B[a]) - std::min(A[a], B[a]);
        int xo[3] = {0, 0, 0}, yo[3] = {0, 0, 0};
        if (nrmv[0] == 0) {
            xo[0] = 1;
            if (nrmv[1] == 0) yo[1] = 1; else yo[2] = 1;
        } else {
            xo[1] = 1;
            yo[2] = 1;
        }
        int mn[3];
        for (int a = 0; a < 3; ++a) mn[a] = std::max(A[a], B[a]);
        // computeCellWallValues reads unclamped; positions that lie outside
        // the grid only arise from broken input and are clamped here
        if (mn[0] < 0 || mn[1] < 0 || mn[2] < 0 || mn[0] + 1 >= g.d[0] || mn[1] + 1 >= g.d[1] ||
            mn[2] + 1 >= g.d[2])
            m.anomalies |= kSWall;
        Real w[4];
        w[0] = g.atClamped(mn[0], mn[1], mn[2]);
        w[1] = g.atClamped(mn[0] + xo[0], mn[1] + xo[1], mn[2] + xo[2]);
        w[2] = g.atClamped(mn[0] + xo[0] + yo[0], mn[1] + xo[1] + yo[1], mn[2] + xo[2] + yo[2]);
        w[3] = g.atClamped(mn[0] + yo[0], mn[1] + yo[1], mn[2] + yo[2]);
        V3 corner0 = add(g.o(), mul(g.dl(), v3((Real)mn[0], (Real)mn[1], (Real)mn[2])));
        V3 corner2 = add(g.o(), mul(g.dl(), v3((Real)(mn[0] + xo[0] + yo[0]), (Real)(mn[1] + xo[1] + yo[1]),
                                              (Real)(mn[2] + xo[2] + yo[2]))));
        bool omitX = xo[0] == 0 && yo[0] == 0;
        bool omitY = xo[1] == 0 && yo[1] == 0;
        auto down = [&](V3 p, Real& u, Real& v) {
            if (omitX) { u = p.y; v = p.z; }
            else if (omitY) { u = p.x; v = p.z; }
            else { u = p.x; v = p.y; }
        };
        Real minU, minV, maxU, maxV;
        down(corner0, minU, minV);
        down(corner2, maxU, maxV);
        int sorted[4] = {-1, -1, -1, -1};
        for (int i = 0; i < 4; ++i) {
            int hid = b.ids[i];
            int opp = m.he[m.he[m.he[hid].next].next].origin;
            Real u, v;
            down(m.P(opp), u, v);
            Real mnU = u - minU, mnV = v - minV, mxU = u - maxU, mxV = v - maxV;
            if (mnV < 0.f) sorted[0] = hid;
            if (mxU > 0.f) sorted[1] = hid;
            if (mxV > 0.f) sorted[2] = hid;
            if (mnU < 0.f) sorted[3] = hid;
        }
        bool ok = true;
        for (int i = 0; i < 4; ++i) ok = ok && sorted[i] != -1;
        if (!ok) continue;
        // AsymptoticDecider2D::quadrant0BelongsTogether, D/Utils/AsymptoticDecider.h:119-164
        Real m00 = w[0], m10 = w[1], m11 = w[2], m01 = w[3];
        Real C = m00 - m10;
        C = C - m01;
        C = C + m11;
        Real delta = (m00 * m11 - m10 * m01) / C;
        bool together = (m00 < iso && delta >= iso) || (m00 >= iso && delta < iso);
        bool connect01 = !together;
        if (connect01) {
            m.he[sorted[0]].twin = sorted[1]; m.he[sorted[1]].twin = sorted[0];
            m.he[sorted[2]].twin = sorted[3]; m.he[sorted[3]].twin = sorted[2];
        } else {
            m.he[sorted[0]].twin = sorted[3]; m.he[sorted[3]].twin = sorted[0];
            m.he[sorted[1]].twin = sorted[2]; m.he[sorted[2]].twin = sorted[1];
        }
    }
}

// ------------------------------------------------------------------------ //
// ManifoldSplitter, D/PostProcesses/ManifoldSplitter.cu:25-1387
// ------------------------------------------------------------------------ //
enum SplittingStep {
    StepNone = 0,
    StepSubdivide = 1,
    StepCollapse = 2,
    StepMerge = 3,
    StepTwins = 4,
    StepMove = 5,
    StepIterate = 6,
    StepAll = 100
};

// DeviceMergeList with the partner slots kept in ascending order
struct MergeList {
    std::vector<int> num;      // partners + 1
    std::vector<int> slot;     // 4 per element
    int64_t overflow = 0;
    explicit MergeList(size_t n) : num(n, 1), slot(4 * n, -1) {}
    // markVerticesAsMergable / markHalfedgesAsMergeable, :749-765
    void mark(int a, int b) {
        int idx = num[a]++;
        if (idx - 1 < 4) slot[4 * a + idx - 1] = b;
        if (idx > 2) ++overflow;  // the reference keeps two partners per element
    }
    void finish() {
        for (size_t a = 0; a < num.size(); ++a) {
            int n = std::min(num[a] - 1, 4);
            std::sort(slot.begin() + 4 * a, slot.begin() + 4 * a + n);
        }
    }
    int get(int a, int k) const { return slot[4 * a + k]; }
    int count(int a) const { return std::min(num[a], 5); }
    // getAllPartnersOf, :25-62 (breadth-first closure, at most 12 partners)
    int closure(int v, int out[12], uint32_t& anomalies) const {
        int np = count(v);
        if (np <= 1) return np;
        for (int i = 0; i < np - 1; ++i) out[i] = get(v, i);
        for (int i = 0; i < np - 1; ++i) {
            int p = out[i];
            int npp = count(p);
            for (int k = 0; k < npp - 1; ++k) {
                int pp = get(p, k);
                bool contained = (pp == v);
                for (int z = 0; z < np - 1; ++z) contained = contained || out[z] == pp;
                if (!contained) {
                    if (np - 1 >= 12) { anomalies |= kSPartner; continue; }
                    out[np - 1] = pp;
                    ++np;
                }
            }
        }
        return np;
    }
};

static int runSplitter(Mesh& m, const Grid& g, Real iso, int step) {
    int iterations = 0;
    while (true) {
        std::vector<int> nm;
        for (size_t f = 0; f < m.faceAttr.size(); ++f)
            if (m.faceAttr[f] & kAttrNonManifold) nm.push_back((int)f);
        const int n = (int)nm.size();
        if (n == 0) break;
        const int F = (int)m.faceFirst.size(), H = (int)m.he.size(), V = m.numV();
        const bool doSub = step >= StepSubdivide;
        const int nv = 4 * n + (doSub ? 4 * n : 0);
        const int nh = 4 * n + (doSub ? 16 * n : 0);
        const int nf = n + (doSub ? 4 * n : 0);
        // working copies
        std::vector<Real> cpos(3 * (size_t)nv, 0.f), cnrm(3 * (size_t)nv, 0.f);
        std::vector<uint8_t> vfl(nv, 0), hfl(nh, 0), ffl(nf, 0);
        std::vector<int> vC2O(nv, -1), hC2O(nh, -1), fC2O(nf, -1);
        std::vector<int> cparent(nv, -1);  // mesh vertex each working vertex comes from
        std::vector<int> vO2C(V, -1), hO2C(H, -1), fO2C(F, -1);
        std::vector<HE> ch(nh, HE{-1, -1, -1, -1});
        std::vector<int> cfirst(nf, -1);
        std::vector<uint16_t> cattr(nf, kAttrInvalidColor);

        // copyVerticesToWorkingCopy :307-341 (+ representative choice of
        // markDuplicateVertices :343-355: the smallest copy index)
        for (int k = 0; k < n; ++k) {
            int h = m.faceFirst[nm[k]];
            for (int i = 0; i < 4; ++i) {
                int v = m.he[h].origin, c = 4 * k + i;
                for (int a = 0; a < 3; ++a) { cpos[3 * c + a] = m.pos[3 * v + a]; cnrm[3 * c + a] = m.nrm[3 * v + a]; }
                vC2O[c] = v;
                cparent[c] = v;
                if (vO2C[v] == -1) vO2C[v] = c;
                h = m.he[h].next;
            }
        }
        // copyHalfedgesToWorkingCopy :383-408
        for (int k = 0; k < n; ++k) {
            int h = m.faceFirst[nm[k]];
            for (int i = 0; i < 4; ++i) {
                int c = 4 * k + i;
                ch[c] = m.he[h];
                hC2O[c] = h;
                hO2C[h] = c;
                h = m.he[h].next;
            }
        }
        // copyFacesToWorkingCopy :425-446
        for (int k = 0; k < n; ++k) {
            cfirst[k] = hO2C[m.faceFirst[nm[k]]];
            cattr[k] = m.faceAttr[nm[k]];
            fC2O[k] = nm[k];
            fO2C[nm[k]] = k;
        }
        // updateWorkingCopyHalfedges :463-505
        for (int c = 0; c < 4 * n; ++c) {
            HE& e = ch[c];
            e.origin = vO2C[e.origin];
            e.face = fO2C[e.face];
            e.next = hO2C[e.next];
            if (e.twin >= 0) {
                int t = hO2C[e.twin];
                e.twin = (t == -1) ? -e.twin - 2 : t;
            }
        }
        // markHalfedgesAsNonManifold :527-555
        for (auto& kv : m.table.map) {
            const Bucket& b = kv.second;
            if (b.count < 4) continue;
            for (int i = 0; i < 4; ++i) {
                int c = hO2C[b.ids[i]];
                if (c < 0) { m.anomalies |= kSBadTwin; continue; }
                hfl[c] |= kFlagNonManifold;
                vfl[ch[c].origin] |= kFlagNonManifold;
            }
        }
        // performSubdivideQuads :650-731
        if (doSub) {
            const Real uvs[4][2] = {{0.33f, 0.33f}, {0.67f, 0.33f}, {0.67f, 0.67f}, {0.33f, 0.67f}};
            for (int k = 0; k < n; ++k) {
                int hid[4], vid[4];
                int h = cfirst[k];
                for (int i = 0; i < 4; ++i) { hid[i] = h; vid[i] = ch[h].origin; h = ch[h].next; }
                V3 P[4], N[4];
                for (int i = 0; i < 4; ++i) {
                    P[i] = v3(cpos[3 * vid[i]], cpos[3 * vid[i] + 1], cpos[3 * vid[i] + 2]);
                    N[i] = v3(cnrm[3 * vid[i]], cnrm[3 * vid[i] + 1], cnrm[3 * vid[i] + 2]);
                }
                int inner[4];
                for (int i = 0; i < 4; ++i) {
                    Real u = uvs[i][0], v = uvs[i][1];
                    // Interpolation<Vertex>::interpolateBilinearly with glm::mix
                    auto mix = [](V3 a, V3 b, Real f) { return add(muls(a, 1.f - f), muls(b, f)); };
                    V3 pa = mix(P[0], P[1], u), pb = mix(P[3], P[2], u), pp = mix(pa, pb, v);
                    V3 na = mix(N[0], N[1], u), nb = mix(N[3], N[2], u), nn = mix(na, nb, v);
                    int c = 4 * n + 4 * k + i;
                    cparent[c] = vC2O[vid[i]];  // inner vertex i comes from corner i
                    cpos[3 * c] = pp.x; cpos[3 * c + 1] = pp.y; cpos[3 * c + 2] = pp.z;
                    cnrm[3 * c] = nn.x; cnrm[3 * c + 1] = nn.y; cnrm[3 * c + 2] = nn.z;
                    inner[i] = c;
                }
                const int hb = 4 * n + 16 * k;
                int ih[4];
                for (int i = 0; i < 4; ++i) { ih[i] = hb + i; ch[ih[i]] = HE{inner[i], -1, -1, -1}; }
                for (int i = 0; i < 4; ++i) ch[ih[i]].next = ih[(i + 1) & 3];
                for (int i = 0; i < 4; ++i) ch[ih[i]].face = k;
                cfirst[k] = ih[0];
                int of[4][4];
                int prev = 3;
                for (int j = 0; j < 4; ++j) {
                    int qv[4] = {vid[j], inner[j], inner[prev], vid[prev]};
                    for (int t = 0; t < 3; ++t) { of[j][t] = hb + 4 + 3 * j + t; ch[of[j][t]] = HE{qv[t], -1, -1, -1}; }
                    of[j][3] = hid[prev];
                    for (int t = 0; t < 4; ++t) ch[of[j][t]].next = of[j][(t + 1) & 3];
                    int nf2 = n + 4 * k + j;
                    cattr[nf2] = kAttrInvalidColor;
                    for (int t = 0; t < 4; ++t) ch[of[j][t]].face = nf2;
                    cfirst[nf2] = of[j][0];
                    prev = j;
                }
                prev = 3;
                for (int j = 0; j < 4; ++j) {
                    ch[of[j][2]].twin = of[prev][0]; ch[of[prev][0]].twin = of[j][2];
                    ch[of[j][1]].twin = ih[prev]; ch[ih[prev]].twin = of[j][1];
                    prev = j;
                }
                // swapHalfedgeMappings :629-648
                for (int i = 0; i < 4; ++i) {
                    int a = hid[i], b = ih[i];
                    int ao = hC2O[a], bo = hC2O[b];
                    hC2O[a] = bo;
                    hC2O[b] = ao;
                    if (ao != -1 && bo == -1) hO2C[ao] = b;
                    else m.anomalies |= kSMapping;
                }
            }
        }
        // collapseNonManifoldEdges :749-1124
        if (step >= StepCollapse) {
            MergeList vml(nv), hml(nh);
            for (int t = 0; t < nh; ++t) {
                if (!(hfl[t] & kFlagNonManifold)) continue;
                int tw = ch[t].twin;
                if (tw < 0) { m.anomalies |= kSBadTwin; continue; }
                if (tw < t) continue;
                // collapseHalfedge :767-835
                int f0[4], f1[4];
                HE cur = ch[t], ctw = ch[tw];
                f0[0] = t;
                f1[0] = tw;
                for (int i = 1; i < 4; ++i) {
                    f0[i] = cur.next;
                    f1[4 - i] = ctw.next;
                    cur = ch[cur.next];
                    ctw = ch[ctw.next];
                }
                for (int i = 0; i < 4; ++i) { hfl[f0[i]] |= kFlagRemove; hfl[f1[i]] |= kFlagRemove; }
                ffl[ch[f0[0]].face] |= kFlagRemove;
                ffl[ch[f1[0]].face] |= kFlagRemove;
                {
                    int a = ch[f0[2]].origin, b = ch[f1[1]].origin;
                    vml.mark(a, b); vml.mark(b, a);
                }
                {
                    int a = ch[f0[3]].origin, b = ch[f1[2]].origin;
                    vml.mark(a, b); vml.mark(b, a);
                }
                for (int i = 1; i < 4; ++i) {
                    int a = f0[i], b = f1[i];
                    int at = ch[a].twin, bt = ch[b].twin;
                    if (at < 0 || bt < 0) { m.anomalies |= kSBadTwin; continue; }
                    hml.mark(a, bt); hml.mark(bt, a);
                    hml.mark(b, at); hml.mark(at, b);
                }
            }
            vml.finish();
            hml.finish();
            if (vml.overflow + hml.overflow) m.anomalies |= kSPartner;
            if (step >= StepMerge) {
                // mergeVertices :936-990
                for (int v = 0; v < nv; ++v) {
                    int part[12];
                    int np = vml.closure(v, part, m.anomalies);
                    if (np <= 1) continue;
                    if (np > 12) { m.anomalies |= kSPartner; continue; }  // :954-958
                    int smallest = v;
                    V3 p = v3(cpos[3 * v], cpos[3 * v + 1], cpos[3 * v + 2]);
                    bool obsolete = false;
                    for (int i = 0; i < np - 1; ++i) {
                        int q = part[i];
                        p = add(p, v3(cpos[3 * q], cpos[3 * q + 1], cpos[3 * q + 2]));
                        if (q < smallest) { obsolete = true; smallest = q; }
                    }
                    if (obsolete) { vfl[v] |= kFlagRemove; continue; }
                    p = divs(p, (Real)np);
                    cpos[3 * smallest] = p.x; cpos[3 * smallest + 1] = p.y; cpos[3 * smallest + 2] = p.z;
                    // the reference stores the averaged position as the normal (:989)
                    cnrm[3 * smallest] = p.x; cnrm[3 * smallest + 1] = p.y; cnrm[3 * smallest + 2] = p.z;
                }
                // updateHalfedgeVertexIDs :992-1019
                for (int t = 0; t < nh; ++t) {
                    int v = ch[t].origin;
                    if (v < 0) continue;
                    int part[12];
                    int np = vml.closure(v, part, m.anomalies);
                    if (np <= 1) continue;
                    int s = v;
                    for (int i = 0; i < np - 1; ++i) s = std::min(s, part[i]);
                    ch[t].origin = s;
                }
            }
            if (step >= StepTwins) {
                // mergeHalfedges :1021-1067 (decisions read only removed partners)
                std::vector<std::pair<int, int>> pairs;
                for (int t = 0; t < nh; ++t) {
                    if (hfl[t] & kFlagRemove) continue;
                    int part[12];
                    int np = hml.closure(t, part, m.anomalies);
                    if (np <= 1) continue;
                    int valid = -1;
                    for (int i = 0; i < np - 1; ++i) {
                        int tw = ch[part[i]].twin;
                        if (tw < 0) continue;
                        if (!(hfl[tw] & kFlagRemove)) { valid = tw; break; }
                    }
                    if (valid == -1 || valid < t) continue;
                    pairs.push_back({t, valid});
                }
                for (auto& pr : pairs) { ch[pr.first].twin = pr.second; ch[pr.second].twin = pr.first; }
            }
        }
        // performMoveVerticesToSurface :1130-1160
        if (step >= StepMove) {
            for (int v = 0; v < nv; ++v) {
                if (vfl[v] & kFlagRemove) continue;
                V3 p = v3(cpos[3 * v], cpos[3 * v + 1], cpos[3 * v + 2]);
                int idx[3];
                cellOf(g, p, idx);
                Real s[8];
                cornerValues(g, idx[0], idx[1], idx[2], s);
                V3 fi = v3((Real)idx[0], (Real)idx[1], (Real)idx[2]);
                V3 fi1 = v3((Real)(idx[0] + 1), (Real)(idx[1] + 1), (Real)(idx[2] + 1));
                V3 mn = add(g.o(), mul(fi, g.dl()));
                V3 mx = add(g.o(), mul(fi1, g.dl()));
                V3 local = divv(sub(p, mn), sub(mx, mn));
                SurfaceIterator it{s, iso};
                it.move(local);
                V3 w = add(g.o(), mul(add(fi, local), g.dl()));
                cpos[3 * v] = w.x; cpos[3 * v + 1] = w.y; cpos[3 * v + 2] = w.z;
            }
        }
        // copyWorkingCopiesBack :1176-1387
        {
            for (int v = 0; v < nv; ++v) {
                if (vfl[v] & kFlagRemove) continue;
                int o = vC2O[v];
                if (o == -1) {
                    o = m.numV();
                    for (int a = 0; a < 3; ++a) { m.pos.push_back(cpos[3 * v + a]); m.nrm.push_back(cnrm[3 * v + a]); }
                    m.vflags.push_back(0);
                    m.parent.push_back(cparent[v] >= 0 && cparent[v] < V ? m.parent[cparent[v]] : -1);
                    vC2O[v] = o;
                } else {
                    for (int a = 0; a < 3; ++a) { m.pos[3 * o + a] = cpos[3 * v + a]; m.nrm[3 * o + a] = cnrm[3 * v + a]; }
                }
            }
            for (int t = 0; t < nh; ++t) {
                if (hfl[t] & kFlagRemove) continue;
                int o = hC2O[t];
                if (o == -1) {
                    o = (int)m.he.size();
                    m.he.push_back(ch[t]);
                    hC2O[t] = o;
                } else {
                    m.he[o] = ch[t];
                }
            }
            for (int f = 0; f < nf; ++f) {
                if (ffl[f] & kFlagRemove) continue;
                int o = fC2O[f];
                int first = hC2O[cfirst[f]];
                if (o == -1) {
                    o = (int)m.faceFirst.size();
                    m.faceFirst.push_back(first);
                    m.faceAttr.push_back(cattr[f]);
                    fC2O[f] = o;
                } else {
                    m.faceFirst[o] = first;
                    m.faceAttr[o] = cattr[f];
                }
            }
            for (int t = 0; t < nh; ++t) {
                if (hfl[t] & kFlagRemove) continue;
                HE& e = m.he[hC2O[t]];
                e.next = hC2O[e.next];
                e.face = fC2O[e.face];
                e.origin = vC2O[e.origin];
                int tw = e.twin;
                if (tw < 0) {
                    tw = -tw - 2;
                    e.twin = tw;
                    if (tw != -1) m.he[tw].twin = hC2O[t];
                } else {
                    e.twin = hC2O[tw];
                }
            }
        }
        m.refresh();
        ++iterations;
        if (!(step >= StepIterate)) break;
        if (iterations >= 64) { m.anomalies |= kSIterCap; break; }  // the reference has no cap
    }
    return iterations;
}

// ------------------------------------------------------------------------ //
// detectNonManifoldVertices, D/PostProcesses/ManifoldCreator.cu:319-536
// ------------------------------------------------------------------------ //
static void detectNonManifoldVertices(Mesh& m) {
    const int H = (int)m.he.size();
    auto stepCW = [&](int h) -> int {
        const HE& e = m.he[h];
        if (e.twin != -1) return m.he[e.twin].next;
        return -1;
    };
    auto stepCCW = [&](int h) -> int {
        int p = m.he[m.he[m.he[h].next].next].next;
        if (m.he[p].twin != -1) return m.he[p].twin;
        return -1;
    };
    auto walk = [&](int start, bool cw) -> int {
        int origin = m.he[start].origin;
        int result = start;
        int cur = cw ? stepCW(start) : stepCCW(start);
        int guard = 0;
        while (cur != -1) {
            if (cur == result) break;
            if (origin != m.he[cur].origin) break;
            if (cur < result) result = cur;
            cur = cw ? stepCW(cur) : stepCCW(cur);
            if (++guard > 4096) { m.anomalies |= kSWalk; break; }
        }
        return result;
    };
    // A fan key is the smallest halfedge id of the fan and has the same origin
    // as the halfedge it was found from, so "distinct (origin, key) pairs per
    // origin" equals "halfedges that some halfedge names as key, per origin".
    std::vector<uint8_t> isKey(H, 0);
    for (int h = 0; h < H; ++h) {
        int k = std::min(h, std::min(walk(h, true), walk(h, false)));
        isKey[k] = 1;
    }
    std::vector<int> fans(m.numV(), 0);
    for (int h = 0; h < H; ++h)
        if (isKey[h]) fans[m.he[h].origin]++;
    for (int v = 0; v < m.numV(); ++v) {
        if (fans[v] > 1) m.vflags[v] |= kFlagMultiFan;
        else m.vflags[v] &= (uint8_t)~kFlagMultiFan;
    }
}

// ------------------------------------------------------------------------ //
// Standard Marching Cubes (OriginalDMC standard_mc, O/DualMarchingCubes.cu:
// 201-307, and map_triangles :316-328): one vertex per intersected grid edge,
// at the linear crossing, with the interpolated corner gradient divided by its
// length; triangles from the case table.  The reference numbers vertices and
// triangles in atomic order; here vertices follow the global edge id
// 3 * sample + axis and triangles the cells' (z, y, x) order, then the table.
// ------------------------------------------------------------------------ //
struct MCMesh {
    std::vector<Real> pos, nrm;
    std::vector<int> tris;
};

// central-difference gradient at grid point (x, y, z) with clamped neighbours
// (UniformGrid::gradient, O/UniformGrid.h:278-330: each corner's entry)
static V3 pointGradient(const Grid& g, int x, int y, int z) {
    V3 d = g.dl();
    Real gx = 0.5f * (g.atClamped(x + 1, y, z) - g.atClamped(x - 1, y, z)) / d.x;
    Real gy = 0.5f * (g.atClamped(x, y + 1, z) - g.atClamped(x, y - 1, z)) / d.y;
    Real gz = 0.5f * (g.atClamped(x, y, z + 1) - g.atClamped(x, y, z - 1)) / d.z;
    return v3(gx, gy, gz);
}

static MCMesh* standardMC(const Grid& g, Real iso) {
    MCMesh* m = new MCMesh();
    const int X = g.d[0], Y = g.d[1], Z = g.d[2];
    if (X < 2 || Y < 2 || Z < 2) return m;  // no cells
    const size_t S = (size_t)X * Y * Z;
    std::vector<int> vid(3 * S, -1);
    const V3 o = g.o(), dl = g.dl();
    for (int z = 0; z < Z; ++z)
        for (int y = 0; y < Y; ++y)
            for (int x = 0; x < X; ++x)
                for (int a = 0; a < 3; ++a) {
                    const int x1 = x + (a == 0), y1 = y + (a == 1), z1 = z + (a == 2);
                    if (x1 >= X || y1 >= Y || z1 >= Z) continue;
                    const Real u0 = g.at(x, y, z), u1 = g.at(x1, y1, z1);
                    if ((u0 >= iso) == (u1 >= iso)) continue;
                    const size_t e = 3 * (((size_t)z * Y + y) * X + x) + a;
                    vid[e] = (int)(m->pos.size() / 3);
                    const Real l = (iso - u0) / (u1 - u0);
                    const Real p0[3] = {o.x + (Real)x * dl.x, o.y + (Real)y * dl.y, o.z + (Real)z * dl.z};
                    const Real p1[3] = {o.x + (Real)x1 * dl.x, o.y + (Real)y1 * dl.y, o.z + (Real)z1 * dl.z};
                    const V3 n0 = pointGradient(g, x, y, z), n1 = pointGradient(g, x1, y1, z1);
                    V3 ni = v3(n0.x + l * (n1.x - n0.x), n0.y + l * (n1.y - n0.y), n0.z + l * (n1.z - n0.z));
                    const Real f = std::sqrt(ni.x * ni.x + ni.y * ni.y + ni.z * ni.z);
                    ni = v3(ni.x / f, ni.y / f, ni.z / f);
                    for (int k = 0; k < 3; ++k) m->pos.push_back(p0[k] + l * (p1[k] - p0[k]));
                    m->nrm.push_back(ni.x);
                    m->nrm.push_back(ni.y);
                    m->nrm.push_back(ni.z);
                }
    for (int z = 0; z + 1 < Z; ++z)
        for (int y = 0; y + 1 < Y; ++y)
            for (int x = 0; x + 1 < X; ++x) {
                Real sv[8];
                cornerValues(g, x, y, z, sv);
                int cs = 0;
                for (int i = 0; i < 8; ++i) cs |= (sv[i] >= iso ? 1 : 0) << i;
                const uint64_t w = kTriangleTable[cs];
                const int n = (int)(w & 0xF);
                for (int k = 0; k < 3 * n; ++k) {
                    const int e = (int)((w >> (4 + 4 * k)) & 0xF);
                    const int a0 = kEdgeV0[e];
                    const size_t gid = 3 * (((size_t)(z + ((a0 >> 2) & 1)) * Y + (y + ((a0 >> 1) & 1))) * X +
                                            (x + (a0 & 1))) + kEdgeAxis[e];
                    m->tris.push_back(vid[gid]);
                }
            }
    return m;
}

// ------------------------------------------------------------------------ //
// HalfedgeMesh::initialize from a quad list, D/Halfedges/HalfedgeMesh.cu:14-60,
// :173-291, :848-857: halfedge i of quad q is 4q+i, twins and flags from the
// edge table, face attributes from the quads'
// ------------------------------------------------------------------------ //
static void initializeFromQuads(Mesh& m, const std::vector<int>& quads, const std::vector<uint16_t>& attr) {
    const int Q = (int)attr.size();
    m.he.resize(4 * (size_t)Q);
    m.faceFirst.resize(Q);
    m.faceAttr = attr;
    m.vflags.assign(m.numV(), 0);
    for (int q = 0; q < Q; ++q) {
        for (int i = 0; i < 4; ++i) m.he[4 * q + i] = HE{quads[4 * q + i], q, 4 * q + ((i + 1) & 3), -1};
        m.faceFirst[q] = 4 * q;
    }
    m.buildTable();
    m.connectTwins();
    m.vertexFlagsFromTable();
}

// ------------------------------------------------------------------------ //
// Valence-pattern simplifications, D/Halfedges/HalfedgeMesh.cu:296-683 and
// :859-1048.  They run right after the halfedge mesh is built, on its vertex
// and quad lists, and end with a rebuild from the reduced lists.  Where the
// reference is not deterministic or reads outside its arrays, this
// restatement fixes one behaviour:
//  - a quad edge without a twin (the reference then reads halfedges[-1])
//    makes the quad ineligible;
//  - vertices and quads are compacted in their order (the reference appends
//    with atomics);
//  - in the 3333 pass every face's pattern bits are cleared before any face
//    sets a neighbour's remove flag (the reference's threads race there).
// ------------------------------------------------------------------------ //
static const uint16_t kAttrPattern = 0x40, kAttrRemove = 0x80, kAttrBoundary = 0x100;
enum { kTypeNeutral = 0, kTypePattern = 1, kTypeRemovable = 3 };

// computeVertexValence, :296-312: outgoing halfedges, plus one per halfedge
// without twin for the vertex it points to
static std::vector<int> vertexValence(const Mesh& m) {
    std::vector<int> val(m.numV(), 0);
    for (const HE& e : m.he) {
        val[e.origin]++;
        if (e.twin == -1) val[m.he[e.next].origin]++;
    }
    return val;
}

static void faceVertices(const Mesh& m, int f, int q[4], int hs[4]) {
    int h = m.faceFirst[f];
    for (int i = 0; i < 4; ++i) {
        hs[i] = h;
        q[i] = m.he[h].origin;
        h = m.he[h].next;
    }
}

// removeVertices*, removeQuadrilaterals* / removeQuads*: keep the vertices that
// are not removed (in order), remap the kept quads, then rebuild
static void compactAndRebuild(Mesh& m, const std::vector<int>& type, int removedType, const std::vector<int>& target,
                              bool remapPatternQuads) {
    const int V = m.numV(), F = (int)m.faceFirst.size();
    std::vector<int> addr(V, -1);
    std::vector<Real> pos, nrm;
    std::vector<int> parent;
    for (int v = 0; v < V; ++v) {
        if (type[v] == removedType) continue;
        addr[v] = (int)(pos.size() / 3);
        for (int a = 0; a < 3; ++a) {
            pos.push_back(m.pos[3 * v + a]);
            nrm.push_back(m.nrm[3 * v + a]);
        }
        parent.push_back(v < (int)m.parent.size() ? m.parent[v] : -1);
    }
    std::vector<int> quads;
    std::vector<uint16_t> attr;
    for (int f = 0; f < F; ++f) {
        const uint16_t a = m.faceAttr[f];
        if (a & kAttrRemove) continue;
        int q[4], hs[4];
        faceVertices(m, f, q, hs);
        for (int i = 0; i < 4; ++i) {
            int v = q[i];
            if (remapPatternQuads ? (a & kAttrPattern) != 0 : type[v] == removedType) v = target[v];
            const int n = (v >= 0 && v < V) ? addr[v] : -1;
            if (n < 0) m.anomalies |= kSMapping;
            quads.push_back(n < 0 ? 0 : n);
        }
        // a new QuadrilateralAttribute (INVALID_COLOR) keeps the NM and boundary bits
        attr.push_back((uint16_t)(kAttrInvalidColor | (a & kAttrNonManifold) | (a & kAttrBoundary)));
    }
    m.pos = std::move(pos);
    m.nrm = std::move(nrm);
    m.parent = std::move(parent);
    initializeFromQuads(m, quads, attr);
}

// handleMerge, :358-378: vertex a takes the midpoint of b and d (position and
// normalized normal), c is removed in favour of a
static void handleMerge(Mesh& m, int a, int b, int c, int d, std::vector<int>& type, std::vector<int>& target,
                        uint16_t& attr) {
    V3 p = m.P(b);
    p = add(p, smul(0.5f, sub(m.P(d), p)));
    V3 n = v3(m.nrm[3 * b], m.nrm[3 * b + 1], m.nrm[3 * b + 2]);
    const V3 nd = v3(m.nrm[3 * d], m.nrm[3 * d + 1], m.nrm[3 * d + 2]);
    n = normalize(add(n, smul(0.5f, sub(nd, n))));
    m.pos[3 * a] = p.x; m.pos[3 * a + 1] = p.y; m.pos[3 * a + 2] = p.z;
    m.nrm[3 * a] = n.x; m.nrm[3 * a + 1] = n.y; m.nrm[3 * a + 2] = n.z;
    type[c] = kTypeRemovable;
    target[c] = a;
    attr |= kAttrRemove;
}

// simplify3X3Y (color based, :859-921; markElementsP3X3Y :318-340,
// mergeVerticesP3X3YColor :381-442) and simplify3X3YOld (:923-985;
// countVerticesP3X3Y :342-364, mergeVerticesP3X3Y :448-496)
static void simplify3X3Y(Mesh& m, bool color) {
    const int V = m.numV(), F = (int)m.faceFirst.size();
    const std::vector<int> val = vertexValence(m);
    std::vector<int> count(V, 0), type(V, kTypeNeutral), target(V, -1);
    std::vector<uint16_t>& attr = m.faceAttr;
    auto patternA = [&](const int q[4]) { return val[q[0]] == 3 && val[q[1]] >= 5 && val[q[2]] == 3 && val[q[3]] >= 5; };
    auto patternB = [&](const int q[4]) { return val[q[0]] >= 5 && val[q[1]] == 3 && val[q[2]] >= 5 && val[q[3]] == 3; };
    for (int f = 0; f < F; ++f) {
        int q[4], hs[4];
        faceVertices(m, f, q, hs);
        if (color) {
            if (attr[f] & (kAttrNonManifold | kAttrBoundary)) continue;
            attr[f] &= 0x3F;
            if (patternA(q) || patternB(q)) attr[f] |= kAttrPattern;
        } else {
            attr[f] &= 0x3F;
            if (patternA(q)) {
                count[q[0]]++;
                count[q[2]]++;
                attr[f] |= kAttrPattern;
            } else if (patternB(q)) {
                count[q[1]]++;
                count[q[3]]++;
                attr[f] |= kAttrPattern;
            }
        }
    }
    for (int f = 0; f < F; ++f) {
        if (!color && (attr[f] & (kAttrNonManifold | kAttrBoundary))) continue;
        if (!(attr[f] & kAttrPattern)) continue;
        int q[4], hs[4];
        faceVertices(m, f, q, hs);
        int nb[4];
        bool ok = true;
        for (int i = 0; i < 4 && ok; ++i) {
            const int t = m.he[hs[i]].twin;
            if (t < 0) { ok = false; break; }
            nb[i] = m.he[t].face;
            // the reference tests the neighbour's NM flag and its own boundary flag
            if ((attr[nb[i]] & kAttrNonManifold) || (attr[f] & kAttrBoundary)) ok = false;
        }
        if (!ok) continue;
        if (color) {
            const int c = attr[f] & 0x1F;
            for (int i = 0; i < 4; ++i)
                if ((attr[nb[i]] & kAttrPattern) && (attr[nb[i]] & 0x1F) <= c) ok = false;
            if (!ok) continue;
        }
        if (patternA(q) && (color || (count[q[0]] == 1 && count[q[2]] == 1)))
            handleMerge(m, q[0], q[1], q[2], q[3], type, target, attr[f]);
        else if (patternB(q) && (color || (count[q[1]] == 1 && count[q[3]] == 1)))
            handleMerge(m, q[1], q[0], q[3], q[2], type, target, attr[f]);
    }
    compactAndRebuild(m, type, kTypeRemovable, target, false);
}

// simplify3333 (:987-1048; markElementsP3333 :544-625)
static void simplify3333(Mesh& m) {
    const int V = m.numV(), F = (int)m.faceFirst.size();
    const std::vector<int> val = vertexValence(m);
    std::vector<int> type(V, kTypeNeutral), target(V, -1);
    std::vector<uint16_t>& attr = m.faceAttr;
    for (int f = 0; f < F; ++f)
        if (!(attr[f] & (kAttrNonManifold | kAttrBoundary))) attr[f] &= 0x3F;
    for (int f = 0; f < F; ++f) {
        if (attr[f] & (kAttrNonManifold | kAttrBoundary)) continue;
        int q[4], hs[4];
        faceVertices(m, f, q, hs);
        bool ok = true;
        for (int i = 0; i < 4; ++i) ok = ok && val[q[i]] == 3;
        if (!ok) continue;
        int nb[4], nv[4], nval[4];
        for (int i = 0; i < 4 && ok; ++i) {
            const int t = m.he[hs[i]].twin;
            if (t < 0) { ok = false; break; }
            nb[i] = m.he[t].face;
            if (attr[nb[i]] & (kAttrNonManifold | kAttrBoundary)) { ok = false; break; }
            nv[i] = m.he[m.he[m.he[t].next].next].origin;
            nval[i] = val[nv[i]];
            if (nval[i] == 3) ok = false;
        }
        if (!ok) continue;
        if (nval[0] == 4 && nval[1] == 4 && nval[2] == 4 && nval[3] == 4) continue;
        attr[f] |= kAttrPattern;
        for (int i = 0; i < 4; ++i) {
            attr[nb[i]] |= kAttrRemove;
            type[q[i]] = kTypePattern;
            target[q[i]] = nv[i];
        }
    }
    compactAndRebuild(m, type, kTypePattern, target, true);
}

static Result* run(const Grid& g, Real iso, const mdmc_oracle_options& opt) {
    Result* r = new Result();
    std::memset(r->stats, 0, sizeof r->stats);
    uint32_t anomalies = 0;
    runDMC(g, iso, opt.surface_iteration != 0, r->dmcPos, r->dmcNrm, r->dmcQuads, r->dmcAttr, r->dmcCell,
           r->dmcEdges, anomalies);

    Mesh m;
    m.pos = r->dmcPos;
    m.nrm = r->dmcNrm;
    m.parent.resize(m.numV());
    for (int v = 0; v < m.numV(); ++v) m.parent[v] = v;
    const int Q = (int)r->dmcAttr.size();
    if (m.numV() > 0) {
        initializeFromQuads(m, r->dmcQuads, r->dmcAttr);
        (void)Q;
        // runPostProcesses, D/DualMarchingCubes.cu:335-380: simplifications, then repair
        if (opt.simplify_3x3y_color) simplify3X3Y(m, true);
        if (opt.simplify_3x3y_old) simplify3X3Y(m, false);
        if (opt.simplify_3333) simplify3333(m);
        reconnect(m, g, iso);  // fixManifoldTwins
        if (opt.split_non_manifold)
            r->stats[MDMC_ORC_STAT_SPLIT_ITERATIONS] = runSplitter(m, g, iso, opt.splitting_step);
        if (opt.detect_non_manifold_vertices) detectNonManifoldVertices(m);
    }
    anomalies |= m.table.anomalies | m.anomalies;
    if (m.numV() == 0) {  // the reference logs and returns before post-processing
        for (int k = 0; k < MDMC_ORC_NUM_STATS; ++k) r->stats[k] = -1;
        r->stats[MDMC_ORC_STAT_SPLIT_ITERATIONS] = 0;
        r->stats[MDMC_ORC_STAT_ANOMALIES] = anomalies;
        return r;
    }

    // statistics getters, D/Halfedges/HalfedgeMesh.cu:1164-1239, ManifoldCreator.cu:545-549
    int64_t e = 0, e3 = 0, e4 = 0;
    for (auto& kv : m.table.map) {
        if (kv.second.count > 0) ++e;
        if (kv.second.count == 3) ++e3;
        if (kv.second.count == 4) ++e4;
    }
    r->stats[MDMC_ORC_STAT_EDGES] = e;
    r->stats[MDMC_ORC_STAT_EDGES3] = e3;
    r->stats[MDMC_ORC_STAT_EDGES4] = e4;
    int64_t nmv = 0;
    for (uint8_t f : m.vflags) if (f & kFlagMultiFan) ++nmv;
    r->stats[MDMC_ORC_STAT_NM_VERTICES] = opt.detect_non_manifold_vertices ? nmv : -1;
    int64_t qk[5] = {0, 0, 0, 0, 0};
    for (size_t f = 0; f < m.faceFirst.size(); ++f) {
        int h = m.faceFirst[f];
        int cnt = 0;
        for (int i = 0; i < 4; ++i) {
            int nx = m.he[h].next;
            if (m.table.valence(m.he[h].origin, m.he[nx].origin) > 2) ++cnt;
            h = nx;
        }
        qk[cnt]++;
    }
    for (int k = 1; k <= 4; ++k) r->stats[MDMC_ORC_STAT_QUADS_NM1 + k - 1] = qk[k];
    r->stats[MDMC_ORC_STAT_ANOMALIES] = anomalies;

    r->parent = std::move(m.parent);
    r->pos = std::move(m.pos);
    r->nrm = std::move(m.nrm);
    r->he = std::move(m.he);
    r->faceFirst = std::move(m.faceFirst);
    r->faceAttr = std::move(m.faceAttr);
    r->vflags = std::move(m.vflags);
    r->vflags.resize(r->pos.size() / 3, 0);
    r->vertexHE.assign(r->pos.size() / 3, -1);
    for (size_t h = 0; h < r->he.size(); ++h) {
        int v = r->he[h].origin;
        if (v >= 0 && (r->vertexHE[v] == -1 || (int)h < r->vertexHE[v])) r->vertexHE[v] = (int)h;
    }
    return r;
}

}  // namespace oracle

// ------------------------------------------------------------------------ //
// C API
// ------------------------------------------------------------------------ //
namespace {
// float input as the restatement's arithmetic type (a copy unless that is float)
struct RealInput {
    std::vector<oracle::Real> copy;
    const oracle::Real* p = nullptr;
    RealInput(const float* v, size_t n) {
        if (std::is_same<oracle::Real, float>::value) {
            p = reinterpret_cast<const oracle::Real*>(v);
        } else {
            copy.assign(v, v + n);
            p = copy.data();
        }
    }
};
template <class T>
void copyFloats(float* dst, const std::vector<T>& v) {
    if (std::is_same<T, float>::value) std::memcpy(dst, v.data(), v.size() * sizeof(float));
    else
        for (size_t i = 0; i < v.size(); ++i) dst[i] = (float)v[i];
}
oracle::Grid gridOf(const RealInput& in, const int dims[3], const float origin[3], const float spacing[3]) {
    oracle::Grid g;
    for (int a = 0; a < 3; ++a) {
        g.d[a] = dims[a];
        g.origin[a] = origin[a];
        g.deltas[a] = spacing[a];
    }
    g.v = in.p;
    return g;
}
size_t samplesOf(const int dims[3]) { return (size_t)dims[0] * dims[1] * dims[2]; }
}  // namespace

extern "C" {

void mdmc_oracle_default_options(mdmc_oracle_options* o) {
    o->surface_iteration = 1;
    o->simplify_3x3y_color = 0;
    o->simplify_3x3y_old = 0;
    o->simplify_3333 = 0;
    o->split_non_manifold = 1;
    o->detect_non_manifold_vertices = 1;
    o->splitting_step = oracle::StepAll;
}

int mdmc_oracle_read_bin(const char* path, int dims[3], float spacing[3], float origin[3], float* out) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return -1;
    int ok = std::fread(dims, sizeof(int), 3, f) == 3 && std::fread(spacing, sizeof(float), 3, f) == 3;
    if (!ok || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) { std::fclose(f); return -2; }
    for (int a = 0; a < 3; ++a) origin[a] = (-0.5f * (float)(dims[a] - 1)) * spacing[a];
    if (out) {
        size_t n = (size_t)dims[0] * dims[1] * dims[2];
        std::vector<uint16_t> raw(n);
        if (std::fread(raw.data(), sizeof(uint16_t), n, f) != n) { std::fclose(f); return -3; }
        for (size_t i = 0; i < n; ++i) out[i] = (float)raw[i];
    }
    std::fclose(f);
    return 0;
}

void mdmc_oracle_refine(const float* in, const int dims[3], const float origin[3], const float spacing[3],
                        int refinement, int pad, float* out, int out_dims[3], float out_origin[3],
                        float out_spacing[3]) {
    const RealInput input(in, samplesOf(dims));
    const oracle::Grid g = gridOf(input, dims, origin, spacing);
    std::vector<oracle::Real> res;
    oracle::Real oo[3], os[3];
    oracle::refine(g, refinement, pad != 0, res, out_dims, oo, os);
    for (int a = 0; a < 3; ++a) {
        out_origin[a] = (float)oo[a];
        out_spacing[a] = (float)os[a];
    }
    if (out) copyFloats(out, res);
}

// refine + run in one call, the refined grid kept in the arithmetic type
void* mdmc_oracle_run_refined(const float* coarse, const int dims[3], const float origin[3], const float spacing[3],
                              int refinement, int pad, float iso, const mdmc_oracle_options* opt) {
    const RealInput input(coarse, samplesOf(dims));
    const oracle::Grid cg = gridOf(input, dims, origin, spacing);
    std::vector<oracle::Real> res;
    oracle::Grid g;
    oracle::refine(cg, refinement, pad != 0, res, g.d, g.origin, g.deltas);
    g.v = res.data();
    mdmc_oracle_options o;
    if (opt) o = *opt; else mdmc_oracle_default_options(&o);
    return oracle::run(g, iso, o);
}

void* mdmc_oracle_run(const float* grid, const int dims[3], const float origin[3], const float spacing[3],
                      float iso, const mdmc_oracle_options* opt) {
    const RealInput input(grid, samplesOf(dims));
    const oracle::Grid g = gridOf(input, dims, origin, spacing);
    mdmc_oracle_options o;
    if (opt) o = *opt; else mdmc_oracle_default_options(&o);
    return oracle::run(g, iso, o);
}

void mdmc_oracle_counts(const void* res, int64_t counts[MDMC_ORC_NUM_COUNTS]) {
    const oracle::Result* r = (const oracle::Result*)res;
    counts[MDMC_ORC_NUM_VERTICES] = (int64_t)(r->pos.size() / 3);
    counts[MDMC_ORC_NUM_FACES] = (int64_t)r->faceFirst.size();
    counts[MDMC_ORC_NUM_HALFEDGES] = (int64_t)r->he.size();
    counts[MDMC_ORC_NUM_DMC_VERTICES] = (int64_t)(r->dmcPos.size() / 3);
    counts[MDMC_ORC_NUM_DMC_QUADS] = (int64_t)r->dmcAttr.size();
}

void mdmc_oracle_stats(const void* res, int64_t stats[MDMC_ORC_NUM_STATS]) {
    const oracle::Result* r = (const oracle::Result*)res;
    std::memcpy(stats, r->stats, sizeof r->stats);
}

void mdmc_oracle_get(const void* res, float* positions, float* normals, int* halfedges, int* face_first,
                     uint16_t* face_attr, uint8_t* vertex_flags, int* vertex_he) {
    const oracle::Result* r = (const oracle::Result*)res;
    if (positions) copyFloats(positions, r->pos);
    if (normals) copyFloats(normals, r->nrm);
    if (halfedges) std::memcpy(halfedges, r->he.data(), r->he.size() * sizeof(oracle::HE));
    if (face_first) std::memcpy(face_first, r->faceFirst.data(), r->faceFirst.size() * sizeof(int));
    if (face_attr) std::memcpy(face_attr, r->faceAttr.data(), r->faceAttr.size() * sizeof(uint16_t));
    if (vertex_flags) std::memcpy(vertex_flags, r->vflags.data(), r->vflags.size());
    if (vertex_he) std::memcpy(vertex_he, r->vertexHE.data(), r->vertexHE.size() * sizeof(int));
}

void mdmc_oracle_get_dmc(const void* res, float* positions, float* normals, int* quads, uint16_t* quad_attr) {
    const oracle::Result* r = (const oracle::Result*)res;
    if (positions) copyFloats(positions, r->dmcPos);
    if (normals) copyFloats(normals, r->dmcNrm);
    if (quads) std::memcpy(quads, r->dmcQuads.data(), r->dmcQuads.size() * sizeof(int));
    if (quad_attr) std::memcpy(quad_attr, r->dmcAttr.data(), r->dmcAttr.size() * sizeof(uint16_t));
}

void mdmc_oracle_free(void* res) { delete (oracle::Result*)res; }

void* mdmc_oracle_standard_mc(const float* grid, const int dims[3], const float origin[3], const float spacing[3],
                              float iso, int64_t counts[2]) {
    const RealInput input(grid, samplesOf(dims));
    const oracle::Grid g = gridOf(input, dims, origin, spacing);
    oracle::MCMesh* m = oracle::standardMC(g, iso);
    counts[0] = (int64_t)(m->pos.size() / 3);
    counts[1] = (int64_t)(m->tris.size() / 3);
    return m;
}

void mdmc_oracle_get_standard_mc(const void* mesh, float* positions, float* normals, int* triangles) {
    const oracle::MCMesh* m = (const oracle::MCMesh*)mesh;
    if (positions) copyFloats(positions, m->pos);
    if (normals) copyFloats(normals, m->nrm);
    if (triangles) std::memcpy(triangles, m->tris.data(), m->tris.size() * sizeof(int));
}

void mdmc_oracle_free_standard_mc(void* mesh) { delete (oracle::MCMesh*)mesh; }

void mdmc_oracle_get_topology(const void* res, int* cells, uint16_t* edges, int* parents) {
    const oracle::Result* r = (const oracle::Result*)res;
    if (cells) std::memcpy(cells, r->dmcCell.data(), r->dmcCell.size() * sizeof(int));
    if (edges) std::memcpy(edges, r->dmcEdges.data(), r->dmcEdges.size() * sizeof(uint16_t));
    if (parents) {
        const size_t V = r->pos.size() / 3;
        for (size_t v = 0; v < V; ++v) parents[v] = v < r->parent.size() ? r->parent[v] : (int)v;
    }
}

// FP64 restatement of the differentiable vertex position (surface iteration
// off): origin + (cell + mean of the contour's edge points) * spacing, the edge
// point taking w = (iso - s0) / (s1 - s0) on the edge's axis
// (computeLocalCoordinateOffset, D/CellIntersection.inl:176-200)
static double gridAt(const double* g, const int d[3], int x, int y, int z) {
    x = x < 0 ? 0 : (x > d[0] - 1 ? d[0] - 1 : x);
    y = y < 0 ? 0 : (y > d[1] - 1 ? d[1] - 1 : y);
    z = z < 0 ? 0 : (z > d[2] - 1 ? d[2] - 1 : z);
    return g[((size_t)z * d[1] + y) * d[0] + x];
}

void mdmc_oracle_positions_f64(const void* res, const double* grid, const int dims[3], const double origin[3],
                               const double spacing[3], double iso, double* out) {
    const oracle::Result* r = (const oracle::Result*)res;
    const size_t Vd = r->dmcEdges.size();
    for (size_t v = 0; v < Vd; ++v) {
        const int* c = &r->dmcCell[3 * v];
        double s[8];
        for (int k = 0; k < 8; ++k) s[k] = gridAt(grid, dims, c[0] + (k & 1), c[1] + ((k >> 1) & 1), c[2] + ((k >> 2) & 1));
        double q[3] = {0, 0, 0};
        int n = 0;
        for (int e = 0; e < 12; ++e) {
            if (!((r->dmcEdges[v] >> e) & 1)) continue;
            const int a0 = oracle::kEdgeV0[e], a1 = oracle::kEdgeV1[e], ax = oracle::kEdgeAxis[e];
            double p[3] = {(double)(a0 & 1), (double)((a0 >> 1) & 1), (double)((a0 >> 2) & 1)};
            p[ax] = (iso - s[a0]) / (s[a1] - s[a0]);
            for (int a = 0; a < 3; ++a) q[a] += p[a];
            ++n;
        }
        for (int a = 0; a < 3; ++a) out[3 * v + a] = origin[a] + ((double)c[a] + q[a] / n) * spacing[a];
    }
}

// FP64 gradient of sum_v dLdpos[v] . pos[v] with respect to the grid samples,
// added to out.  Final vertices that the splitter made pass their gradient to
// the DMC vertex they descend from.
void mdmc_oracle_backward(const void* res, const double* grid, const int dims[3], const double spacing[3], double iso,
                          const double* dLdpos, double* out) {
    const oracle::Result* r = (const oracle::Result*)res;
    const size_t Vd = r->dmcEdges.size(), V = r->pos.size() / 3;
    std::vector<double> gs(3 * Vd, 0.0);
    for (size_t v = 0; v < V; ++v) {
        const int p = v < Vd ? (int)v : (v < r->parent.size() ? r->parent[v] : -1);
        if (p < 0 || (size_t)p >= Vd) continue;
        for (int a = 0; a < 3; ++a) gs[3 * p + a] += dLdpos[3 * v + a];
    }
    for (size_t v = 0; v < Vd; ++v) {
        const int* c = &r->dmcCell[3 * v];
        int idx[8];
        double s[8];
        for (int k = 0; k < 8; ++k) {
            int x = c[0] + (k & 1), y = c[1] + ((k >> 1) & 1), z = c[2] + ((k >> 2) & 1);
            x = x > dims[0] - 1 ? dims[0] - 1 : x;
            y = y > dims[1] - 1 ? dims[1] - 1 : y;
            z = z > dims[2] - 1 ? dims[2] - 1 : z;
            idx[k] = (int)(((size_t)z * dims[1] + y) * dims[0] + x);
            s[k] = grid[idx[k]];
        }
        int n = 0;
        for (int e = 0; e < 12; ++e) n += (r->dmcEdges[v] >> e) & 1;
        for (int e = 0; e < 12; ++e) {
            if (!((r->dmcEdges[v] >> e) & 1)) continue;
            const int a0 = oracle::kEdgeV0[e], a1 = oracle::kEdgeV1[e], ax = oracle::kEdgeAxis[e];
            const double d = s[a1] - s[a0];
            const double coef = gs[3 * v + ax] * spacing[ax] / n;
            out[idx[a0]] += coef * (iso - s[a1]) / (d * d);
            out[idx[a1]] += coef * (-(iso - s[a0]) / (d * d));
        }
    }
}

// refineGrid's weights (D/UniformGrid.inl:279-319) applied in FP64, and their
// adjoint: every refined sample is a fixed trilinear combination of 8 coarse
// samples (clamped indices; the padded layer repeats the boundary)
static void refineWeights(const int in[3], int r, int pad, int x, int y, int z, int idx[8], double w[8]) {
    int od[3];
    for (int a = 0; a < 3; ++a) od[a] = in[a] + (in[a] - 1) * r + (pad ? 2 : 0);
    int ix = x, iy = y, iz = z;
    if (pad) {
        ix = std::min(std::max(ix, 1), od[0] - 2) - 1;
        iy = std::min(std::max(iy, 1), od[1] - 2) - 1;
        iz = std::min(std::max(iz, 1), od[2] - 2) - 1;
    }
    const float f = (float)(r + 1);
    const float qx = (float)ix / f, qy = (float)iy / f, qz = (float)iz / f;
    const int mx = (int)std::floor(qx), my = (int)std::floor(qy), mz = (int)std::floor(qz);
    const double dx = (double)(qx - (float)mx), dy = (double)(qy - (float)my), dz = (double)(qz - (float)mz);
    for (int k = 0; k < 8; ++k) {
        int cx = mx + (k & 1), cy = my + ((k >> 1) & 1), cz = mz + ((k >> 2) & 1);
        cx = cx < 0 ? 0 : (cx > in[0] - 1 ? in[0] - 1 : cx);
        cy = cy < 0 ? 0 : (cy > in[1] - 1 ? in[1] - 1 : cy);
        cz = cz < 0 ? 0 : (cz > in[2] - 1 ? in[2] - 1 : cz);
        idx[k] = (int)(((size_t)cz * in[1] + cy) * in[0] + cx);
        w[k] = ((k & 1) ? dx : 1.0 - dx) * (((k >> 1) & 1) ? dy : 1.0 - dy) * (((k >> 2) & 1) ? dz : 1.0 - dz);
    }
}

void mdmc_oracle_refine_f64(const double* in, const int dims[3], int r, int pad, double* out) {
    int od[3];
    for (int a = 0; a < 3; ++a) od[a] = dims[a] + (dims[a] - 1) * r + (pad ? 2 : 0);
    for (int z = 0; z < od[2]; ++z)
        for (int y = 0; y < od[1]; ++y)
            for (int x = 0; x < od[0]; ++x) {
                int idx[8];
                double w[8], v = 0.0;
                refineWeights(dims, r, pad, x, y, z, idx, w);
                for (int k = 0; k < 8; ++k) v += w[k] * in[idx[k]];
                out[((size_t)z * od[1] + y) * od[0] + x] = v;
            }
}

void mdmc_oracle_refine_backward(const double* dout, const int dims[3], int r, int pad, double* din) {
    int od[3];
    for (int a = 0; a < 3; ++a) od[a] = dims[a] + (dims[a] - 1) * r + (pad ? 2 : 0);
    for (int z = 0; z < od[2]; ++z)
        for (int y = 0; y < od[1]; ++y)
            for (int x = 0; x < od[0]; ++x) {
                const double g = dout[((size_t)z * od[1] + y) * od[0] + x];
                if (g == 0.0) continue;
                int idx[8];
                double w[8];
                refineWeights(dims, r, pad, x, y, z, idx, w);
                for (int k = 0; k < 8; ++k) din[idx[k]] += w[k] * g;
            }
}

int mdmc_oracle_case_ambiguous(int c) { return oracle::caseIsAmbiguous(c) ? 1 : 0; }

// FaceColoring::colorFaces (O/FaceColoring.cu:116-141; color_faces :13-66,
// optimize_face_coloring :67-116): classes 5..23 in turn pick the first free
// color of 0..4 (the test for 4 compares c2 twice and never c3, :63), then
// the faces of color 4 the first free of 0..3.  Faces of the class being
// recolored see each other with their color from before that pass.
void mdmc_oracle_color_faces(const int32_t* halfedges, int64_t num_halfedges, const int32_t* face_first,
                             uint16_t* face_attr, int64_t num_faces) {
    std::vector<int> orig(num_faces);
    auto neighbours = [&](int64_t f, int cls, const std::vector<int>& mark, int nc[4]) {
        int e = face_first[f];
        for (int k = 0; k < 4; ++k) {
            nc[k] = -1;
            if (e < 0 || e >= num_halfedges) continue;
            const int t = halfedges[4 * (int64_t)e + 3];
            if (t > -1 && t < num_halfedges) {
                const int g = halfedges[4 * (int64_t)t + 1];
                if (g >= 0 && g < num_faces) nc[k] = mark[g] == cls ? cls : (face_attr[g] & 0x1F);
            }
            e = halfedges[4 * (int64_t)e + 2];
        }
    };
    auto setColor = [&](int64_t f, int c) { face_attr[f] = (uint16_t)((face_attr[f] & ~0x1F) | c); };
    for (int64_t f = 0; f < num_faces; ++f) orig[f] = face_attr[f] & 0x1F;
    for (int cls = 5; cls < 24; ++cls) {
        std::vector<std::pair<int64_t, int>> next;
        for (int64_t f = 0; f < num_faces; ++f) {
            if (orig[f] != cls) continue;
            int c[4];
            neighbours(f, cls, orig, c);
            int pick = -1;
            for (int k = 0; k < 4 && pick < 0; ++k)
                if (c[0] != k && c[1] != k && c[2] != k && c[3] != k) pick = k;
            if (pick < 0 && c[0] != 4 && c[1] != 4 && c[2] != 4) pick = 4;
            if (pick >= 0) next.push_back({f, pick});
        }
        for (auto& fc : next) setColor(fc.first, fc.second);
    }
    std::vector<int> four(num_faces);
    for (int64_t f = 0; f < num_faces; ++f) four[f] = (face_attr[f] & 0x1F) == 4 ? 4 : 0xFF;
    std::vector<std::pair<int64_t, int>> next;
    for (int64_t f = 0; f < num_faces; ++f) {
        if (four[f] != 4) continue;
        int c[4];
        neighbours(f, 4, four, c);
        for (int k = 0; k < 4; ++k)
            if (c[0] != k && c[1] != k && c[2] != k && c[3] != k) {
                next.push_back({f, k});
                break;
            }
    }
    for (auto& fc : next) setColor(fc.first, fc.second);
}

// quadrilateral_to_triangle, O/DualMarchingCubes.cu:51-60
void mdmc_oracle_quads_to_triangles(const int32_t* quads, int64_t num_quads, int32_t* tris) {
    for (int64_t q = 0; q < num_quads; ++q) {
        const int32_t* v = quads + 4 * q;
        int32_t* t = tris + 6 * q;
        t[0] = v[0];
        t[1] = v[1];
        t[2] = v[3];
        t[3] = v[3];
        t[4] = v[2];
        t[5] = v[0];
    }
}

// QualityMeasure::mean_ratio and area, O/QualityMeasure.h:45-66
void mdmc_oracle_mean_ratio(const float* pos, const int32_t* tris, int64_t num_triangles, float* q) {
    for (int64_t t = 0; t < num_triangles; ++t) {
        const float* p0 = pos + 3 * (int64_t)tris[3 * t];
        const float* p1 = pos + 3 * (int64_t)tris[3 * t + 1];
        const float* p2 = pos + 3 * (int64_t)tris[3 * t + 2];
        const float l0 = (p1[0] - p0[0]) * (p1[0] - p0[0]) + (p1[1] - p0[1]) * (p1[1] - p0[1]) +
                         (p1[2] - p0[2]) * (p1[2] - p0[2]);
        const float l1 = (p2[0] - p1[0]) * (p2[0] - p1[0]) + (p2[1] - p1[1]) * (p2[1] - p1[1]) +
                         (p2[2] - p1[2]) * (p2[2] - p1[2]);
        const float l2 = (p0[0] - p2[0]) * (p0[0] - p2[0]) + (p0[1] - p2[1]) * (p0[1] - p2[1]) +
                         (p0[2] - p2[2]) * (p0[2] - p2[2]);
        const float l = l0 + l1 + l2;
        const float x1 = p1[0] - p0[0], x2 = p2[0] - p0[0];
        const float y1 = p1[1] - p0[1], y2 = p2[1] - p0[1];
        const float z1 = p1[2] - p0[2], z2 = p2[2] - p0[2];
        const float a1 = (y1 * z2 - z1 * y2) * (y1 * z2 - z1 * y2);
        const float a2 = (x1 * z2 - z1 * x2) * (x1 * z2 - z1 * x2);
        const float a3 = (x1 * y2 - y1 * x2) * (x1 * y2 - y1 * x2);
        const float a = std::sqrt(a1 + a2 + a3);
        q[t] = 2.0f * std::sqrt(3.0f) * a / l;
    }
}

}  // extern "C"
