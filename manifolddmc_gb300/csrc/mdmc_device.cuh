// Device-side building blocks of the Dual Marching Cubes path.
//
// Every float expression keeps the reference's operation order (glm
// semantics) and the library is compiled with -fmad=false, so results are
// rounded exactly as the reference's expressions are written; the CPU oracle
// does the same and the two agree bit for bit.
#pragma once

#include <cstdint>

#include "mc_contour_table.h"
#include "mdmc_types.h"

namespace mdmc {

// ---------------------------------------------------------------------------
// float3 helpers (glm::vec3 arithmetic, one rounding per operation)
// ---------------------------------------------------------------------------
struct F3 {
    float x, y, z;
};
__host__ __device__ __forceinline__ F3 f3(float x, float y, float z) { return {x, y, z}; }
__host__ __device__ __forceinline__ F3 operator+(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ F3 operator-(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ F3 operator*(F3 a, F3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__host__ __device__ __forceinline__ F3 operator/(F3 a, F3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
__host__ __device__ __forceinline__ F3 operator*(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__host__ __device__ __forceinline__ F3 operator*(float s, F3 a) { return {s * a.x, s * a.y, s * a.z}; }
__host__ __device__ __forceinline__ F3 operator/(F3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__host__ __device__ __forceinline__ float gmin(float x, float y) { return (y < x) ? y : x; }
__host__ __device__ __forceinline__ float gmax(float x, float y) { return (x < y) ? y : x; }
__host__ __device__ __forceinline__ float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
// glm::normalize: v * (1 / sqrt((x*x + y*y) + z*z))
__device__ __forceinline__ F3 gnormalize(F3 v) {
    float d = v.x * v.x + v.y * v.y;
    d = d + v.z * v.z;
    float inv = 1.0f / sqrtf(d);
    return v * inv;
}

constexpr float kEpsilon = 0.0001f;  // LazyEngine::Constants::EPSILON

// Interpolation<float>::interpolateTrilinearly, D/Utils/Interpolation.inl:76-84
__device__ __forceinline__ float trilinear(const float s[8], F3 p) {
    float a = s[0] + p.x * (s[1] - s[0]);
    float b = s[2] + p.x * (s[3] - s[2]);
    float c = s[4] + p.x * (s[5] - s[4]);
    float e = s[6] + p.x * (s[7] - s[6]);
    float lo = (1.f - p.y) * a + p.y * b;
    float hi = (1.f - p.y) * c + p.y * e;
    return (1.f - p.z) * lo + p.z * hi;
}

// ---------------------------------------------------------------------------
// cell edges and the packed contour word (D/CellIntersection.h:28-137)
// ---------------------------------------------------------------------------
// corner pair of every cell edge; corner i sits at (i&1, (i>>1)&1, (i>>2)&1)
__host__ __device__ constexpr int edgeV0(int e) { return (int)((0x231046540210ULL >> (4 * e)) & 0xF); }
__host__ __device__ constexpr int edgeV1(int e) { return (int)((0x675467752331ULL >> (4 * e)) & 0xF); }
// axis of every edge (0 = x, 1 = y, 2 = z)
__host__ __device__ constexpr int edgeAxis(int e) { return (int)((0xAA4444u >> (2 * e)) & 0x3); }

__host__ __device__ __forceinline__ int nib(uint64_t w, int i) { return (int)((w >> (4 * i)) & 0xF); }
__device__ __forceinline__ int contourSize(uint64_t c, int t) { return nib(c, t); }
__device__ __forceinline__ int contourEdge(uint64_t c, int t, int pos) {
    int before = 0;
    for (int k = 0; k < t; ++k) before += nib(c, k);
    return (int)((c >> (16 + 4 * (before + pos))) & 0xF);
}
__device__ __forceinline__ int numContours(uint64_t c) {
    int n = 0;
#pragma unroll
    for (int t = 0; t < 4; ++t) n += nib(c, t) > 0 ? 1 : 0;
    return n;
}

// quad slot of an edge (computeVertexPosition, D/CellIntersection.inl:361-366)
__host__ __device__ constexpr int quadSlot(int e, int edgyBit) {
    return (int)((240177437832960ULL >> (4 * e + 2 * edgyBit)) & 3);
}

// a face of the cell has the diagonal sign pattern (four crossing edges)
__host__ __device__ constexpr bool caseHasDiagonalFace(int c) {
    const unsigned short fc[6] = {0x3120, 0x6475, 0x1504, 0x7362, 0x2064, 0x7531};
    for (int f = 0; f < 6; ++f) {
        int m = 0;
        for (int i = 0; i < 4; ++i) m |= ((c >> ((fc[f] >> (4 * i)) & 0xF)) & 1) << i;
        if (m == 6 || m == 9) return true;
    }
    return false;
}
// The reference takes the asymptotic-decider path for a case
// (s_triangleAmbiguities == MC_AMBIGUOUS, D/DualMarchingCubes.cpp:301) exactly
// when a face of the cell has the diagonal sign pattern, or when the inside
// corners are just the two ends of one cell diagonal (or all but those two).
__host__ __device__ constexpr bool caseIsAmbiguous(int c) {
    if (caseHasDiagonalFace(c)) return true;
    for (int i = 0; i < 4; ++i) {
        int pair = (1 << i) | (1 << (7 - i));
        if (c == pair || c == (255 ^ pair)) return true;
    }
    return false;
}

// marchingCubesAsymptoticPolygon, D/CellIntersection.inl:202-338.  Faces are
// classified, their oriented segments connected, ambiguous faces decided by
// the bilinear saddle value, and the segments chained into contours starting
// from the lowest unused edge.
// The procedure depends on the cell's values only through its case and, for
// each face with the diagonal pattern, one bit: the decider's value >= iso.
// contoursFromDecisions runs it on those bits (bit f of `hi` for face f), so
// every (case, decisions) pair can be tabulated at compile time below.
// cell faces in the flattened orientation (D/CellIntersection.inl:290-292)
__host__ __device__ constexpr int faceEdgeC(int f, int i) {
    const unsigned short fe[6] = {0x0123, 0x4765, 0x4908, 0x2A6B, 0x83B7, 0x95A1};
    return (fe[f] >> (4 * i)) & 0xF;
}
__host__ __device__ constexpr int faceCornerC(int f, int i) {
    const unsigned short fc[6] = {0x3120, 0x6475, 0x1504, 0x7362, 0x2064, 0x7531};
    return (fc[f] >> (4 * i)) & 0xF;
}
__host__ __device__ constexpr unsigned faceSigns(int cs, int f) {
    unsigned fc = 0;
    for (int i = 0; i < 4; ++i) fc |= (unsigned)((cs >> faceCornerC(f, i)) & 1) << i;
    return fc;
}
__host__ __device__ constexpr uint64_t contoursFromDecisions(int cs, unsigned hi) {
    uint32_t seg[12] = {0xFF, 0xFF, 0xFF, 0xFF, 0xFF, 0xFF, 0xFF, 0xFF, 0xFF, 0xFF, 0xFF, 0xFF};
    auto connect = [&seg](int in, int out) {
        seg[in] = (seg[in] & 0xF0u) | (uint32_t)(out & 0xF);
        seg[out] = (seg[out] & 0x0Fu) | (uint32_t)(in << 4);
    };
    for (int f = 0; f < 6; ++f) {
        const int e0 = faceEdgeC(f, 0), e1 = faceEdgeC(f, 1), e2 = faceEdgeC(f, 2), e3 = faceEdgeC(f, 3);
        const unsigned fc = faceSigns(cs, f);
        const bool h = ((hi >> f) & 1u) != 0;
        switch (fc) {
            case 1: connect(e0, e3); break;
            case 2: connect(e1, e0); break;
            case 3: connect(e1, e3); break;
            case 4: connect(e3, e2); break;
            case 5: connect(e0, e2); break;
            case 7: connect(e1, e2); break;
            case 8: connect(e2, e1); break;
            case 10: connect(e2, e0); break;
            case 11: connect(e2, e3); break;
            case 12: connect(e3, e1); break;
            case 13: connect(e0, e1); break;
            case 14: connect(e3, e0); break;
            case 6:
                if (h) { connect(e3, e0); connect(e1, e2); }
                else { connect(e1, e0); connect(e3, e2); }
                break;
            case 9:
                if (h) { connect(e0, e1); connect(e2, e3); }
                else { connect(e0, e3); connect(e2, e1); }
                break;
            default: break;
        }
    }
    uint64_t c = 0xFFFFFFFFFFFF0000ULL;
    int n = 0;
    int used = 0;  // edges already written, across contours
    for (int edge = 0; edge < 12; ++edge) {
        if (seg[edge] == 0xFF) continue;
        const int start = edge;
        int out = (int)(seg[edge] & 0xF);
        int pos = 0;
        int bit = 16 + 4 * used;
        c = (c & ~(0xFULL << bit)) | ((uint64_t)start << bit);
        int guard = 0;
        while (out != start && guard < 12) {
            ++pos;
            bit = 16 + 4 * (used + pos);
            if (bit <= 60) c = (c & ~(0xFULL << bit)) | ((uint64_t)out << bit);
            const int in = out;
            if (in < 12) {
                out = (int)(seg[in] & 0xF);
                seg[in] = 0xFF;
            } else {
                out = start;
            }
            ++guard;
        }
        if (n < 4) c = (c & ~(0xFULL << (4 * n))) | ((uint64_t)(pos + 1) << (4 * n));
        used += pos + 1;
        ++n;
    }
    return c;
}

// edge -> contour map of a packed contour word (2 bits per edge, contour t
// of every edge of contour t) and, in bits 24-26, the number of contours
__host__ __device__ constexpr uint32_t contourEdgeMap(uint64_t c) {
    int n = 0;
    for (int t = 0; t < 4; ++t) n += ((c >> (4 * t)) & 0xF) != 0 ? 1 : 0;
    uint32_t emap = 0;
    int before = 0;
    for (int t = 0; t < n; ++t) {
        const int sz = (int)((c >> (4 * t)) & 0xF);
        for (int i = 0; i < sz; ++i) emap |= (uint32_t)t << (2 * (int)((c >> (16 + 4 * (before + i))) & 0xF));
        before += sz;
    }
    return emap | ((uint32_t)n << 24);
}

// Per-case tables made at compile time, with the ambiguous cases (which take
// the asymptotic decider instead) tagged so that one shared-memory read both
// classifies a cell and gives its table entry:
// - contour words: 0 = ambiguous with a diagonal face, 1 = ambiguous without
//   (a real word's first contour size is at least 3);
// - edge maps (contourEdgeMap of the word): 0xFFFFFFFF = ambiguous.
struct CaseTables {
    unsigned long long words[256];
    uint32_t edgeMaps[256];
};
constexpr unsigned long long kContourWordsConst[256] = {MDMC_CONTOUR_WORDS};
constexpr CaseTables makeCaseTables() {
    CaseTables t{};
    for (int i = 0; i < 256; ++i) {
        const bool amb = caseIsAmbiguous(i);
        t.words[i] = amb ? (caseHasDiagonalFace(i) ? 0ull : 1ull) : kContourWordsConst[i];
        t.edgeMaps[i] = amb ? 0xFFFFFFFFu : contourEdgeMap(kContourWordsConst[i]);
    }
    return t;
}
__device__ const CaseTables kCaseTables = makeCaseTables();

// Every case with every combination of decisions on its diagonal faces:
// info[cs] = first entry (bits 0-15) | the case's diagonal-face mask << 16;
// entry first + b holds the contour word and edge map for decision bits b
// (bit j: the j-th diagonal face in face order).  656 entries.
__host__ __device__ constexpr unsigned diagonalFaces(int cs) {
    unsigned m = 0;
    for (int f = 0; f < 6; ++f) {
        const unsigned fc = faceSigns(cs, f);
        if (fc == 6 || fc == 9) m |= 1u << f;
    }
    return m;
}
__host__ __device__ constexpr int popcount6(unsigned m) {
    int n = 0;
    for (int f = 0; f < 6; ++f) n += (m >> f) & 1u;
    return n;
}
constexpr int countDecisionEntries() {
    int n = 0;
    for (int cs = 0; cs < 256; ++cs) n += 1 << popcount6(diagonalFaces(cs));
    return n;
}
constexpr int kDecisionEntries = countDecisionEntries();
static_assert(kDecisionEntries == 656, "decision table size");
struct DecisionTables {
    uint32_t info[256];
    unsigned long long words[kDecisionEntries];
    uint32_t edgeMaps[kDecisionEntries];
};
constexpr DecisionTables makeDecisionTables() {
    DecisionTables t{};
    int at = 0;
    for (int cs = 0; cs < 256; ++cs) {
        const unsigned m = diagonalFaces(cs);
        const int k = popcount6(m);
        t.info[cs] = (uint32_t)at | (m << 16);
        for (unsigned b = 0; b < (1u << k); ++b) {
            // spread decision bits b over the diagonal faces
            unsigned hi = 0;
            int j = 0;
            for (int f = 0; f < 6; ++f)
                if ((m >> f) & 1u) hi |= ((b >> j++) & 1u) << f;
            t.words[at + (int)b] = contoursFromDecisions(cs, hi);
            t.edgeMaps[at + (int)b] = contourEdgeMap(t.words[at + (int)b]);
        }
        at += 1 << k;
    }
    return t;
}
__device__ const DecisionTables kDecisionTables = makeDecisionTables();

// marchingCubesAsymptoticPolygon on the cell's values: the case, the
// decider's bit for each diagonal face (the bilinear saddle value
// (v0 v3 - v1 v2) / (v0 + v3 - v1 - v2) against iso, D/CellIntersection.inl:
// 248-252), and the entry of that combination.  Not inlined: the passes
// that call it run it for a minority of cells, and kept out of line it
// leaves their common path smaller (refined vertex pass 115 -> 106 us,
// 256^3 noise DMC stage 7.1 -> 6.9 ms).
static __device__ __noinline__ int asymptoticEntry(const float s[8], float iso) {
    int cs = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) cs |= (s[i] >= iso ? 1 : 0) << i;
    const uint32_t info = kDecisionTables.info[cs];
    const unsigned m = info >> 16;
    unsigned bits = 0;
    int j = 0;
#pragma unroll
    for (int f = 0; f < 6; ++f) {
        if (!((m >> f) & 1u)) continue;
        const float v0 = s[faceCornerC(f, 0)], v1 = s[faceCornerC(f, 1)], v2 = s[faceCornerC(f, 2)],
                    v3 = s[faceCornerC(f, 3)];
        const float num = v0 * v3 - v1 * v2;
        float den = v0 + v3;
        den = den - v1;
        den = den - v2;
        const float decision = num / den;
        bits |= (decision >= iso ? 1u : 0u) << j;
        ++j;
    }
    return (int)(info & 0xFFFFu) + (int)bits;
}
__device__ __forceinline__ uint64_t asymptoticContours(const float s[8], float iso) {
    return kDecisionTables.words[asymptoticEntry(s, iso)];
}

// contours of an active cell from a tagged word table (above)
__device__ __forceinline__ uint64_t taggedContours(uint64_t word, const float s[8], float iso) {
    return word <= 1 ? asymptoticContours(s, iso) : word;
}

// contours of an active cell: table word or asymptotic decider
__device__ __forceinline__ uint64_t cellContours(int cs, const float s[8], float iso, const uint64_t* table) {
    if (caseIsAmbiguous(cs)) return asymptoticContours(s, iso);
    return table[cs];
}

// VertexToSurfaceIterator, D/CellIntersection.inl:12-122
struct SurfaceIterator {
    const float* s;
    float iso;

    __device__ F3 gradient(F3 p) const {
        float gx = (1 - p.z) * ((1 - p.y) * (s[1] - s[0]) + p.y * (s[3] - s[2])) +
                   p.z * ((1 - p.y) * (s[5] - s[4]) + p.y * (s[7] - s[6]));
        float gy = (1 - p.z) * ((1 - p.x) * (s[2] - s[0]) + p.x * (s[3] - s[1])) +
                   p.z * ((1 - p.x) * (s[6] - s[4]) + p.x * (s[7] - s[5]));
        float gz = (1 - p.y) * ((1 - p.x) * (s[4] - s[0]) + p.x * (s[5] - s[1])) +
                   p.y * ((1 - p.x) * (s[6] - s[2]) + p.x * (s[7] - s[3]));
        return f3(gx, gy, gz);
    }
    __device__ bool update(F3& point, F3& grad, F3 in1, F3& in2, float v1, float& v2, bool cl[3]) const {
        grad = gnormalize(grad);
        in2 = in1 + 0.05f * grad;
        cl[0] = in2.x <= 0.f || in2.x >= 1.f;
        cl[1] = in2.y <= 0.f || in2.y >= 1.f;
        cl[2] = in2.z <= 0.f || in2.z >= 1.f;
        in2 = f3(gclamp(in2.x, 0.f, 1.f), gclamp(in2.y, 0.f, 1.f), gclamp(in2.z, 0.f, 1.f));
        v2 = trilinear(s, in2);
        if ((v1 <= iso && iso <= v2) || (v2 <= iso && iso <= v1)) {
            float e = v1;
            if (v1 != v2) e = (iso - v1) / (v2 - v1);
            point = in1 + e * (in2 - in1);
            return true;
        }
        return false;
    }
    __device__ void move(F3& point) const {
        F3 in1 = point;
        float v1 = trilinear(s, in1);
        float v2 = 0.f;
        for (int i = 0; i < 30; ++i) {
            F3 g = gradient(in1);
            if (v1 > iso) g = f3(-g.x, -g.y, -g.z);
            F3 in2 = in1;
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
        const float lo = kEpsilon, hi = 1.f - kEpsilon;
        point = f3(gclamp(point.x, lo, hi), gclamp(point.y, lo, hi), gclamp(point.z, lo, hi));
    }
};

// ---------------------------------------------------------------------------
// grid access.  Two views share the geometry: PlainView reads a dense grid;
// RefinedView evaluates the refined and/or padded grid of refineGrid
// (D/UniformGrid.inl:279-319) from the coarse input on demand, with the same
// float operations, so it returns exactly the values the dense refined grid
// would hold without that grid ever being written.
// ---------------------------------------------------------------------------
// Unsigned division by a divisor fixed for a launch, as a multiply-high and
// two shifts (Granlund and Montgomery, "Division by Invariant Integers using
// Multiplication", PLDI 1994, section 4): for 1 <= d < 2^31 and every 32-bit
// n, n / d = (t + ((n - t) >> s1)) >> s2 with t = umulhi(m, n),
// l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1, s1 = min(l, 1),
// s2 = max(l - 1, 0).  Exact; made on the host.
struct FastDiv {
    uint32_t d = 1, m = 1, s1 = 0, s2 = 0;
    FastDiv() = default;
    __host__ explicit FastDiv(uint32_t div) : d(div < 1 ? 1 : div) {
        uint32_t l = 0;
        while ((1ull << l) < d) ++l;
        m = (uint32_t)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
        s1 = l > 0 ? 1 : 0;
        s2 = l > 0 ? l - 1 : 0;
    }
    __device__ __forceinline__ uint32_t div(uint32_t n) const {
        const uint32_t t = __umulhi(m, n);
        return (t + ((n - t) >> s1)) >> s2;
    }
};

struct GridGeom {
    FastDiv divX, divY;  // by X and Y (decoding linear sample ids; set by setDivisors)
    int X, Y, Z;       // samples of the (refined) grid
    float ox, oy, oz;  // origin
    float dx, dy, dz;  // spacing
    __device__ __forceinline__ F3 origin() const { return f3(ox, oy, oz); }
    __device__ __forceinline__ F3 deltas() const { return f3(dx, dy, dz); }
    // getIndex3DFromPosition, D/UniformGrid.inl:441-448
    __device__ __forceinline__ void cellOf(F3 p, int c[3]) const {
        F3 off = (p - origin()) / deltas();
        c[0] = (int)floorf(off.x);
        c[1] = (int)floorf(off.y);
        c[2] = (int)floorf(off.z);
    }
};

struct PlainView : GridGeom {
    const float* v;
    static constexpr bool kRefined = false;
    __device__ __forceinline__ float at(int x, int y, int z) const { return __ldg(v + ((size_t)z * Y + y) * X + x); }
};

struct RefinedView : GridGeom {
    const float* c;            // coarse samples
    int cX, cY, cZ;            // coarse dims
    int r, pad;                // refinement, replicated boundary layer
    float f;                   // r + 1
    const uint32_t* mayCross;  // per coarse cell: may a refined cell inside cross iso (bitmask, x fastest)
    static constexpr bool kRefined = true;

    float invf;                // 1 / f when f is a power of two (then i * invf == i / f exactly)
    int fPow2;
    FastDiv divCX1, divCY1;    // by the coarse cells per row and per layer (set by setDivisors)

    // sample index of the unpadded refined grid (refineGrid's clamp and shift)
    __device__ __forceinline__ int unpad(int i, int n) const { return pad ? min(max(i, 1), n - 2) - 1 : i; }
    // (float)i / f, computed by a multiplication when that is exact
    __device__ __forceinline__ float divf(int i) const { return fPow2 ? (float)i * invf : (float)i / f; }
    __device__ __forceinline__ float at(int x, int y, int z) const {
        x = unpad(x, X);
        y = unpad(y, Y);
        z = unpad(z, Z);
        const float qx = divf(x), qy = divf(y), qz = divf(z);
        const int mx = (int)floorf(qx), my = (int)floorf(qy), mz = (int)floorf(qz);
        const F3 diff = f3(qx - (float)mx, qy - (float)my, qz - (float)mz);
        float s[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int cx = min(max(mx + (k & 1), 0), cX - 1);
            const int cy = min(max(my + ((k >> 1) & 1), 0), cY - 1);
            const int cz = min(max(mz + ((k >> 2) & 1), 0), cZ - 1);
            s[k] = __ldg(c + ((size_t)cz * cY + cy) * cX + cx);
        }
        return trilinear(s, diff);
    }
    // coarse cell containing the refined cell whose lowest corner is i
    __device__ __forceinline__ int coarseCell(int i, int n, int cn) const {
        const int u = unpad(i, n);
        return min((int)floorf(divf(u)), cn - 2);
    }
    __device__ __forceinline__ bool coarseMayCross(int mx, int my, int mz) const {
        const size_t bit = ((size_t)mz * (cY - 1) + my) * (size_t)(cX - 1) + mx;
        return (__ldg(mayCross + (bit >> 5)) >> (bit & 31)) & 1u;
    }
};

template <class View>
__device__ __forceinline__ float atClamped(const View& g, int x, int y, int z) {
    x = x < 0 ? 0 : (x > g.X - 1 ? g.X - 1 : x);
    y = y < 0 ? 0 : (y > g.Y - 1 ? g.Y - 1 : y);
    z = z < 0 ? 0 : (z > g.Z - 1 ? g.Z - 1 : z);
    return g.at(x, y, z);
}

// UniformGrid::evaluateCellCornerValues, D/UniformGrid.inl:414-427
template <class View>
__device__ __forceinline__ void corners(const View& g, int x, int y, int z, float s[8]) {
#pragma unroll
    for (int i = 0; i < 8; ++i) s[i] = atClamped(g, x + (i & 1), y + ((i >> 1) & 1), z + ((i >> 2) & 1));
}

// UniformGrid::computeGradients, D/UniformGrid.inl:325-379
template <class View>
__device__ inline void cornerGradients(const View& g, int x, int y, int z, const float s[8], F3 out[8]) {
    auto cl = [](int dim, int ii) { return ii < 0 ? 0 : (ii >= dim ? dim - 1 : ii); };
    const int X = g.X, Y = g.Y, Z = g.Z;
    F3 gr[8];
    gr[0] = f3(s[1] - g.at(cl(X, x - 1), y, z), s[2] - g.at(x, cl(Y, y - 1), z), s[4] - g.at(x, y, cl(Z, z - 1)));
    gr[1] = f3(g.at(cl(X, x + 2), y, z) - s[0], s[3] - g.at(x + 1, cl(Y, y - 1), z), s[5] - g.at(x + 1, y, cl(Z, z - 1)));
    gr[2] = f3(s[3] - g.at(cl(X, x - 1), y + 1, z), g.at(x, cl(Y, y + 2), z) - s[0], s[6] - g.at(x, y + 1, cl(Z, z - 1)));
    gr[3] = f3(g.at(cl(X, x + 2), y + 1, z) - s[2], g.at(x + 1, cl(Y, y + 2), z) - s[1],
               s[7] - g.at(x + 1, y + 1, cl(Z, z - 1)));
    gr[4] = f3(s[5] - g.at(cl(X, x - 1), y, z + 1), s[6] - g.at(x, cl(Y, y - 1), z + 1), g.at(x, y, cl(Z, z + 2)) - s[0]);
    gr[5] = f3(g.at(cl(X, x + 2), y, z + 1) - s[4], s[7] - g.at(x + 1, cl(Y, y - 1), z + 1),
               g.at(x + 1, y, cl(Z, z + 2)) - s[1]);
    gr[6] = f3(s[7] - g.at(cl(X, x - 1), y + 1, z + 1), g.at(x, cl(Y, y + 2), z + 1) - s[4],
               g.at(x, y + 1, cl(Z, z + 2)) - s[2]);
    gr[7] = f3(g.at(cl(X, x + 2), y + 1, z + 1) - s[6], g.at(x + 1, cl(Y, y + 2), z + 1) - s[5],
               g.at(x + 1, y + 1, cl(Z, z + 2)) - s[3]);
    const F3 dl = g.deltas();
#pragma unroll
    for (int i = 0; i < 8; ++i) out[i] = (0.5f * gr[i]) / dl;
}

// The samples a cell's corners and corner gradients read: stencil sample
// (i, j, k), i, j, k in 0..3, is View::at(clamp(x - 1 + i), clamp(y - 1 + j),
// clamp(z - 1 + k)) with the same float operations.  The per-axis part of
// each coordinate (clamped sample offset; for refined grids the coarse index
// pair and fraction) is computed once per cell instead of once per sample.
template <class View>
struct CellStencil;

template <>
struct CellStencil<PlainView> {
    const float* v;
    int xo[4];
    int64_t yo[4], zo[4];
    __device__ __forceinline__ CellStencil(const PlainView& g, int x, int y, int z) : v(g.v) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            xo[k] = min(max(x - 1 + k, 0), g.X - 1);
            yo[k] = (int64_t)min(max(y - 1 + k, 0), g.Y - 1) * g.X;
            zo[k] = (int64_t)min(max(z - 1 + k, 0), g.Z - 1) * g.Y * g.X;
        }
    }
    __device__ __forceinline__ float at(int i, int j, int k) const { return __ldg(v + zo[k] + yo[j] + xo[i]); }
};

// (refined grids have fewer than 2^32 samples, so their coarse grids too:
// 32-bit element offsets suffice)
template <>
struct CellStencil<RefinedView> {
    const float* c;
    uint32_t x0[4], x1[4], y0[4], y1[4], z0[4], z1[4];
    float dx[4], dy[4], dz[4];
    __device__ __forceinline__ static void axis(const RefinedView& g, int p, int n, int cn, uint32_t stride, uint32_t& o0,
                                                uint32_t& o1, float& d) {
        const int u = g.unpad(min(max(p, 0), n - 1), n);
        const float q = g.divf(u);
        const int m = (int)floorf(q);
        d = q - (float)m;
        o0 = (uint32_t)min(max(m, 0), cn - 1) * stride;
        o1 = (uint32_t)min(max(m + 1, 0), cn - 1) * stride;
    }
    __device__ __forceinline__ CellStencil(const RefinedView& g, int x, int y, int z) : c(g.c) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            axis(g, x - 1 + k, g.X, g.cX, 1u, x0[k], x1[k], dx[k]);
            axis(g, y - 1 + k, g.Y, g.cY, (uint32_t)g.cX, y0[k], y1[k], dy[k]);
            axis(g, z - 1 + k, g.Z, g.cZ, (uint32_t)g.cX * (uint32_t)g.cY, z0[k], z1[k], dz[k]);
        }
    }
    __device__ __forceinline__ float at(int i, int j, int k) const {
        float s[8];
        s[0] = __ldg(c + (z0[k] + y0[j] + x0[i]));
        s[1] = __ldg(c + (z0[k] + y0[j] + x1[i]));
        s[2] = __ldg(c + (z0[k] + y1[j] + x0[i]));
        s[3] = __ldg(c + (z0[k] + y1[j] + x1[i]));
        s[4] = __ldg(c + (z1[k] + y0[j] + x0[i]));
        s[5] = __ldg(c + (z1[k] + y0[j] + x1[i]));
        s[6] = __ldg(c + (z1[k] + y1[j] + x0[i]));
        s[7] = __ldg(c + (z1[k] + y1[j] + x1[i]));
        return trilinear(s, f3(dx[i], dy[j], dz[k]));
    }
};

// The stencil of a refined grid whose refinement factor f is at least 3,
// evaluated separably.  Along an axis the four stencil positions span at most
// three refined steps, so their coarse index pairs are (b + e, b + e + 1)
// with e in {0, 1} for one base b: the stencil reads a 3x3x3 block of coarse
// samples.  RefinedView::at's trilinear interpolation takes x-lerps along
// coarse rows, then y-lerps of two x-lerps, then the z-lerp of two y-lerps;
// here each x-lerp (position i, coarse row) and y-lerp (positions i, j,
// coarse layer) is computed once from the 27 loaded samples, with the
// operands and operations at() uses, and the 32 samples the corners and
// gradients read are finished by their z-lerps.  Valid when e stays in
// {0, 1}: f >= 3 and the rounding of i / f never reaches the next integer,
// which holds for f and the refined dims up to 2^20 (sepStencilApplies).
struct SepStencil {
    float v[4][4][4];  // [k][j][i]; only samples with at most one index outside 1..2 are set
    __device__ __forceinline__ float at(int i, int j, int k) const { return v[k][j][i]; }

    // the axis's coarse rows (element offsets) and per-position fraction and row step
    __device__ __forceinline__ static void axis(const RefinedView& g, int p, int n, int cn, uint32_t stride,
                                                uint32_t o[3], float d[4], bool up[4]) {
        int b = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int u = g.unpad(min(max(p - 1 + j, 0), n - 1), n);
            const float q = g.divf(u);
            const int m = (int)floorf(q);
            d[j] = q - (float)m;
            if (j == 0) b = m;
            up[j] = m != b;
        }
#pragma unroll
        for (int r = 0; r < 3; ++r) o[r] = (uint32_t)min(max(b + r, 0), cn - 1) * stride;
    }

    __device__ __forceinline__ SepStencil(const RefinedView& g, int x, int y, int z) {
        uint32_t ox[3], oy[3], oz[3];
        float dx[4], dy[4], dz[4];
        bool ux[4], uy[4], uz[4];
        axis(g, x, g.X, g.cX, 1u, ox, dx, ux);
        axis(g, y, g.Y, g.cY, (uint32_t)g.cX, oy, dy, uy);
        axis(g, z, g.Z, g.cZ, (uint32_t)g.cX * (uint32_t)g.cY, oz, dz, uz);
        float yl[3][4][4];  // [coarse layer][j][i]
#pragma unroll
        for (int rz = 0; rz < 3; ++rz) {
            float xl[3][4];  // [coarse row][i]
#pragma unroll
            for (int ry = 0; ry < 3; ++ry) {
                const float* row = g.c + (oz[rz] + oy[ry]);
                const float c0 = __ldg(row + ox[0]), c1 = __ldg(row + ox[1]), c2 = __ldg(row + ox[2]);
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const float s0 = ux[i] ? c1 : c0, s1 = ux[i] ? c2 : c1;
                    xl[ry][i] = s0 + dx[i] * (s1 - s0);
                }
            }
#pragma unroll
            for (int j = 0; j < 4; ++j)
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    if ((i == 0 || i == 3) && (j == 0 || j == 3)) continue;
                    const float a = uy[j] ? xl[1][i] : xl[0][i], b = uy[j] ? xl[2][i] : xl[1][i];
                    yl[rz][j][i] = (1.f - dy[j]) * a + dy[j] * b;
                }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int j = 0; j < 4; ++j)
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int outside = (i == 0 || i == 3) + (j == 0 || j == 3) + (k == 0 || k == 3);
                    if (outside > 1) continue;
                    const float lo = uz[k] ? yl[1][j][i] : yl[0][j][i], hi = uz[k] ? yl[2][j][i] : yl[1][j][i];
                    v[k][j][i] = (1.f - dz[k]) * lo + dz[k] * hi;
                }
    }
};

// host-side test of SepStencil's condition for a refined grid
__host__ __device__ __forceinline__ bool sepStencilApplies(int refinement, int X, int Y, int Z) {
    const int lim = 1 << 20;
    return refinement >= 2 && refinement < lim && X <= lim && Y <= lim && Z <= lim;
}

// the cell's corner values (corner i at stencil (1 + bit0, 1 + bit1, 1 + bit2))
template <class St>
__device__ __forceinline__ void stencilCorners(const St& st, float s[8]) {
#pragma unroll
    for (int i = 0; i < 8; ++i) s[i] = st.at(1 + (i & 1), 1 + ((i >> 1) & 1), 1 + ((i >> 2) & 1));
}

// 1 / d when d is a power of two whose reciprocal is a normal float.  Then
// x / d and x * (1 / d) are the correctly rounded values of the same real
// number and agree bit for bit.
__device__ __forceinline__ bool pow2Reciprocal(float d, float& inv) {
    const uint32_t b = __float_as_uint(d);
    const uint32_t e = (b >> 23) & 0xFFu;
    inv = __uint_as_float((b & 0x80000000u) | (((254u - e) & 0xFFu) << 23));
    return (b & 0x7FFFFFu) == 0u && e >= 1u && e <= 253u;
}

// cornerGradients from the stencil: along axis a, corner i's neighbour is
// the stencil sample one step outside the cell (index 0 below, 3 above).
// The division by the spacing is a multiplication when that is exact.
template <class St>
__device__ __forceinline__ void stencilGradients(const St& st, const float s[8], F3 dl, F3 out[8]) {
    F3 half[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int bx = i & 1, by = (i >> 1) & 1, bz = (i >> 2) & 1;
        const float nx = st.at(bx ? 3 : 0, 1 + by, 1 + bz);
        const float ny = st.at(1 + bx, by ? 3 : 0, 1 + bz);
        const float nz = st.at(1 + bx, 1 + by, bz ? 3 : 0);
        const F3 gr = f3(bx ? nx - s[i ^ 1] : s[i ^ 1] - nx, by ? ny - s[i ^ 2] : s[i ^ 2] - ny,
                         bz ? nz - s[i ^ 4] : s[i ^ 4] - nz);
        half[i] = 0.5f * gr;
    }
    F3 inv;
    const bool exact = pow2Reciprocal(dl.x, inv.x) & pow2Reciprocal(dl.y, inv.y) & pow2Reciprocal(dl.z, inv.z);
    if (exact) {
#pragma unroll
        for (int i = 0; i < 8; ++i) out[i] = half[i] * inv;
    } else {
#pragma unroll
        for (int i = 0; i < 8; ++i) out[i] = half[i] / dl;
    }
}

// Interpolation<glm::vec3>::interpolateTrilinearly of the corner gradients
__device__ __forceinline__ F3 trilinear3(const F3 n[8], F3 p) {
    float xs[8], ys[8], zs[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) { xs[i] = n[i].x; ys[i] = n[i].y; zs[i] = n[i].z; }
    return f3(trilinear(xs, p), trilinear(ys, p), trilinear(zs, p));
}

}  // namespace mdmc
