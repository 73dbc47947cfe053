// Internal types shared by the library's translation units.
#pragma once

#include <cstddef>
#include <cstdint>

#include "mdmc.h"

namespace mdmc {

// Device status bits.  Kernels never trap: a hit limit sets a bit, the kernel
// skips the offending element and the host reports the bits after the run.
enum : uint32_t {
    kStatusProbeLimit = 1u << 0,       // reserved (no probing structure is left)
    kStatusSlotConflict = 1u << 1,     // two cells claimed the same quad slot
    kStatusBucketOverflow = 1u << 2,   // more than 4 halfedges on one edge
    kStatusPartnerOverflow = 1u << 3,  // merge list longer than the reference's
    kStatusWalkLimit = 1u << 4,        // fan walk did not close
    kStatusBadTwin = 1u << 5,          // twin outside the working copy
    kStatusIterationCap = 1u << 6,     // splitter iteration cap
    kStatusWallOutOfGrid = 1u << 7,    // cell wall outside the grid (clamped)
    kStatusMissingCell = 1u << 8,      // quad neighbour cell not found
    kStatusMappingSwap = 1u << 9,      // unexpected working-copy mapping swap
    kStatusCountMismatch = 1u << 10,   // a write outside the sizes the count pass gave
    kStatusBadIndex = 1u << 11,        // an element id outside its array (skipped)
    kStatusCountOverflow = 1u << 12,   // a vertex's count of non-two-halfedge edges past its field
};

// unsigned range check used before every data-dependent access
// 0 <= i < n (false for every i when n <= 0)
__host__ __device__ __forceinline__ bool inb(long long i, long long n) {
    return (unsigned long long)i < (unsigned long long)(n > 0 ? n : 0);
}

// current element counts of the mesh arrays
struct MeshDims {
    int V, F, H;
};

// Active cell record written by the DMC emit pass (16 bytes):
//   cell  = linear sample index of the cell's corner 0
//   qbase = index of the first quad the cell owns
//   info  = case (8 bits) | edge -> contour map (2 bits per edge) << 8
// The index of a cell's first vertex lives in a separate array (a prefix sum
// over the cells' contour counts).
struct __align__(16) ActiveCell {
    uint32_t cell;
    int32_t qbase;
    uint32_t info;
    int32_t pad;
};

// Device counters filled during a run and read back once at its end.
struct DevCounters {
    uint32_t status;
    uint32_t specStatus;  // status bits of work that may be discarded (merged by the host when kept)
    unsigned long long edges, edges3, edges4, nmVertices;
    unsigned long long quadsNM[5];
    unsigned long long nmBuckets;  // length of the 4-face bucket list
    unsigned long long candidates; // coarse cells that may cross iso (refined grids)
    unsigned long long slowFans;   // vertices the single fan walk did not settle
    int gathered[4];               // active cells, DMC vertices, quads (one read-back)
};

}  // namespace mdmc
