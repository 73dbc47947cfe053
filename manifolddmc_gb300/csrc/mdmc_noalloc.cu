// mdmc_count_cells_noalloc: the DMC count pass (active cells and quads of a
// grid at an iso-value) for callers that cannot allocate device memory.
//
// Who needs it: code that sizes its output buffers before a run from inside a
// frame or stream loop whose device memory is fixed up front (a renderer's or
// simulator's pre-allocated pool, a process under a hard memory cap), or that
// must not stall the device: cudaMalloc and cudaFree synchronize the whole
// device, and mdmc_run grows its context buffers with them.  This entry point
// needs no context, allocates nothing and does not synchronize; its per-row
// count kernel classifies cells exactly as mdmc_run's mask pass does.
//
// Scratch: two file-scope device arrays, shared by every call in the process
// on a device and keeping the last call's contents:
//   g_rowScratch     one int4 per x-row of cells, kMaxRows rows (4 MiB);
//   g_mayCrossScratch one bit per coarse cell of a refined grid,
//                    kMaxCoarseCells cells (2 MiB), plus one spare word: the
//                    refined row walker loads the word after a row's first
//                    word too (its bits are masked off), as mdmc_run's own
//                    bit mask allows for.
// Every call rewrites all the words it reads (the count kernel writes each
// row's record, the coarse pre-pass each word of its bit mask, the reduction
// writes the caller's totals outright), so nothing has to start at zero.
// Calls that overlap on the GPU (two streams, or two host threads) race on
// this scratch: serialize them.
//
// Device set-up: the first call on a device, with that device current, looks
// up the arrays' addresses (cudaGetSymbolAddress), which also makes the CUDA
// runtime load this file's module (and with it the arrays) on that device.
// Make that first call before any stream capture begins.  The addresses are
// kept per device together with the id of the context they belong to; when
// the caller has reset the device (cudaDeviceReset) the next call finds a new
// context and looks them up again, which is then again a set-up call.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "mdmc.h"
#include "mdmc_kernels.h"

namespace mdmc {
namespace {

constexpr int64_t kMaxRows = int64_t(1) << 18;          // (dims[1]-1)*(dims[2]-1)
constexpr int64_t kMaxCoarseCells = int64_t(1) << 24;   // refined grids: coarse cells
constexpr int64_t kMaxMayCrossWords = kMaxCoarseCells / 32;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) int4 g_rowScratch[kMaxRows];
static __device__ __align__(256) uint32_t g_mayCrossScratch[kMaxMayCrossWords + 1];

struct DeviceScratch {
    bool ready = false;
    unsigned long long context = 0;  // cuCtxGetId of the context the addresses belong to
    int4* rows = nullptr;
    uint32_t* mayCross = nullptr;
};

// the driver's context id calls, reached through the runtime (no link to libcuda)
typedef int (*CtxGetCurrentFn)(void** ctx);
typedef int (*CtxGetIdFn)(void* ctx, unsigned long long* id);

std::mutex g_setupLock;
DeviceScratch g_scratch[kMaxDevices];

void setMessage(char* message, int len, const char* text) {
    if (message && len > 0) std::snprintf(message, (size_t)len, "%s", text);
}

// id of the current context, 0 when there is none yet (or the driver lacks the calls)
unsigned long long currentContextId() {
    static CtxGetCurrentFn getCurrent = nullptr;
    static CtxGetIdFn getId = nullptr;
    static bool looked = false;
    if (!looked) {
        looked = true;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            getCurrent = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            getId = reinterpret_cast<CtxGetIdFn>(f);
        (void)cudaGetLastError();
    }
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (!getCurrent || !getId || getCurrent(&ctx) != 0 || !ctx || getId(ctx, &id) != 0) return 0;
    return id;
}

// once per device and context, with that device current
cudaError_t scratchFor(int device, DeviceScratch& out) {
    std::lock_guard<std::mutex> lock(g_setupLock);
    DeviceScratch& d = g_scratch[device];
    const unsigned long long ctx = currentContextId();
    if (!d.ready || ctx == 0 || ctx != d.context) {
        void* rows = nullptr;
        void* may = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&rows, g_rowScratch);
        if (e != cudaSuccess) return e;
        e = cudaGetSymbolAddress(&may, g_mayCrossScratch);
        if (e != cudaSuccess) return e;
        d.rows = static_cast<int4*>(rows);
        d.mayCross = static_cast<uint32_t*>(may);
        d.context = currentContextId();  // the lookup has made the context current
        d.ready = true;
    }
    out = d;
    return cudaSuccess;
}

// sum of the per-row {active cells, quads} records into totals[0..1]
__global__ void __launch_bounds__(1024) kSumRows(const int4* __restrict__ rows, int numRows, int64_t* __restrict__ totals) {
    __shared__ long long part[2][32];
    long long a = 0, q = 0;
    for (int i = threadIdx.x; i < numRows; i += blockDim.x) {
        const int4 r = rows[i];
        a += r.x;
        q += r.y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        q += __shfl_down_sync(0xffffffffu, q, o);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        part[0][warp] = a;
        part[1][warp] = q;
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = (int)(blockDim.x >> 5);
        a = lane < nw ? part[0][lane] : 0;
        q = lane < nw ? part[1][lane] : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            q += __shfl_down_sync(0xffffffffu, q, o);
        }
        if (lane == 0) {
            totals[0] = a;
            totals[1] = q;
        }
    }
}

__global__ void kZeroTotals(int64_t* totals) {
    if (threadIdx.x < 2) totals[threadIdx.x] = 0;
}

}  // namespace
}  // namespace mdmc

using namespace mdmc;

extern "C" MDMC_API mdmc_status mdmc_count_cells_noalloc(const mdmc_grid* grid, float iso_value, int64_t* totals,
                                                          void* stream, char* message, int message_len) {
    setMessage(message, message_len, "");
    if (!grid || !totals) {
        setMessage(message, message_len, "null argument");
        return MDMC_ERROR_INVALID_ARGUMENT;
    }
    const int X = grid->dims[0], Y = grid->dims[1], Z = grid->dims[2];
    if (X < 1 || Y < 1 || Z < 1) {
        setMessage(message, message_len, "invalid grid dims");
        return MDMC_ERROR_INVALID_ARGUMENT;
    }
    if ((uint64_t)X * Y * Z >= 0xFFFFFFFFull) {
        setMessage(message, message_len, "grid has 2^32 samples or more");
        return MDMC_ERROR_INVALID_ARGUMENT;
    }
    const int64_t numRows = (X > 1 && Y > 1 && Z > 1) ? (int64_t)(Y - 1) * (Z - 1) : 0;
    if (numRows > kMaxRows) {
        char text[160];
        std::snprintf(text, sizeof text, "grid has %lld x-rows of cells, more than the %lld this entry point's scratch holds",
                      (long long)numRows, (long long)kMaxRows);
        setMessage(message, message_len, text);
        return MDMC_ERROR_LIMIT;
    }

    // the grid's view, as mdmc_run builds it
    GridDesc d;
    GridGeom geom;
    geom.X = X;
    geom.Y = Y;
    geom.Z = Z;
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
    int64_t coarseCells = 0;
    if (!d.refined) {
        if (!grid->samples) {
            setMessage(message, message_len, "grid has no samples");
            return MDMC_ERROR_INVALID_ARGUMENT;
        }
    } else {
        for (int a = 0; a < 3; ++a) {
            const int cd = grid->coarse_dims[a];
            if (cd < 1 || grid->refinement < 0 ||
                (int64_t)cd + (int64_t)(cd - 1) * grid->refinement + 2 * d.ref.pad != grid->dims[a]) {
                setMessage(message, message_len, "coarse dims do not match the refined dims");
                return MDMC_ERROR_INVALID_ARGUMENT;
            }
        }
        if (d.ref.cX >= 2 && d.ref.cY >= 2 && d.ref.cZ >= 2)
            coarseCells = (int64_t)(d.ref.cX - 1) * (d.ref.cY - 1) * (d.ref.cZ - 1);
        if (coarseCells > kMaxCoarseCells) {
            char text[160];
            std::snprintf(text, sizeof text,
                          "refined grid has %lld coarse cells, more than the %lld this entry point's scratch holds",
                          (long long)coarseCells, (long long)kMaxCoarseCells);
            setMessage(message, message_len, text);
            return MDMC_ERROR_LIMIT;
        }
    }

    int device = -1;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices) {
        (void)cudaGetLastError();
        setMessage(message, message_len, "no usable current CUDA device");
        return MDMC_ERROR_NO_DEVICE;
    }
    DeviceScratch sc;
    cudaError_t e = scratchFor(device, sc);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        setMessage(message, message_len, cudaGetErrorString(e));
        return MDMC_ERROR_CUDA;
    }

    cudaStream_t s = (cudaStream_t)stream;
    if (coarseCells > 0) {
        d.ref.mayCross = sc.mayCross;
        launchCoarseMayCross(d.ref, iso_value, sc.mayCross, s);
    }
    if (numRows > 0) {
        launchRowCount(d, iso_value, sc.rows, (int)numRows, s);
        countLaunch();
        kSumRows<<<1, 1024, 0, s>>>(sc.rows, (int)numRows, totals);
    } else {
        countLaunch();
        kZeroTotals<<<1, 32, 0, s>>>(totals);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        setMessage(message, message_len, cudaGetErrorString(e));
        return MDMC_ERROR_CUDA;
    }
    return MDMC_OK;
}
