// Adjoint of the DMC vertex positions with respect to the grid samples, the
// topology of the last forward run held fixed.  No counterpart in the
// reference, which is not differentiable.
//
// With the surface iteration off, a DMC vertex is
//   p = origin + (cell + q) * spacing,  q = (1/n) sum over its contour's n
// edges of the edge point, whose coordinate on the edge's axis is
//   w = (iso - s0) / (s1 - s0)
// (computeLocalCoordinateOffset, D/CellIntersection.inl:176-200), so
//   dw/ds0 = (iso - s1) / (s1 - s0)^2,  dw/ds1 = -(iso - s0) / (s1 - s0)^2.
// Vertices the splitter appended pass their gradient to the DMC vertex they
// descend from.  On refined or padded grids the sample gradients continue
// through refineGrid's trilinear weights (D/UniformGrid.inl:279-319) onto the
// coarse input samples.  Sums use float atomics (order-dependent rounding).
#include <cuda_runtime.h>

#include "mc_contour_table.h"
#include "mdmc_device.cuh"
#include "mdmc_kernels.h"

namespace mdmc {

__global__ void kGatherParents(const float* __restrict__ dlDpos, int numVertices, int dmcVertices,
                               const int* __restrict__ appParent, float* __restrict__ vertexGrad) {
    const int o = dmcVertices + blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= numVertices) return;
    const int p = appParent[o - dmcVertices];
    if (!inb(p, dmcVertices)) return;
    for (int a = 0; a < 3; ++a) atomicAdd(&vertexGrad[3 * (int64_t)p + a], dlDpos[3 * (int64_t)o + a]);
}

void launchGatherParents(const float* dlDpos, int numVertices, int dmcVertices, const int* appParent, float* vertexGrad,
                         cudaStream_t s) {
    const int n = numVertices - dmcVertices;
    if (n <= 0) return;
    countLaunch();
    kGatherParents<<<(n + 255) / 256, 256, 0, s>>>(dlDpos, numVertices, dmcVertices, appParent, vertexGrad);
}

// gradient v of processed-grid sample (x, y, z) onto the input samples
__device__ __forceinline__ void scatterSample(const PlainView& g, float* out, int x, int y, int z, float v) {
    atomicAdd(out + ((size_t)z * g.Y + y) * g.X + x, v);
}
__device__ __forceinline__ void scatterSample(const RefinedView& g, float* out, int x, int y, int z, float v) {
    x = g.unpad(x, g.X);
    y = g.unpad(y, g.Y);
    z = g.unpad(z, g.Z);
    const float qx = g.divf(x), qy = g.divf(y), qz = g.divf(z);
    const int mx = (int)floorf(qx), my = (int)floorf(qy), mz = (int)floorf(qz);
    const float dx = qx - (float)mx, dy = qy - (float)my, dz = qz - (float)mz;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int cx = min(max(mx + (k & 1), 0), g.cX - 1);
        const int cy = min(max(my + ((k >> 1) & 1), 0), g.cY - 1);
        const int cz = min(max(mz + ((k >> 2) & 1), 0), g.cZ - 1);
        const float w = ((k & 1) ? dx : 1.f - dx) * (((k >> 1) & 1) ? dy : 1.f - dy) * (((k >> 2) & 1) ? dz : 1.f - dz);
        if (w != 0.f) atomicAdd(out + ((size_t)cz * g.cY + cy) * g.cX + cx, w * v);
    }
}

// one thread per active cell: the cell's contours as in the forward, each
// contour's vertex gradient spread over its edges' two samples
template <class View>
__global__ void __launch_bounds__(128) kBackwardCells(View g, float iso, const ActiveCell* __restrict__ act,
                                                      int numActive, const float* __restrict__ vertexGrad,
                                                      int dmcVertices, float* __restrict__ out, uint32_t* status) {
    __shared__ uint64_t table[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) table[i] = kContourTable[i];
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= numActive) return;
    const ActiveCell rec = act[i];
    const uint32_t line = rec.cell / (uint32_t)g.X;
    const int x = (int)(rec.cell - line * (uint32_t)g.X), y = (int)(line % (uint32_t)g.Y), z = (int)(line / (uint32_t)g.Y);
    const int cs = (int)(rec.info & 255u);
    float s[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) s[k] = g.at(x + (k & 1), y + ((k >> 1) & 1), z + ((k >> 2) & 1));
    const uint64_t c = cellContours(cs, s, iso, table);
    const int n = numContours(c);
    if (rec.pad < 0 || rec.pad + n > dmcVertices) {
        atomicOr(status, kStatusCountMismatch);
        return;
    }
    const F3 dl = g.deltas();
    const float sp[3] = {dl.x, dl.y, dl.z};
    int before = 0;
    for (int t = 0; t < n; ++t) {
        const int csz = nib(c, t);
        const int64_t v = rec.pad + t;
        const float gv[3] = {vertexGrad[3 * (int64_t)v], vertexGrad[3 * (int64_t)v + 1], vertexGrad[3 * (int64_t)v + 2]};
        for (int k = 0; k < csz; ++k) {
            const int e = (int)((c >> (16 + 4 * (before + k))) & 0xF);
            const int a0 = edgeV0(e), a1 = edgeV1(e), ax = edgeAxis(e);
            const float d = s[a1] - s[a0];
            const float coef = gv[ax] * sp[ax] / (float)csz;
            const float g0 = coef * ((iso - s[a1]) / (d * d));
            const float g1 = -coef * ((iso - s[a0]) / (d * d));
            scatterSample(g, out, x + (a0 & 1), y + ((a0 >> 1) & 1), z + ((a0 >> 2) & 1), g0);
            scatterSample(g, out, x + (a1 & 1), y + ((a1 >> 1) & 1), z + ((a1 >> 2) & 1), g1);
        }
        before += csz;
    }
}

void launchBackwardCells(const GridDesc& g, float iso, const ActiveCell* act, int numActive, const float* vertexGrad,
                         int dmcVertices, float* dlDsamples, uint32_t* status, cudaStream_t s) {
    if (numActive <= 0) return;
    countLaunch();
    const unsigned blocks = (unsigned)((numActive + 127) / 128);
    if (g.refined)
        kBackwardCells<RefinedView><<<blocks, 128, 0, s>>>(g.ref, iso, act, numActive, vertexGrad, dmcVertices,
                                                           dlDsamples, status);
    else
        kBackwardCells<PlainView><<<blocks, 128, 0, s>>>(g.plain, iso, act, numActive, vertexGrad, dmcVertices,
                                                         dlDsamples, status);
}

}  // namespace mdmc
