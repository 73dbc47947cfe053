// Volume generators of UniformGridHost::generateVolume / generateEdgeCase
// (D/UniformGrid.inl:20-269, :463-509): implicit surfaces sampled on
// [-1, 1]^3 and the two 4x4x3 non-manifold-vertex grids.  Each expression is
// written with the reference's float/double types (its PI is a double
// constant: the trigonometric arguments are products in double rounded to
// float, and cos of a float argument is the float cos).
#include <cuda_runtime.h>

#include "mdmc.h"
#include "mdmc_kernels.h"

namespace mdmc {
namespace {

constexpr double kPi = 3.14159265358979323846;

__device__ __forceinline__ float sq(float x) { return x * x; }
__device__ __forceinline__ float qu(float x) { return x * x * x * x; }

__device__ float torusH(float px, float py, float pz, float cx, float cy, float cz, float p0, float p1) {
    const float c = sq(p0), a = sq(p1);
    const float x = sq(px - cx), y = sq(py - cy), z = sq(pz - cz);
    return sq(x + y + z + c - a) - 4 * c * (x + y);
}
__device__ float torusV(float px, float py, float pz, float cx, float cy, float cz, float p0, float p1) {
    const float c = sq(p0), a = sq(p1);
    const float x = sq(px - cx), y = sq(py - cy), z = sq(pz - cz);
    return sq(x + y + z + c - a) - 4 * c * (x + z);
}

__device__ float surfaceValue(int sc, float px, float py, float pz) {
    switch (sc) {
        case 0:  // sphere (the 0.16 is a double constant)
            return (float)((double)(px * px + py * py + pz * pz) - 0.16);
        case 1:  // torus
            return torusH(px, py, pz, 0.f, 0.f, 0.f, 0.3f, 0.15f);
        case 2: {  // two-holed torus
            const float vt1 = torusH(px, py, pz, -0.38f, 0.f, 0.f, 0.3f, 0.15f);
            const float vt2 = torusH(px, py, pz, 0.2f, 0.38f, 0.f, 0.3f, 0.15f);
            return fminf(vt1, vt2);
        }
        case 3: {  // four-holed torus
            const float t = 0.38f;
            const float v1 = torusH(px, py, pz, -t, 0.f, 0.f, 0.3f, 0.15f);
            const float v2 = torusH(px, py, pz, t, 0.f, 0.f, 0.3f, 0.15f);
            const float v3 = torusV(px, py, pz, 0.f, 0.f, -t, 0.3f, 0.15f);
            const float v4 = torusV(px, py, pz, 0.f, 0.f, t, 0.3f, 0.15f);
            float v = fminf(v1, v2);
            v = fminf(v, v3);
            return fminf(v, v4);
        }
        case 5: {  // iWP, iso 0 (the float arguments select the float cos)
            const float alpha = 5.01f;
            const float x = (float)((double)(alpha * (px + 1)) * kPi), y = (float)((double)(alpha * (py + 1)) * kPi),
                        z = (float)((double)(alpha * (pz + 1)) * kPi);
            return cosf(x) * cosf(y) + cosf(y) * cosf(z) + cosf(z) * cosf(x) - cosf(x) * cosf(y) * cosf(z);
        }
        case 6: {  // pwHybrid, iso 0
            const float alpha = 1.01f;
            const float x = (float)((double)(alpha * (px + 1)) * kPi), y = (float)((double)(alpha * (py + 1)) * kPi),
                        z = (float)((double)(alpha * (pz + 1)) * kPi);
            return 4.0f * (cosf(x) * cosf(y) + cosf(y) * cosf(z) + cosf(z) * cosf(x)) - 3 * cosf(x) * cosf(y) * cosf(z) +
                   0.8f;
        }
        case 7: {  // neovius, iso 0
            const float alpha = 1.f;
            const float x = (float)((double)(alpha * (px + 1)) * kPi), y = (float)((double)(alpha * (py + 1)) * kPi),
                        z = (float)((double)(alpha * (pz + 1)) * kPi);
            return 3 * (cosf(x) + cosf(y) + cosf(z)) + 4 * cosf(x) * cosf(y) * cosf(z);
        }
        case 8: {  // Goursat
            const float a = -1.0f, b = 0.0f, c = 0.5f;
            return qu(px) + qu(py) + qu(pz) + a * (sq(px) + sq(py) + sq(pz)) + b * (sq(px) + sq(py) + sq(pz)) + c;
        }
        case 9: {  // Steiner's Roman surface
            const float alpha = 1.5f;
            const float x = alpha * px, y = alpha * py, z = alpha * pz;
            return sq(x * x + y * y + z * z - 1.0f) - (sq(z - 1) - 2.0f * x * x) * (sq(z + 1) - 2 * y * y);
        }
        default: {  // genus two (case 4 and unknown cases)
            const float alpha = 1.0f;
            float x = (px + 1.0f) / 2.0f, y = (py + 1.0f) / 2.0f, z = (pz + 1.0f) / 2.0f;
            x = alpha * (4.0f * x - 2.0f);
            y = alpha * (4.0f * y - 2.0f);
            z = alpha * (4.0f * z - 2.0f);
            float t = 2 * y * (y * y - 3 * x * x) * (1 - z * z);
            t += (x * x + y * y) * (x * x + y * y);
            t -= (9 * z * z - 1) * (1 - z * z);
            return t;
        }
    }
}

__global__ void kFillVolume(int sc, int X, int Y, int Z, float ox, float oy, float oz, float dx, float dy, float dz,
                            float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)X * Y * Z) return;
    const int x = (int)(i % X), y = (int)((i / X) % Y), z = (int)(i / ((int64_t)X * Y));
    // getCellVertex, D/UniformGrid.h:160-162: origin + vec3(index) * deltas
    out[i] = surfaceValue(sc, ox + (float)x * dx, oy + (float)y * dy, oz + (float)z * dz);
}

// nonManifoldVertex{0,1}Values, D/UniformGrid.inl:191-250: a 4x4x3 grid of
// 850 with 950 at (2,1,0), (1,2,0) and, for the second case, (1,2,1)
__global__ void kFillEdgeCase(int which, float* __restrict__ out) {
    const int i = threadIdx.x;
    if (i >= 48) return;
    const int x = i % 4, y = (i / 4) % 4, z = i / 16;
    const bool hi = (z == 0 && ((y == 1 && x == 2) || (y == 2 && x == 1))) || (which == 1 && z == 1 && y == 2 && x == 1);
    out[i] = hi ? 950.f : 850.f;
}

// generateVolume / generateEdgeCase geometry: [-1, 1]^3,
// deltas = (max - min) / (vec3(dims) - 1)
void unitGeometry(const int32_t dims[3], float origin[3], float spacing[3]) {
    for (int a = 0; a < 3; ++a) {
        origin[a] = -1.f;
        spacing[a] = (1.f - -1.f) / ((float)dims[a] - 1.f);
    }
}

}  // namespace
}  // namespace mdmc

using namespace mdmc;

extern "C" MDMC_API mdmc_status mdmc_generate_volume(int32_t surface_case, const int32_t dims[3], float* samples,
                                                     float origin[3], float spacing[3], void* stream) {
    if (!dims || !samples || dims[0] < 2 || dims[1] < 2 || dims[2] < 2) return MDMC_ERROR_INVALID_ARGUMENT;
    float o[3], d[3];
    unitGeometry(dims, o, d);
    if (origin)
        for (int a = 0; a < 3; ++a) origin[a] = o[a];
    if (spacing)
        for (int a = 0; a < 3; ++a) spacing[a] = d[a];
    const int64_t n = (int64_t)dims[0] * dims[1] * dims[2];
    countLaunch();
    kFillVolume<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        surface_case, dims[0], dims[1], dims[2], o[0], o[1], o[2], d[0], d[1], d[2], samples);
    return cudaGetLastError() == cudaSuccess ? MDMC_OK : MDMC_ERROR_CUDA;
}

extern "C" MDMC_API mdmc_status mdmc_generate_edge_case(int32_t which, float* samples, int32_t dims[3], float origin[3],
                                                        float spacing[3], void* stream) {
    if (!samples || which < 0 || which > 1) return MDMC_ERROR_INVALID_ARGUMENT;
    const int32_t d[3] = {4, 4, 3};
    float o[3], sp[3];
    unitGeometry(d, o, sp);
    for (int a = 0; a < 3; ++a) {
        if (dims) dims[a] = d[a];
        if (origin) origin[a] = o[a];
        if (spacing) spacing[a] = sp[a];
    }
    countLaunch();
    kFillEdgeCase<<<1, 64, 0, (cudaStream_t)stream>>>(which, samples);
    return cudaGetLastError() == cudaSuccess ? MDMC_OK : MDMC_ERROR_CUDA;
}
