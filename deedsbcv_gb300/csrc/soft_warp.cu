// Differentiable field upsampling and image warping for the multi-level soft-min
// form, with hand-written adjoints (float arithmetic; the soft form has no
// bit-exact contract).
//
// Upsampling follows upsampleDeformationsCL (src/transformations.h:245-279): output
// node (i, j, k) of an m x n x o grid reads the source grid (mA x nA x oA) at
// (i / (m/mA), j / (n/nA), k / (o/oA)) with trilinear weights and corners clamped
// to the source.  Warping follows warpAffine with the identity
// (src/dataCostD.h:267-295): voxel p samples the moving image at p + field(p),
// field = the grid upsampled to full resolution, trilinear, corners clamped.
// Fields are stored component-major: u (x) | v (y) | w (z).
#include "common.cuh"
#include "kernels.h"

namespace deeds {

namespace {

struct Axis {
    int i0, i1;  // clamped corners
    float f;     // fraction
};

__device__ __forceinline__ Axis axis_at(float c, int size) {
    const float fl = floorf(c);
    Axis a;
    a.f = c - fl;
    const int i = (int)fl;
    a.i0 = clampi(i, 0, size - 1);
    a.i1 = clampi(i + 1, 0, size - 1);
    return a;
}

__device__ __forceinline__ float tri(const float* __restrict__ v, const Axis& y, const Axis& x, const Axis& z, int m,
                                     int64_t mn) {
    auto at = [&](int yy, int xx, int zz) { return v[yy + (int64_t)xx * m + (int64_t)zz * mn]; };
    const float c00 = at(y.i0, x.i0, z.i0) * (1.0f - y.f) + at(y.i1, x.i0, z.i0) * y.f;
    const float c10 = at(y.i0, x.i1, z.i0) * (1.0f - y.f) + at(y.i1, x.i1, z.i0) * y.f;
    const float c01 = at(y.i0, x.i0, z.i1) * (1.0f - y.f) + at(y.i1, x.i0, z.i1) * y.f;
    const float c11 = at(y.i0, x.i1, z.i1) * (1.0f - y.f) + at(y.i1, x.i1, z.i1) * y.f;
    const float c0 = c00 * (1.0f - x.f) + c10 * x.f;
    const float c1 = c01 * (1.0f - x.f) + c11 * x.f;
    return c0 * (1.0f - z.f) + c1 * z.f;
}

struct Dims {
    int m, n, o;
};

// source coordinate of output index i along an axis: i / (dst / src)
__device__ __forceinline__ float src_coord(int i, int dst, int src) { return (float)i / ((float)dst / (float)src); }

__global__ void k_soft_upsample(const float* __restrict__ in, Dims A, float* __restrict__ out, Dims D) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i >= D.m) return;
    const Axis y = axis_at(src_coord(i, D.m, A.m), A.m), x = axis_at(src_coord(j, D.n, A.n), A.n),
               z = axis_at(src_coord(k, D.o, A.o), A.o);
    const int64_t szA = (int64_t)A.m * A.n * A.o, szD = (int64_t)D.m * D.n * D.o;
    const int64_t p = i + (int64_t)j * D.m + (int64_t)k * D.m * D.n;
    const int64_t mnA = (int64_t)A.m * A.n;
#pragma unroll
    for (int c = 0; c < 3; c++) out[c * szD + p] = tri(in + c * szA, y, x, z, A.m, mnA);
}

// Weight of output index i (of dst) on source node s along an axis (0 if none).
__device__ __forceinline__ float axis_weight(int i, int dst, int src, int s) {
    const Axis a = axis_at(src_coord(i, dst, src), src);
    float w = 0.0f;
    if (a.i0 == s) w += 1.0f - a.f;
    if (a.i1 == s) w += a.f;
    return w;
}

// The output indices that can touch source node s along an axis: [lo, hi].
__device__ __forceinline__ void axis_support(int s, int dst, int src, int& lo, int& hi) {
    const float scale = (float)dst / (float)src;
    lo = max(0, (int)floorf((float)(s - 1) * scale) - 1);
    hi = min(dst - 1, (int)ceilf((float)(s + 1) * scale) + 1);
    if (s == src - 1) hi = dst - 1;  // clamped corners pile onto the last node
}

// Adjoint of k_soft_upsample as a gather: one thread per source node and component.
__global__ void k_soft_upsample_adj(const float* __restrict__ gout, Dims D, float* __restrict__ gin, Dims A) {
    const int64_t szA = (int64_t)A.m * A.n * A.o, szD = (int64_t)D.m * D.n * D.o;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * szA) return;
    const int c = (int)(t / szA);
    const int64_t s = t % szA;
    const int sy = (int)(s % A.m), sx = (int)((s / A.m) % A.n), sz = (int)(s / ((int64_t)A.m * A.n));
    int ylo, yhi, xlo, xhi, zlo, zhi;
    axis_support(sy, D.m, A.m, ylo, yhi);
    axis_support(sx, D.n, A.n, xlo, xhi);
    axis_support(sz, D.o, A.o, zlo, zhi);
    const float* g = gout + c * szD;
    float acc = 0.0f;
    for (int k = zlo; k <= zhi; k++) {
        const float wz = axis_weight(k, D.o, A.o, sz);
        if (wz == 0.0f) continue;
        for (int j = xlo; j <= xhi; j++) {
            const float wx = axis_weight(j, D.n, A.n, sx);
            if (wx == 0.0f) continue;
            float row = 0.0f;
            for (int i = ylo; i <= yhi; i++) {
                const float wy = axis_weight(i, D.m, A.m, sy);
                if (wy != 0.0f) row += wy * g[i + (int64_t)j * D.m + (int64_t)k * D.m * D.n];
            }
            acc += wz * wx * row;
        }
    }
    gin[t] = acc;
}

__global__ void k_soft_warp(const float* __restrict__ mov, const float* __restrict__ grid, Dims A,
                            float* __restrict__ out, Dims D) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i >= D.m) return;
    const int64_t szA = (int64_t)A.m * A.n * A.o, mnA = (int64_t)A.m * A.n, mn = (int64_t)D.m * D.n;
    const Axis gy = axis_at(src_coord(i, D.m, A.m), A.m), gx = axis_at(src_coord(j, D.n, A.n), A.n),
               gz = axis_at(src_coord(k, D.o, A.o), A.o);
    const float u = tri(grid, gy, gx, gz, A.m, mnA), v = tri(grid + szA, gy, gx, gz, A.m, mnA),
                w = tri(grid + 2 * szA, gy, gx, gz, A.m, mnA);
    const Axis y = axis_at((float)i + v, D.m), x = axis_at((float)j + u, D.n), z = axis_at((float)k + w, D.o);
    out[i + (int64_t)j * D.m + (int64_t)k * mn] = tri(mov, y, x, z, D.m, mn);
}

// Adjoint of k_soft_warp: dL/dmoving by scattering the 8 trilinear weights (atomics;
// the corners of neighbouring voxels overlap) and dL/dfield at full resolution
// (the derivative of the trilinear sample w.r.t. its position), which the caller
// pulls back to the grid with k_soft_upsample_adj.
__global__ void k_soft_warp_adj(const float* __restrict__ mov, const float* __restrict__ grid, Dims A,
                                const float* __restrict__ gout, float* __restrict__ gmov, float* __restrict__ gfull,
                                Dims D) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i >= D.m) return;
    const int64_t szA = (int64_t)A.m * A.n * A.o, mnA = (int64_t)A.m * A.n, mn = (int64_t)D.m * D.n,
                  sz = mn * D.o;
    const int64_t p = i + (int64_t)j * D.m + (int64_t)k * mn;
    const Axis gy = axis_at(src_coord(i, D.m, A.m), A.m), gx = axis_at(src_coord(j, D.n, A.n), A.n),
               gz = axis_at(src_coord(k, D.o, A.o), A.o);
    const float u = tri(grid, gy, gx, gz, A.m, mnA), v = tri(grid + szA, gy, gx, gz, A.m, mnA),
                w = tri(grid + 2 * szA, gy, gx, gz, A.m, mnA);
    const Axis y = axis_at((float)i + v, D.m), x = axis_at((float)j + u, D.n), z = axis_at((float)k + w, D.o);
    const float g = gout[p];
    auto at = [&](int yy, int xx, int zz) { return mov[yy + (int64_t)xx * D.m + (int64_t)zz * mn]; };
    const float v000 = at(y.i0, x.i0, z.i0), v100 = at(y.i1, x.i0, z.i0), v010 = at(y.i0, x.i1, z.i0),
                v110 = at(y.i1, x.i1, z.i0), v001 = at(y.i0, x.i0, z.i1), v101 = at(y.i1, x.i0, z.i1),
                v011 = at(y.i0, x.i1, z.i1), v111 = at(y.i1, x.i1, z.i1);
    const float wy0 = 1.0f - y.f, wy1 = y.f, wx0 = 1.0f - x.f, wx1 = x.f, wz0 = 1.0f - z.f, wz1 = z.f;
    if (gmov) {
        auto add = [&](int yy, int xx, int zz, float wgt) {
            atomicAdd(gmov + yy + (int64_t)xx * D.m + (int64_t)zz * mn, g * wgt);
        };
        add(y.i0, x.i0, z.i0, wy0 * wx0 * wz0); add(y.i1, x.i0, z.i0, wy1 * wx0 * wz0);
        add(y.i0, x.i1, z.i0, wy0 * wx1 * wz0); add(y.i1, x.i1, z.i0, wy1 * wx1 * wz0);
        add(y.i0, x.i0, z.i1, wy0 * wx0 * wz1); add(y.i1, x.i0, z.i1, wy1 * wx0 * wz1);
        add(y.i0, x.i1, z.i1, wy0 * wx1 * wz1); add(y.i1, x.i1, z.i1, wy1 * wx1 * wz1);
    }
    if (gfull) {
        // d sample / d position along each axis (the fraction moves with the position)
        const float dy = ((v100 - v000) * wx0 + (v110 - v010) * wx1) * wz0 + ((v101 - v001) * wx0 + (v111 - v011) * wx1) * wz1;
        const float dx = ((v010 - v000) * wy0 + (v110 - v100) * wy1) * wz0 + ((v011 - v001) * wy0 + (v111 - v101) * wy1) * wz1;
        const float dz = ((v001 - v000) * wy0 + (v101 - v100) * wy1) * wx0 + ((v011 - v010) * wy0 + (v111 - v110) * wy1) * wx1;
        gfull[p] = g * dx;           // u
        gfull[sz + p] = g * dy;      // v
        gfull[2 * sz + p] = g * dz;  // w
    }
}

}  // namespace

cudaError_t launch_soft_upsample(const float* in, int mA, int nA, int oA, float* out, int m, int n, int o,
                                 cudaStream_t s) {
    k_soft_upsample<<<dim3((m + 127) / 128, n, o), 128, 0, s>>>(in, Dims{mA, nA, oA}, out, Dims{m, n, o});
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_soft_upsample_adj(const float* gout, int m, int n, int o, float* gin, int mA, int nA, int oA,
                                     cudaStream_t s) {
    const int64_t n3 = 3LL * mA * nA * oA;
    k_soft_upsample_adj<<<(unsigned)((n3 + 127) / 128), 128, 0, s>>>(gout, Dims{m, n, o}, gin, Dims{mA, nA, oA});
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_soft_warp(const float* mov, const float* grid, int mA, int nA, int oA, float* out, int m, int n,
                             int o, cudaStream_t s) {
    k_soft_warp<<<dim3((m + 127) / 128, n, o), 128, 0, s>>>(mov, grid, Dims{mA, nA, oA}, out, Dims{m, n, o});
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_soft_warp_adj(const float* mov, const float* grid, int mA, int nA, int oA, const float* gout,
                                 float* gmov, float* gfull, int m, int n, int o, cudaStream_t s) {
    k_soft_warp_adj<<<dim3((m + 127) / 128, n, o), 128, 0, s>>>(mov, grid, Dims{mA, nA, oA}, gout, gmov, gfull,
                                                                 Dims{m, n, o});
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace deeds
