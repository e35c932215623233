// Field and image transforms on sm_103a (replaces upsampleDeformationsCL,
// interp3, warpAffine, warpImageCL, warpAffineS, consistentMappingCL and jacobian;
// src/transformations.h:5-279, src/dataCostD.h:213-315).
//
// The full-resolution field is never materialised on the hot path: a warp kernel
// evaluates upsampleDeformationsCL's trilinear grid interpolation for its own
// voxel (identical arithmetic) and immediately warps the image.  Interpolation
// weights are evaluated in FP64 exactly where the reference's C++ promotes to
// double (see common.cuh).  The blends run in float-float first and take the
// double evaluation only where the float-float value cannot prove the
// reference's rounding (ff_blend8): GB300's FP64 rate would otherwise bound
// these kernels (~80 DP operations per voxel for field + image).  Roofline: per
// voxel 4 B image gather (L2) + 4 B write; the grid field is L2-resident.
#include "common.cuh"
#include "kernels.h"

namespace deeds {

namespace {

struct Grid3 {
    const float* u;
    const float* v;
    const float* w;
    int m, n, o;
    float sm, sn, so;  // (float)full / (float)grid per axis
};

// upsampleDeformationsCL at voxel (i,j,k) of the full-resolution grid
// (src/transformations.h:248-267): coordinate index/scale, floor, trilinear.
__device__ __forceinline__ void upsample_at(const Grid3& g, int i, int j, int k, float& u, float& v, float& w) {
    int x, y, z;
    float dx, dy, dz;
    split_coord(__fdiv_rn((float)j, g.sn), x, dx);
    split_coord(__fdiv_rn((float)i, g.sm), y, dy);
    split_coord(__fdiv_rn((float)k, g.so), z, dz);
    const Corners c = corners(y, x, z, g.m, g.n, g.o);
    const FFWeights b = ff_weights(dx, dy, dz);
    u = sample_ff(g.u, c, b, dx, dy, dz);
    v = sample_ff(g.v, c, b, dx, dy, dz);
    w = sample_ff(g.w, c, b, dx, dy, dz);
}

struct Affine12 {
    float x[12];
};

__global__ void k_shift(const float* __restrict__ in, float* __restrict__ out, int64_t n, float neg_shift) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) out[p] = __fsub_rn(in[p], neg_shift);
}

__global__ void k_upsample(Grid3 g, float* __restrict__ u, float* __restrict__ v, float* __restrict__ w, int m, int n,
                           int o) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i >= m) return;
    const int64_t p = i + (int64_t)j * m + (int64_t)k * m * n;
    float a, b, c;
    upsample_at(g, i, j, k, a, b, c);
    u[p] = a; v[p] = b; w[p] = c;
}

// warpAffine (src/dataCostD.h:278-295) with the field taken either from a grid
// (upsampled on the fly), from full-resolution arrays, or zero.
// mode 0: zero field, 1: full-res arrays fu/fv/fw, 2: grid g.
__global__ void k_warp_affine(const float* __restrict__ in, Affine12 X, int mode, Grid3 g,
                              const float* __restrict__ fu, const float* __restrict__ fv,
                              const float* __restrict__ fw, float* __restrict__ out, int m, int n, int o,
                              float* __restrict__ keep_u, float* __restrict__ keep_v, float* __restrict__ keep_w) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i >= m) return;
    const int64_t p = i + (int64_t)j * m + (int64_t)k * m * n;
    float u = 0.0f, v = 0.0f, w = 0.0f;
    if (mode == 1) { u = fu[p]; v = fv[p]; w = fw[p]; }
    else if (mode == 2) upsample_at(g, i, j, k, u, v, w);
    if (keep_u) { keep_u[p] = u; keep_v[p] = v; keep_w[p] = w; }
    const float fi = (float)i, fj = (float)j, fk = (float)k;
    const float y1 = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(fi, X.x[0]), __fmul_rn(fj, X.x[1])), __fmul_rn(fk, X.x[2])), X.x[3]), v);
    const float x1 = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(fi, X.x[4]), __fmul_rn(fj, X.x[5])), __fmul_rn(fk, X.x[6])), X.x[7]), u);
    const float z1 = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(fi, X.x[8]), __fmul_rn(fj, X.x[9])), __fmul_rn(fk, X.x[10])), X.x[11]), w);
    int x, y, z;
    float dx, dy, dz;
    split_coord(x1, x, dx);
    split_coord(y1, y, dy);
    split_coord(z1, z, dz);
    out[p] = sample_ff(in, corners(y, x, z, m, n, o), ff_weights(dx, dy, dz), dx, dy, dz);
}

// warpImageCL = interp3(flag=true) (src/dataCostD.h:213-223, src/transformations.h:9-22)
// with the field upsampled on the fly from a grid (mode 2) or read at full
// resolution (mode 1).
__global__ void k_warp_image(const float* __restrict__ in, int mode, Grid3 g, const float* __restrict__ fu,
                             const float* __restrict__ fv, const float* __restrict__ fw, float* __restrict__ out,
                             int m, int n, int o) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i >= m) return;
    const int64_t p = i + (int64_t)j * m + (int64_t)k * m * n;
    float u, v, w;
    if (mode == 1) { u = fu[p]; v = fv[p]; w = fw[p]; }
    else upsample_at(g, i, j, k, u, v, w);
    int x, y, z;
    float dx, dy, dz;
    split_coord(u, x, dx);
    split_coord(v, y, dy);
    split_coord(w, z, dz);
    out[p] = sample_ff(in, corners(y + i, x + j, z + k, m, n, o), ff_weights(dx, dy, dz), dx, dy, dz);
}

// warpAffineS (src/dataCostD.h:241-266): nearest neighbour, round half away from zero.
__global__ void k_warp_seg(const short* __restrict__ in, Affine12 X, int mode, Grid3 g,
                           const float* __restrict__ fu, const float* __restrict__ fv, const float* __restrict__ fw,
                           short* __restrict__ out, int m, int n, int o) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i >= m) return;
    const int64_t p = i + (int64_t)j * m + (int64_t)k * m * n;
    float u = 0.0f, v = 0.0f, w = 0.0f;
    if (mode == 1) { u = fu[p]; v = fv[p]; w = fw[p]; }
    else if (mode == 2) upsample_at(g, i, j, k, u, v, w);
    const float fi = (float)i, fj = (float)j, fk = (float)k;
    const float y1 = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(fi, X.x[0]), __fmul_rn(fj, X.x[1])), __fmul_rn(fk, X.x[2])), X.x[3]), v);
    const float x1 = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(fi, X.x[4]), __fmul_rn(fj, X.x[5])), __fmul_rn(fk, X.x[6])), X.x[7]), u);
    const float z1 = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(fi, X.x[8]), __fmul_rn(fj, X.x[9])), __fmul_rn(fk, X.x[10])), X.x[11]), w);
    const int x = (int)roundf(x1), y = (int)roundf(y1), z = (int)roundf(z1);
    out[p] = in[clampi(y, 0, m - 1) + (int64_t)clampi(x, 0, n - 1) * m + (int64_t)clampi(z, 0, o - 1) * (int64_t)m * n];
}

__global__ void k_scale6(const float* __restrict__ a0, const float* __restrict__ a1, const float* __restrict__ a2,
                         const float* __restrict__ a3, const float* __restrict__ a4, const float* __restrict__ a5,
                         float* __restrict__ b0, float* __restrict__ b1, float* __restrict__ b2, float* __restrict__ b3,
                         float* __restrict__ b4, float* __restrict__ b5, int64_t n, float f) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    b0[p] = __fmul_rn(a0[p], f); b1[p] = __fmul_rn(a1[p], f); b2[p] = __fmul_rn(a2[p], f);
    b3[p] = __fmul_rn(a3[p], f); b4[p] = __fmul_rn(a4[p], f); b5[p] = __fmul_rn(a5[p], f);
}

// One consistentMappingCL iteration (src/transformations.h:203-226): both new
// fields from the previous ones, u <- 0.5*us - 0.5*(us2 at x+us), and back.
__global__ void k_consistent_step(const float* __restrict__ us, const float* __restrict__ vs,
                                  const float* __restrict__ ws, const float* __restrict__ us2,
                                  const float* __restrict__ vs2, const float* __restrict__ ws2, float* __restrict__ nu,
                                  float* __restrict__ nv, float* __restrict__ nw, float* __restrict__ nu2,
                                  float* __restrict__ nv2, float* __restrict__ nw2, int m, int n, int o) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i >= m) return;
    const int64_t p = i + (int64_t)j * m + (int64_t)k * m * n;
    {
        int x, y, z;
        float dx, dy, dz;
        split_coord(us[p], x, dx);
        split_coord(vs[p], y, dy);
        split_coord(ws[p], z, dz);
        const Corners c = corners(y + i, x + j, z + k, m, n, o);
        const Blend8Weights b = blend8_weights(dx, dy, dz);
        nu[p] = (float)(0.5 * (double)us[p] - 0.5 * (double)sample(us2, c, b));
        nv[p] = (float)(0.5 * (double)vs[p] - 0.5 * (double)sample(vs2, c, b));
        nw[p] = (float)(0.5 * (double)ws[p] - 0.5 * (double)sample(ws2, c, b));
    }
    {
        int x, y, z;
        float dx, dy, dz;
        split_coord(us2[p], x, dx);
        split_coord(vs2[p], y, dy);
        split_coord(ws2[p], z, dz);
        const Corners c = corners(y + i, x + j, z + k, m, n, o);
        const Blend8Weights b = blend8_weights(dx, dy, dz);
        nu2[p] = (float)(0.5 * (double)us2[p] - 0.5 * (double)sample(us, c, b));
        nv2[p] = (float)(0.5 * (double)vs2[p] - 0.5 * (double)sample(vs, c, b));
        nw2[p] = (float)(0.5 * (double)ws2[p] - 0.5 * (double)sample(ws, c, b));
    }
}

// Jacobian determinant per node (src/transformations.h:118-158): central
// differences with replicate padding, /g, +1 on the diagonal; accumulates
// sum J, sum J^2 and count(J<0) for the diagnostic print.
__global__ void k_jacobian(const float* __restrict__ u, const float* __restrict__ v, const float* __restrict__ w,
                           int m, int n, int o, float f1, double* __restrict__ acc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    double sj = 0.0, sj2 = 0.0, neg = 0.0;
    if (i < m) {
        const int64_t mn = (int64_t)m * n;
        auto at = [&](const float* a, int ii, int jj, int kk) {
            return a[clampi(ii, 0, m - 1) + (int64_t)clampi(jj, 0, n - 1) * m + (int64_t)clampi(kk, 0, o - 1) * mn];
        };
        auto d = [&](const float* a, int axis) {
            float r = 0.0f;
            const float gr[3] = {-0.5f, 0.0f, 0.5f};
            for (int f = 0; f < 3; f++) {
                const float s = axis == 1 ? at(a, i + f - 1, j, k) : (axis == 2 ? at(a, i, j + f - 1, k) : at(a, i, j, k + f - 1));
                r = __fadd_rn(r, __fmul_rn(gr[f], s));
            }
            return r;
        };
        const float a11 = (float)((double)__fmul_rn(d(u, 2), f1) + 1.0), a12 = __fmul_rn(d(u, 1), f1), a13 = __fmul_rn(d(u, 3), f1);
        const float a21 = __fmul_rn(d(v, 2), f1), a22 = (float)((double)__fmul_rn(d(v, 1), f1) + 1.0), a23 = __fmul_rn(d(v, 3), f1);
        const float a31 = __fmul_rn(d(w, 2), f1), a32 = __fmul_rn(d(w, 1), f1), a33 = (float)((double)__fmul_rn(d(w, 3), f1) + 1.0);
        const float J = a11 * (a22 * a33 - a23 * a32) - a21 * (a12 * a33 - a13 * a32) + a31 * (a12 * a23 - a13 * a22);
        sj = J; sj2 = (double)J * J; neg = J < 0.0f ? 1.0 : 0.0;
    }
    for (int off = 16; off > 0; off >>= 1) {
        sj += __shfl_xor_sync(0xffffffffu, sj, off);
        sj2 += __shfl_xor_sync(0xffffffffu, sj2, off);
        neg += __shfl_xor_sync(0xffffffffu, neg, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(acc + 0, sj);
        atomicAdd(acc + 1, sj2);
        atomicAdd(acc + 2, neg);
    }
}

inline dim3 vol_grid(int m, int n, int o, int threads) { return dim3((m + threads - 1) / threads, n, o); }

inline Grid3 make_grid(const float* u, const float* v, const float* w, int m2, int n2, int o2, int m, int n, int o) {
    Grid3 g;
    g.u = u; g.v = v; g.w = w;
    g.m = m2; g.n = n2; g.o = o2;
    g.sm = (float)m / (float)m2; g.sn = (float)n / (float)n2; g.so = (float)o / (float)o2;
    return g;
}

inline Affine12 make_affine(const float* X) {
    Affine12 a;
    for (int i = 0; i < 12; i++) a.x[i] = X[i];
    return a;
}

}  // namespace

cudaError_t launch_shift(const float* d_in, float* d_out, int64_t n, float shift, cudaStream_t s) {
    k_shift<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d_in, d_out, n, -shift);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_upsample(const float* u0, const float* v0, const float* w0, int m2, int n2, int o2, float* u,
                            float* v, float* w, int m, int n, int o, cudaStream_t s) {
    k_upsample<<<vol_grid(m, n, o, 128), 128, 0, s>>>(make_grid(u0, v0, w0, m2, n2, o2, m, n, o), u, v, w, m, n, o);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_warp_affine(const float* d_in, const float* X, const FieldRef& f, int m, int n, int o, float* d_out,
                               float* keep_u, float* keep_v, float* keep_w, cudaStream_t s) {
    const Grid3 g = f.mode == 2 ? make_grid(f.u, f.v, f.w, f.m1, f.n1, f.o1, m, n, o) : Grid3{};
    k_warp_affine<<<vol_grid(m, n, o, 128), 128, 0, s>>>(d_in, make_affine(X), f.mode, g, f.u, f.v, f.w, d_out, m, n,
                                                          o, keep_u, keep_v, keep_w);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_warp_image(const float* d_in, const FieldRef& f, int m, int n, int o, float* d_out, cudaStream_t s) {
    const Grid3 g = f.mode == 2 ? make_grid(f.u, f.v, f.w, f.m1, f.n1, f.o1, m, n, o) : Grid3{};
    k_warp_image<<<vol_grid(m, n, o, 128), 128, 0, s>>>(d_in, f.mode, g, f.u, f.v, f.w, d_out, m, n, o);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_warp_seg(const short* d_in, const float* X, const FieldRef& f, int m, int n, int o, short* d_out,
                            cudaStream_t s) {
    const Grid3 g = f.mode == 2 ? make_grid(f.u, f.v, f.w, f.m1, f.n1, f.o1, m, n, o) : Grid3{};
    k_warp_seg<<<vol_grid(m, n, o, 128), 128, 0, s>>>(d_in, make_affine(X), f.mode, g, f.u, f.v, f.w, d_out, m, n, o);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_consistent(float* u, float* v, float* w, float* u2, float* v2, float* w2, int m, int n, int o, int g,
                              float* scratch /* 12*sz */, cudaStream_t s) {
    const int64_t sz = (int64_t)m * n * o;
    float* A[6];
    float* B[6];
    for (int i = 0; i < 6; i++) { A[i] = scratch + i * sz; B[i] = scratch + (6 + i) * sz; }
    const float f1 = (float)(1.0 / (float)g);
    const unsigned nb = (unsigned)((sz + 255) / 256);
    k_scale6<<<nb, 256, 0, s>>>(u, v, w, u2, v2, w2, A[0], A[1], A[2], A[3], A[4], A[5], sz, f1);
    for (int it = 0; it < 10; it++) {
        k_consistent_step<<<vol_grid(m, n, o, 64), 64, 0, s>>>(A[0], A[1], A[2], A[3], A[4], A[5], B[0], B[1], B[2],
                                                               B[3], B[4], B[5], m, n, o);
        for (int i = 0; i < 6; i++) { float* t = A[i]; A[i] = B[i]; B[i] = t; }
    }
    k_scale6<<<nb, 256, 0, s>>>(A[0], A[1], A[2], A[3], A[4], A[5], u, v, w, u2, v2, w2, sz, (float)g);
    count_launches(12);
    return cudaGetLastError();
}

cudaError_t launch_jacobian(const float* u, const float* v, const float* w, int m, int n, int o, int g, double* d_acc,
                            cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(d_acc, 0, 3 * sizeof(double), s);
    if (e != cudaSuccess) return e;
    const float f1 = (float)(1.0 / (float)g);
    k_jacobian<<<vol_grid(m, n, o, 64), 64, 0, s>>>(u, v, w, m, n, o, f1, d_acc);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace deeds
