// Shared device helpers for the deeds sm_103a kernels.
//
// All kernels are compiled with --fmad=false: the reference's float results
// depend on separate IEEE multiply and add roundings (ISO C++ build, no FMA
// contraction), and several stages promote to double exactly where the
// reference's C++ expressions do.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace deeds {

__host__ __device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Trilinear 8-term blend with the reference's evaluation types and order
// (src/transformations.h:15-22, src/dataCostD.h:288-295): terms touching the
// double literal 1.0 are double, dx*dy and dx*dy*dz*v are float, the sum is
// double left to right, rounded to float once.  cYXZ: Y = +1 in y (i), X = +1 in
// x (j), Z = +1 in z (k).
struct Blend8Weights {
    double w000, w100, w010, w001, w110, w101, w011;
    float dxdydz;
};

__device__ __forceinline__ Blend8Weights blend8_weights(float dx, float dy, float dz) {
    Blend8Weights b;
    const double a = 1.0 - (double)dx, bb = 1.0 - (double)dy, c = 1.0 - (double)dz;
    const double ab = a * bb;             // (1-dx)(1-dy)
    const double ady = a * (double)dy;    // (1-dx)dy
    const double dxb = (double)dx * bb;   // dx(1-dy)
    b.w000 = ab * c;
    b.w100 = ady * c;
    b.w010 = dxb * c;
    b.w001 = ab * (double)dz;
    b.w110 = (double)(dx * dy) * c;
    b.w101 = ady * (double)dz;
    b.w011 = dxb * (double)dz;
    b.dxdydz = dx * dy * dz;
    return b;
}

__device__ __forceinline__ float blend8_apply(const Blend8Weights& b, float c000, float c100, float c010,
                                              float c001, float c110, float c101, float c011, float c111) {
    double acc = b.w000 * (double)c000;
    acc = acc + b.w100 * (double)c100;
    acc = acc + b.w010 * (double)c010;
    acc = acc + b.w001 * (double)c001;
    acc = acc + b.w110 * (double)c110;
    acc = acc + b.w101 * (double)c101;
    acc = acc + b.w011 * (double)c011;
    acc = acc + (double)(b.dxdydz * c111);
    return (float)acc;
}

// Corner offsets of a clamp-to-edge trilinear sample at integer corner (y,x,z).
struct Corners {
    int64_t o000, o100, o010, o001, o110, o101, o011, o111;
};

__device__ __forceinline__ Corners corners(int y, int x, int z, int m2, int n2, int o2) {
    const int y0 = clampi(y, 0, m2 - 1), y1 = clampi(y + 1, 0, m2 - 1);
    const int x0 = clampi(x, 0, n2 - 1), x1 = clampi(x + 1, 0, n2 - 1);
    const int z0 = clampi(z, 0, o2 - 1), z1 = clampi(z + 1, 0, o2 - 1);
    const int64_t s1 = m2, s2 = (int64_t)m2 * n2;
    Corners c;
    c.o000 = y0 + x0 * s1 + z0 * s2;
    c.o100 = y1 + x0 * s1 + z0 * s2;
    c.o010 = y0 + x1 * s1 + z0 * s2;
    c.o001 = y0 + x0 * s1 + z1 * s2;
    c.o110 = y1 + x1 * s1 + z0 * s2;
    c.o101 = y1 + x0 * s1 + z1 * s2;
    c.o011 = y0 + x1 * s1 + z1 * s2;
    c.o111 = y1 + x1 * s1 + z1 * s2;
    return c;
}

__device__ __forceinline__ float sample(const float* __restrict__ v, const Corners& c, const Blend8Weights& b) {
    return blend8_apply(b, __ldg(v + c.o000), __ldg(v + c.o100), __ldg(v + c.o010), __ldg(v + c.o001),
                        __ldg(v + c.o110), __ldg(v + c.o101), __ldg(v + c.o011), __ldg(v + c.o111));
}

// Split a float coordinate into floor (as int) and fraction, as `int x=floor(x1);
// float dx=x1-x;` does in the reference.
__device__ __forceinline__ void split_coord(float c, int& i, float& f) {
    i = (int)floorf(c);
    f = c - (float)i;
}

}  // namespace deeds
