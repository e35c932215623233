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

// Exact float -> double widening with integer operations: on GB300 the FP64
// pipe (which also executes F2F conversions) is the bound of the trilinear
// warps, and widening a float is exact.  Normal numbers re-bias the exponent
// and shift the mantissa; zeros keep their sign; subnormals, infinities and NaNs
// (not expected in images or displacement fields) take the hardware conversion.
__device__ __forceinline__ double f2d(float f) {
    const uint32_t b = __float_as_uint(f);
    const uint32_t e = (b >> 23) & 0xffu;
    if (e == 0xffu || (e == 0u && (b & 0x7fffffu) != 0u)) return (double)f;
    const uint64_t sign = (uint64_t)(b & 0x80000000u) << 32;
    const uint64_t mag = e == 0u ? 0ull : ((uint64_t)(e + 896u) << 52) | ((uint64_t)(b & 0x7fffffu) << 29);
    return __longlong_as_double((long long)(sign | mag));
}

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
    const double ddx = f2d(dx), ddy = f2d(dy), ddz = f2d(dz);
    const double a = 1.0 - ddx, bb = 1.0 - ddy, c = 1.0 - ddz;
    const double ab = a * bb;     // (1-dx)(1-dy)
    const double ady = a * ddy;   // (1-dx)dy
    const double dxb = ddx * bb;  // dx(1-dy)
    b.w000 = ab * c;
    b.w100 = ady * c;
    b.w010 = dxb * c;
    b.w001 = ab * ddz;
    b.w110 = f2d(dx * dy) * c;
    b.w101 = ady * ddz;
    b.w011 = dxb * ddz;
    b.dxdydz = dx * dy * dz;
    return b;
}

__device__ __forceinline__ float blend8_apply(const Blend8Weights& b, float c000, float c100, float c010,
                                              float c001, float c110, float c101, float c011, float c111) {
    double acc = b.w000 * f2d(c000);
    acc = acc + b.w100 * f2d(c100);
    acc = acc + b.w010 * f2d(c010);
    acc = acc + b.w001 * f2d(c001);
    acc = acc + b.w110 * f2d(c110);
    acc = acc + b.w101 * f2d(c101);
    acc = acc + b.w011 * f2d(c011);
    acc = acc + f2d(b.dxdydz * c111);
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
