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

// ---- The same blend in float-float, with a proof that it rounds the same way
//
// GB300 runs FP64 at a small fraction of its FP32 rate, and the blends above are
// most of the warps' work.  blend8_apply evaluates a fixed expression: exact
// weight factors 1-d (double), exact products of two of them, one rounded
// product per weight, eight rounded products with the corner values, seven
// rounded sums, one float term (dx*dy*dz*c111) and a final rounding to float.
// With S = sum of |corner values| (weights are at most 1), its double result
// differs from the exact value of the expression by at most ~2^-49.8 S (each of
// the ~16 double roundings adds at most 2^-53 of an intermediate bounded by S).
// The float-float evaluation below (Dekker/Knuth error-free sum and product
// transformations, the product error through fmaf; every non-exact step has a
// relative error of at most ~2^-45) differs from it by at most ~2^-42.6 S.  So
// the two differ by less than eps = 2^-40 S.  If the float-float value lies
// farther than eps from every midpoint between adjacent floats, both round to
// the same float, and that float is returned; otherwise (a value near a
// midpoint, non-finite or very small or large inputs) ff_blend8 reports failure
// and the caller evaluates blend8_apply.
struct FF {
    float hi, lo;
};

__device__ __forceinline__ FF ff_two_sum(float a, float b) {  // exact: hi + lo = a + b
    const float s = __fadd_rn(a, b);
    const float bv = __fsub_rn(s, a);
    const float av = __fsub_rn(s, bv);
    return FF{s, __fadd_rn(__fsub_rn(a, av), __fsub_rn(b, bv))};
}

__device__ __forceinline__ FF ff_prod(float a, float b) {  // exact: hi + lo = a * b
    const float p = __fmul_rn(a, b);
    return FF{p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ FF ff_renorm(float a, float b) {  // |a| >= |b| or a == 0: exact
    const float s = __fadd_rn(a, b);
    return FF{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ FF ff_mul(FF x, FF y) {
    const FF p = ff_prod(x.hi, y.hi);
    return ff_renorm(p.hi, __fadd_rn(p.lo, __fadd_rn(__fmul_rn(x.hi, y.lo), __fmul_rn(x.lo, y.hi))));
}

__device__ __forceinline__ FF ff_mul_f(FF x, float f) {
    const FF p = ff_prod(x.hi, f);
    return ff_renorm(p.hi, __fadd_rn(p.lo, __fmul_rn(x.lo, f)));
}

__device__ __forceinline__ FF ff_add(FF x, FF y) {
    const FF s = ff_two_sum(x.hi, y.hi);
    return ff_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}

// The float nearest to acc (a normalised float-float value) if every value
// within eps of acc rounds to the same float; false if acc is that close to a
// midpoint between adjacent floats, or zero, tiny or huge.
__device__ __forceinline__ bool ff_round_safe(FF acc, float eps, float& out) {
    const float f = __fadd_rn(acc.hi, acc.lo);  // the float nearest to hi + lo
    const uint32_t bits = __float_as_uint(f) & 0x7fffffffu;
    const uint32_t e = bits >> 23;
    if (e < 27u || e > 253u) return false;
    // half the gap to the next float on either side (below a power of two the gap halves)
    const uint32_t he = (bits & 0x7fffffu) ? e - 24u : e - 25u;
    const float half_gap = __uint_as_float(he << 23);
    const float d = __fadd_rn(__fsub_rn(acc.hi, f), acc.lo);  // (hi + lo) - f, to one rounding
    if (!(fabsf(d) * 1.0000005f + eps < half_gap)) return false;
    out = f;
    return true;
}

struct FFWeights {
    FF w000, w100, w010, w001, w110, w101, w011;
    float dxdydz;
};

// The weights of blend8_weights in float-float (the same factors and products).
__device__ __forceinline__ FFWeights ff_weights(float dx, float dy, float dz) {
    FFWeights b;
    const FF a = ff_two_sum(1.0f, -dx), bb = ff_two_sum(1.0f, -dy), c = ff_two_sum(1.0f, -dz);
    const FF ab = ff_mul(a, bb);
    const FF ady = ff_mul_f(a, dy);
    const FF dxb = ff_mul_f(bb, dx);
    const float dxdy = dx * dy;  // float, as the reference's dx*dy
    b.w000 = ff_mul(ab, c);
    b.w100 = ff_mul(ady, c);
    b.w010 = ff_mul(dxb, c);
    b.w001 = ff_mul_f(ab, dz);
    b.w110 = ff_mul_f(c, dxdy);
    b.w101 = ff_mul_f(ady, dz);
    b.w011 = ff_mul_f(dxb, dz);
    b.dxdydz = dxdy * dz;
    return b;
}

// blend8_apply's result if it can be proven from the float-float evaluation.
__device__ __forceinline__ bool ff_blend8(const FFWeights& b, float c000, float c100, float c010, float c001,
                                          float c110, float c101, float c011, float c111, float& out) {
    const float S = fabsf(c000) + fabsf(c100) + fabsf(c010) + fabsf(c001) + fabsf(c110) + fabsf(c101) +
                    fabsf(c011) + fabsf(c111);
    if (!(S >= 0x1p-60f && S <= 0x1p+100f)) return false;  // also NaN / infinite corners
    FF acc = ff_mul_f(b.w000, c000);
    acc = ff_add(acc, ff_mul_f(b.w100, c100));
    acc = ff_add(acc, ff_mul_f(b.w010, c010));
    acc = ff_add(acc, ff_mul_f(b.w001, c001));
    acc = ff_add(acc, ff_mul_f(b.w110, c110));
    acc = ff_add(acc, ff_mul_f(b.w101, c101));
    acc = ff_add(acc, ff_mul_f(b.w011, c011));
    acc = ff_add(acc, FF{b.dxdydz * c111, 0.0f});
    return ff_round_safe(acc, S * 0x1p-40f, out);
}

// sample() through the float-float evaluation, falling back to the double one.
__device__ __forceinline__ float sample_ff(const float* __restrict__ v, const Corners& c, const FFWeights& w,
                                           float dx, float dy, float dz) {
    const float c000 = __ldg(v + c.o000), c100 = __ldg(v + c.o100), c010 = __ldg(v + c.o010),
                c001 = __ldg(v + c.o001), c110 = __ldg(v + c.o110), c101 = __ldg(v + c.o101),
                c011 = __ldg(v + c.o011), c111 = __ldg(v + c.o111);
    float r;
    if (ff_blend8(w, c000, c100, c010, c001, c110, c101, c011, c111, r)) return r;
    return blend8_apply(blend8_weights(dx, dy, dz), c000, c100, c010, c001, c110, c101, c011, c111);
}

// Split a float coordinate into floor (as int) and fraction, as `int x=floor(x1);
// float dx=x1-x;` does in the reference.
__device__ __forceinline__ void split_coord(float c, int& i, float& f) {
    i = (int)floorf(c);
    f = c - (float)i;
}


// ---- shared-memory barriers (mbarrier) with bounded waits
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// One try_wait round, suspended at most kTryWaitNs (the suspend-time hint caps the
// otherwise system-dependent suspension, so a wait of kWaitLimit rounds is bounded
// by about kWaitLimit microseconds); returns as soon as the phase completes.
constexpr uint32_t kTryWaitNs = 1000;
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(kTryWaitNs)
        : "memory");
    return ok != 0;
}
constexpr long long kWaitLimit = 1LL << 20;  // try_wait rounds of at most kTryWaitNs each: ~1 s

// Bounded wait of one thread on an mbarrier phase; false if the limit expired.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    for (long long i = 0; i < kWaitLimit; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

}  // namespace deeds
