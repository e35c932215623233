// Image statistics of primsGraph on sm_103a (src/primsMST.h:101-110): the mean
// and standard deviation that scale the MST edge weights, evaluated on the device
// so that the host trees need no copy of the images.
//
// The reference computes both with sequential float chains over the whole image:
//   mean: v = v + x[i]                                   (float)
//   var:  v = float(double(v) + double(x[i] - mean)^2)   (pow(float, 2) is double)
// and then mean / n, sqrt(var / n) in float.  The chains are evaluated exactly,
// in parallel segments, by the grid-translation argument that the host version
// (tree_host.cpp, image_stats) also uses: while every value of a chain lies
// strictly inside one binade [2^(e-1), 2^e) (or its negative), at least one grid
// step u = 2^(e-24) from its ends, each step is "add exactly, round to the
// u-grid" (the variance first to the double grid, then to the u-grid), so a start
// shifted by an even multiple of u shifts every later value by the same amount
// (rounding commutes with shifts by grid points; ties to even see the same
// parity).  Each segment runs the reference arithmetic from two starts one u
// apart in the binade of an estimated start (double partial sums); one warp then
// walks the segments in order, takes the trajectory whose start differs from the
// true one by an even multiple of u and shifts its end, after checking that it
// and its shifted copy stay inside the binade, and evaluates every other segment
// from the true start.  The result is the reference's to the bit for any data.
//
// Two levels: chunks of 2048 elements; a chunk whose own trajectory leaves its
// binade or comes near one of its ends (the sum crosses a power of two: about
// log2(sum / first element) chunks per chain) or that has no usable estimate is
// also run as 32 sub-segments, in parallel before the walk, so the walk replays
// at most a few sub-segments of 65 elements (staged in shared memory) where a
// chunk fails.  No thread walks a long stretch of global memory alone.
//
// Work: 4 B per voxel read by the chunk sums and once per chain, plus the
// crossing chunks twice more.  Dependency bound: 2048 steps per chunk chain and
// ~4000 sequential chunk checks (bit operations and float compares).
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "kernels.h"

namespace deeds {

namespace {

constexpr int kStatsChunk = 2048;  // elements per chunk (bounds sz * c / nch: 2048 to 4095)
constexpr int kSub = 32;           // sub-segments of a chunk run in parallel

struct ChunkRun {
    float start_a, start_b;  // the two starts (start_b one u from start_a)
    float end_a, lo_a, hi_a; // trajectory from start_a: last, smallest and largest value
    float end_b, lo_b, hi_b; // trajectory from start_b
    int spec;                // 1: both trajectories were run
    int cross;               // chunk level: 1 when its sub-segment runs exist
};

// A chunk's trajectories in units of u of their binade, for the walk's integer
// check: values are multiples of u with magnitudes in [2^23, 2^24) units.  A
// trajectory that leaves the binade carries lo > hi (never accepted).
struct WalkRec {
    int e, neg;                  // binade and sign of start_a (e = 0: no usable trajectories)
    int cross;                   // the chunk's sub-segment runs exist
    int sa, sb, ea, eb;          // starts and ends
    int loa, hia, lob, hib;      // extremes of each trajectory
};

__device__ __forceinline__ size_t chunk_lo(size_t sz, int nch, int c) { return sz * (size_t)c / (size_t)nch; }

// 2^k as a float, for k in the normal range (bit construction: exact)
__device__ __forceinline__ float pow2f(int k) { return __uint_as_float((unsigned)(k + 127) << 23); }

// binade exponent (|v| in [2^(e-1), 2^e)) and its grid step u; false for 0, tiny
// (below 2^-100) or non-finite v.  From the exponent bits: v = f 2^e, f in [0.5, 1).
__device__ __forceinline__ bool binade(float v, int& e, float& u) {
    const int be = (int)((__float_as_uint(v) >> 23) & 0xffu);
    if (be == 0xff || be < 27) return false;
    e = be - 126;
    u = pow2f(e - 24);
    return true;
}

// every value of [lo, hi] (shifted by d) strictly inside the binade e of sign neg
// (at least u from its ends).  Float arithmetic is exact here: the bounds are
// multiples of u inside the binade; with d = 0 nothing is added; with d != 0 the
// caller has checked d = 0 first, so lo, hi and d are multiples of u and every
// sum below 2^e is exact, while a sum at or above 2^e rounds to a value at or
// above 2^e (rounding is monotone and 2^e is a float) and fails as it must.
__device__ __forceinline__ bool inside(float lo, float hi, float d, int e, float u, bool neg) {
    const float inner = pow2f(e - 1) + u, outer = pow2f(e) - 2.0f * u;
    const float l = lo + d, h = hi + d;
    return neg ? (l >= -outer && h <= -inner) : (l >= inner && h <= outer);
}

// Kept out of line so that the compiler cannot if-convert the rare double path
// of var_step into every step (FP64 is slow on this part).
__device__ __noinline__ float var_step_double(float v, float d) {
    return (float)((double)v + (double)d * (double)d);
}

// The variance step float(double(v) + double(d)^2) without FP64 (GB300's FP64
// rate is a small fraction of its FP32 rate).  x = v + d^2 (exact real) needs two
// roundings, to double then to float; fmaf gives s = RN_float(x) with one.  The
// two differ only when RN_double(x) is the midpoint M between the two floats
// around x (a double: 25 significant bits) while x is not M, i.e. when x lies
// within half a double ulp (<= 2^-29 ulp_float) of M.  With d^2 = hi + lo
// exactly (fmaf residual) and v + hi = a + b exactly (TwoSum), e = (a - s) +
// (b + lo) equals x - s up to 2^-23 ulp_float (a - s is exact by Sterbenz: v,
// d^2 >= 0 and a, s are within ulps of x), and x is near a midpoint exactly
// when |e| is near ulp_float / 2.  So: s unless | |e| - ulp/2 | <= 2^-20 ulp
// (or s is a power of two, where the float spacing changes, or tiny or not
// finite), in which case the double formula decides.  Either way the result is
// the reference's.
__device__ __forceinline__ float var_step(float v, float d) {
    const float s = fmaf(d, d, v);
    const float hi = __fmul_rn(d, d);
    const float lo = fmaf(d, d, -hi);
    const float a = __fadd_rn(v, hi);
    const float bv = __fsub_rn(a, hi);
    const float bh = __fsub_rn(a, bv);
    const float b = __fadd_rn(__fsub_rn(v, bv), __fsub_rn(hi, bh));
    const float e = __fadd_rn(__fsub_rn(a, s), __fadd_rn(b, lo));
    const unsigned sb = __float_as_uint(s);
    const unsigned ex = sb & 0x7f800000u;
    // s >= 2^-100, finite, not a power of two (mantissa bits set)
    const bool plain = ex >= 0x0d800000u && ex != 0x7f800000u && (sb & 0x007fffffu) != 0u;
    const float ulp = __uint_as_float(ex) * 0x1p-23f;  // exact for these exponents
    if (plain && fabsf(fabsf(e) - 0.5f * ulp) > ulp * 0x1p-20f) return s;
    return var_step_double(v, d);
}

// One step of a chain: KIND 0 the mean's float sum, KIND 1 the variance's
// double-rounded sum of squares around `mean`.
template <int KIND>
__device__ __forceinline__ float chain_step(float v, float x, float mean) {
    return KIND == 0 ? v + x : var_step(v, x - mean);
}

// Whether a segment's trajectory can be shifted onto the true start v (its
// start's binade is v's, the start differs from v by an even multiple of u and
// the trajectory and its shifted copy stay inside the binade); if so nv is the
// segment's true end.
__device__ __forceinline__ bool shift_ok(const ChunkRun& cr, float v, float& nv) {
    int e, eg;
    float u, ug;
    if (!cr.spec || !binade(v, e, u) || !binade(cr.start_a, eg, ug) || e != eg || signbit(v) != signbit(cr.start_a))
        return false;
    // both are multiples of u below 2^e in magnitude: their distance in units of u
    // is the difference of two exact integers below 2^24
    const float inv_u = pow2f(24 - e);  // exact scalings by a power of two
    const int k = (int)(fabsf(v) * inv_u) - (int)(fabsf(cr.start_a) * inv_u);
    const bool even = (k & 1) == 0;
    const float start = even ? cr.start_a : cr.start_b;
    const float lo = even ? cr.lo_a : cr.lo_b, hi = even ? cr.hi_a : cr.hi_b;
    const float end = even ? cr.end_a : cr.end_b;
    const float d = v - start;  // exact: both multiples of u in one binade
    const bool neg = signbit(v);
    if (!inside(lo, hi, 0.0f, e, u, neg) || !inside(lo, hi, d, e, u, neg)) return false;
    nv = end + d;  // exact: a multiple of u inside the binade
    return true;
}

// The two starts of a segment whose true start is estimated by `est`.
__device__ __forceinline__ void spec_starts(float est, ChunkRun& cr) {
    int e;
    float u;
    cr.start_a = est;
    if (binade(est, e, u)) {
        cr.start_b = fabsf(est + u) < pow2f(e) ? est + u : est - u;  // one u away, same binade
        cr.spec = 1;
    } else {
        cr.start_b = est;
        cr.spec = 0;
    }
    cr.cross = 0;
    cr.end_a = cr.lo_a = cr.hi_a = cr.start_a;
    cr.end_b = cr.lo_b = cr.hi_b = cr.start_b;
}

// Both trajectories of a segment xs[0..n) from cr's starts, continuing cr (lo/hi
// accumulate).  The variance's chains never decrease (squares are added), so
// their extremes are start and end.
template <int KIND>
__device__ __forceinline__ void run_pair(const float* xs, int n, float mean, ChunkRun& cr) {
    float va = cr.end_a, vb = cr.end_b;
    if (KIND == 0) {
        float la = cr.lo_a, ha = cr.hi_a, lb = cr.lo_b, hb = cr.hi_b;
#pragma unroll 8
        for (int i = 0; i < n; i++) {
            const float xi = xs[i];
            va = va + xi;
            vb = vb + xi;
            la = fminf(la, va);
            ha = fmaxf(ha, va);
            lb = fminf(lb, vb);
            hb = fmaxf(hb, vb);
        }
        cr.lo_a = la; cr.hi_a = ha;
        cr.lo_b = lb; cr.hi_b = hb;
    } else {
#pragma unroll 8
        for (int i = 0; i < n; i++) {
            const float d = xs[i] - mean;
            va = var_step(va, d);
            vb = var_step(vb, d);
        }
        cr.hi_a = va;  // lo stays the segment's start
        cr.hi_b = vb;
    }
    cr.end_a = va;
    cr.end_b = vb;
}

// Stage xs[0..n) into shared memory with asynchronous copies (all in flight at
// once), by the calling warp.
__device__ __forceinline__ void stage_async(float* dst, const float* __restrict__ src, int n) {
    const int lane = threadIdx.x & 31;
    for (int i = lane; i < n; i += 32) {
        const unsigned sa = (unsigned)__cvta_generic_to_shared(dst + i);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(src + i) : "memory");
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncwarp();
}

// Chunk sums in double (estimates of the chains' values at chunk starts; any
// order of addition).  Grid (nch, nimg), 256 threads.
__global__ void __launch_bounds__(256) k_stats_sums(const float* __restrict__ im0, const float* __restrict__ im1,
                                                    size_t sz, int nch, double* __restrict__ sx,
                                                    double* __restrict__ sx2) {
    const float* x = blockIdx.y == 0 ? im0 : im1;
    const int c = blockIdx.x;
    const size_t lo = chunk_lo(sz, nch, c), hi = chunk_lo(sz, nch, c + 1);
    double s = 0.0, q = 0.0;
    for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const double v = x[i];
        s += v;
        q += v * v;
    }
    __shared__ double red_s[8], red_q[8];
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        q += __shfl_xor_sync(0xffffffffu, q, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red_s[w] = s;
        red_q[w] = q;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ts = 0.0, tq = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
            ts += red_s[k];
            tq += red_q[k];
        }
        sx[(size_t)blockIdx.y * nch + c] = ts;
        sx2[(size_t)blockIdx.y * nch + c] = tq;
    }
}

// Start estimates of every chunk (exclusive prefix of the chunk sums; for the
// variance, sum (x - m)^2 = sum x^2 - 2 m sum x + n m^2 with the estimated mean
// m) and the two starts of each chunk's trajectories.  One block of 1024 threads
// per image; each thread scans a run of consecutive chunks.
template <int KIND>
__global__ void __launch_bounds__(1024) k_stats_starts(size_t sz, int nch, const double* __restrict__ sx,
                                                       const double* __restrict__ sx2, ChunkRun* __restrict__ run) {
    const int img = blockIdx.x;
    const double* s = sx + (size_t)img * nch;
    const double* q = sx2 + (size_t)img * nch;
    ChunkRun* r = run + (size_t)img * nch;
    __shared__ double part[1024];
    __shared__ double total_s;
    const int T = blockDim.x, t = threadIdx.x;
    const int per = (nch + T - 1) / T;
    const int c0 = min(nch, t * per), c1 = min(nch, c0 + per);
    double m = 0.0;
    if (KIND == 1) {
        double a = 0.0;
        for (int c = c0; c < c1; c++) a += s[c];
        part[t] = a;
        __syncthreads();
        if (t == 0) {
            double tot = 0.0;
            for (int k = 0; k < T; k++) tot += part[k];
            total_s = tot;
        }
        __syncthreads();
        m = total_s / (double)sz;
        __syncthreads();
    }
    auto term = [&](int c) {
        if (KIND == 0) return s[c];
        const double n = (double)(chunk_lo(sz, nch, c + 1) - chunk_lo(sz, nch, c));
        return fmax(0.0, q[c] - 2.0 * m * s[c] + n * m * m);
    };
    double a = 0.0;
    for (int c = c0; c < c1; c++) a += term(c);
    part[t] = a;
    __syncthreads();
    // inclusive Hillis-Steele scan of the per-thread totals
    for (int off = 1; off < T; off <<= 1) {
        const double v = t >= off ? part[t - off] : 0.0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    double pre = t > 0 ? part[t - 1] : 0.0;
    for (int c = c0; c < c1; c++) {
        const float est = (float)pre;
        pre += term(c);
        ChunkRun cr;
        spec_starts(est, cr);
        r[c] = cr;
    }
}

// Both trajectories of every speculated chunk, one lane per chunk: a warp owns
// 32 consecutive chunks and loads them 32 elements per chunk at a time, one
// coalesced 128-byte row per load (the row's base broadcast from its lane), into
// a padded shared tile that each lane then reads along its own row.  A chunk
// whose trajectory leaves its binade or comes near one of its ends, or that has
// no usable estimate, is marked for sub-segment runs; every chunk's integer
// walk record is written.  Grid (ceil(nch / 32), nimg), 32 threads.
template <int KIND>
__global__ void __launch_bounds__(32) k_stats_traj(const float* __restrict__ im0, const float* __restrict__ im1,
                                                   size_t sz, int nch, const float* __restrict__ means,
                                                   ChunkRun* __restrict__ run, WalkRec* __restrict__ walk) {
    __shared__ float tile[32][33];
    const float* x = blockIdx.y == 0 ? im0 : im1;
    const int lane = threadIdx.x;
    const int c = blockIdx.x * 32 + lane;
    size_t lo = 0;
    int len = 0;
    ChunkRun cr;
    cr.spec = 0;
    if (c < nch) {
        lo = chunk_lo(sz, nch, c);
        len = (int)(chunk_lo(sz, nch, c + 1) - lo);
        cr = run[(size_t)blockIdx.y * nch + c];
    }
    const float mean = KIND == 1 ? means[blockIdx.y] : 0.0f;
    const int maxlen = (int)(sz / (size_t)nch) + 1;  // chunk lengths are floor or ceil of sz / nch
    for (int k0 = 0; k0 < maxlen; k0 += 32) {
#pragma unroll
        for (int r = 0; r < 32; r++) {
            const size_t base = __shfl_sync(0xffffffffu, lo, r);
            const int n = __shfl_sync(0xffffffffu, len, r);
            tile[r][lane] = k0 + lane < n ? __ldg(x + base + k0 + lane) : 0.0f;
        }
        __syncwarp();
        if (cr.spec) {
            const int n = min(32, len - k0);
            if (n > 0) run_pair<KIND>(&tile[lane][0], n, mean, cr);
        }
        __syncwarp();
    }
    if (c >= nch) return;
    // also marked: chunks whose trajectory comes within 2^-12 of the binade's
    // width of an end, which a shift onto the true start could push out
    int e = 0;
    float u = 0.0f;
    bool in = cr.spec && binade(cr.start_a, e, u);
    const bool neg = signbit(cr.start_a);
    WalkRec w;
    w.e = 0;
    if (in) {
        const float margin = pow2f(e - 13);
        // (fminf / fmaxf skip NaN, so a trajectory that met a NaN is recognised by its end)
        const bool ina = isfinite(cr.end_a) && inside(cr.lo_a, cr.hi_a, 0.0f, e, u, neg);
        const bool inb = isfinite(cr.end_b) && inside(cr.lo_b, cr.hi_b, 0.0f, e, u, neg);
        const float inv_u = pow2f(24 - e);
        w.e = e;
        w.neg = neg;
        w.sa = (int)(cr.start_a * inv_u);
        w.sb = (int)(cr.start_b * inv_u);
        w.ea = (int)(cr.end_a * inv_u);
        w.eb = (int)(cr.end_b * inv_u);
        w.loa = ina ? (int)(cr.lo_a * inv_u) : 1;
        w.hia = ina ? (int)(cr.hi_a * inv_u) : 0;
        w.lob = inb ? (int)(cr.lo_b * inv_u) : 1;
        w.hib = inb ? (int)(cr.hi_b * inv_u) : 0;
        in = ina && inside(cr.lo_a, cr.hi_a, margin, e, u, neg) && inside(cr.lo_a, cr.hi_a, -margin, e, u, neg);
    }
    cr.cross = !in;
    w.cross = cr.cross;
    run[(size_t)blockIdx.y * nch + c] = cr;
    walk[(size_t)blockIdx.y * nch + c] = w;
}

// Second estimates of every chunk's start: the exclusive prefix of the first
// pass's float increments (end - start of each speculated chunk's trajectory;
// the double chunk sum where there was none).  The float chain drops the parts
// of small terms that round away against a large sum, so these follow the true
// chain far more closely than the exact sums do.  One block of 1024 threads per
// image.
template <int KIND>
__global__ void __launch_bounds__(1024) k_stats_restarts(size_t sz, int nch, const double* __restrict__ sx,
                                                         const double* __restrict__ sx2, ChunkRun* __restrict__ run) {
    const int img = blockIdx.x;
    const double* s = sx + (size_t)img * nch;
    const double* q = sx2 + (size_t)img * nch;
    ChunkRun* r = run + (size_t)img * nch;
    __shared__ double part[1024];
    __shared__ double total_s;
    const int T = blockDim.x, t = threadIdx.x;
    const int per = (nch + T - 1) / T;
    const int c0 = min(nch, t * per), c1 = min(nch, c0 + per);
    double m = 0.0;
    if (KIND == 1) {
        double a = 0.0;
        for (int c = c0; c < c1; c++) a += s[c];
        part[t] = a;
        __syncthreads();
        if (t == 0) {
            double tot = 0.0;
            for (int k = 0; k < T; k++) tot += part[k];
            total_s = tot;
        }
        __syncthreads();
        m = total_s / (double)sz;
        __syncthreads();
    }
    auto inc = [&](int c) {
        const ChunkRun& cr = r[c];
        if (cr.spec) return (double)cr.end_a - (double)cr.start_a;
        if (KIND == 0) return s[c];
        const double n = (double)(chunk_lo(sz, nch, c + 1) - chunk_lo(sz, nch, c));
        return fmax(0.0, q[c] - 2.0 * m * s[c] + n * m * m);
    };
    double a = 0.0;
    for (int c = c0; c < c1; c++) a += inc(c);
    part[t] = a;
    __syncthreads();
    for (int off = 1; off < T; off <<= 1) {
        const double v = t >= off ? part[t - off] : 0.0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    double pre = t > 0 ? part[t - 1] : 0.0;
    for (int c = c0; c < c1; c++) {  // each thread rewrites only its own chunks
        const float est = (float)pre;
        pre += inc(c);
        ChunkRun cr;
        spec_starts(est, cr);
        r[c] = cr;
    }
}

// Sub-segment runs of the chunks marked by k_stats_traj: the chunk is staged in
// shared memory, each lane runs one of its 32 sub-segments (odd length:
// conflict-free) from two starts around the chunk's estimate plus the double
// prefix of the sub-segments before it.  The walk shifts these onto the true
// chunk start.  Grid (nch, nimg), 32 threads; dynamic shared memory: the
// largest chunk.
template <int KIND>
__global__ void __launch_bounds__(32) k_stats_sub(const float* __restrict__ im0, const float* __restrict__ im1,
                                                  size_t sz, int nch, const float* __restrict__ means,
                                                  const ChunkRun* __restrict__ run, ChunkRun* __restrict__ sub) {
    extern __shared__ float buf[];
    const int c = blockIdx.x, img = blockIdx.y, lane = threadIdx.x;
    const ChunkRun cr = run[(size_t)img * nch + c];
    if (!cr.cross) return;
    const float* x = img == 0 ? im0 : im1;
    const size_t lo = chunk_lo(sz, nch, c), hi = chunk_lo(sz, nch, c + 1);
    const int n = (int)(hi - lo);
    stage_async(buf, x + lo, n);
    const float mean = KIND == 1 ? means[img] : 0.0f;
    const int S = ((n + kSub - 1) / kSub) | 1;
    const int b0 = min(n, lane * S), b1 = min(n, b0 + S);
    double part = 0.0;
    for (int i = b0; i < b1; i++) {
        const double xi = KIND == 0 ? (double)buf[i] : (double)(buf[i] - mean);
        part += KIND == 0 ? xi : xi * xi;
    }
    double incl = part;
    for (int o = 1; o < 32; o <<= 1) {
        const double y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    ChunkRun mine;
    spec_starts((float)((double)cr.start_a + (incl - part)), mine);
    if (mine.spec) run_pair<KIND>(buf + b0, b1 - b0, mean, mine);
    sub[((size_t)img * nch + c) * kSub + lane] = mine;
}

// The true chain over one segment xs[0..n) from v by the whole warp (every lane
// computes the same values), with the segment staged in shared memory: the
// sub-segment runs `sr` (or, without them, runs made here from estimates around
// v) are shifted where they allow it and the others replayed.
template <int KIND>
__device__ float warp_segment(const float* __restrict__ xg, int n, float v, float mean, const ChunkRun* sr,
                              float* buf) {
    const int lane = threadIdx.x & 31;
    __syncwarp();
    stage_async(buf, xg, n);
    const int S = ((n + kSub - 1) / kSub) | 1;
    ChunkRun mine;
    if (sr) {
        mine = sr[lane];
    } else {
        const int b0 = min(n, lane * S), b1 = min(n, b0 + S);
        double part = 0.0;
        for (int i = b0; i < b1; i++) {
            const double xi = KIND == 0 ? (double)buf[i] : (double)(buf[i] - mean);
            part += KIND == 0 ? xi : xi * xi;
        }
        double incl = part;
        for (int o = 1; o < 32; o <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        spec_starts((float)((double)v + (incl - part)), mine);
        if (mine.spec) run_pair<KIND>(buf + b0, b1 - b0, mean, mine);
    }
    for (int k = 0; k < kSub; k++) {
        if (isnan(v)) break;  // absorbing for both chains
        ChunkRun cr;
        cr.start_a = __shfl_sync(0xffffffffu, mine.start_a, k);
        cr.start_b = __shfl_sync(0xffffffffu, mine.start_b, k);
        cr.end_a = __shfl_sync(0xffffffffu, mine.end_a, k);
        cr.lo_a = __shfl_sync(0xffffffffu, mine.lo_a, k);
        cr.hi_a = __shfl_sync(0xffffffffu, mine.hi_a, k);
        cr.end_b = __shfl_sync(0xffffffffu, mine.end_b, k);
        cr.lo_b = __shfl_sync(0xffffffffu, mine.lo_b, k);
        cr.hi_b = __shfl_sync(0xffffffffu, mine.hi_b, k);
        cr.spec = __shfl_sync(0xffffffffu, mine.spec, k);
        float nv;
        if (shift_ok(cr, v, nv)) {
            v = nv;
        } else {
            const int e0 = min(n, k * S), e1 = min(n, e0 + S);
            for (int i = e0; i < e1; i++) v = chain_step<KIND>(v, buf[i], mean);
        }
    }
    __syncwarp();
    return v;
}

// The true chain, chunk by chunk (one warp per image; every lane holds the same
// value).  While the value lies in a binade it is kept as an integer V in units
// of u, and a chunk whose trajectory (chosen by the parity of V - its start) and
// that trajectory shifted by V - start stay inside the binade gives V' = its end
// + the shift, with integer operations only; any other chunk is evaluated by
// warp_segment from the float value.  The walk records are read 32 at a time.
// KIND 0 writes the mean, KIND 1 the standard deviation (out[2 img + 0 / 1]).
// Dynamic shared memory: the largest chunk.
template <int KIND>
__global__ void __launch_bounds__(32) k_stats_stitch(const float* __restrict__ im0, const float* __restrict__ im1,
                                                     size_t sz, int nch, const ChunkRun* __restrict__ run,
                                                     const WalkRec* __restrict__ walk, const ChunkRun* __restrict__ sub,
                                                     float* __restrict__ means, float* __restrict__ out) {
    extern __shared__ float buf[];
    __shared__ WalkRec batch[32];
    const int img = blockIdx.x, lane = threadIdx.x;
    const float* x = img == 0 ? im0 : im1;
    const float mean = KIND == 1 ? means[img] : 0.0f;
    constexpr int IN = (1 << 23) + 1, OUT = (1 << 24) - 2;
    float v = 0.0f;
    int ve = 0, vneg = 0, V = 0;  // ve = 0: v is not held as an integer (0, tiny or not finite)
    // the next batch of records is loaded into registers while this one is walked
    WalkRec nextrec;
    if (lane < nch) nextrec = walk[(size_t)img * nch + lane];
    for (int c0 = 0; c0 < nch && !isnan(v); c0 += 32) {
        __syncwarp();
        batch[lane] = nextrec;
        if (c0 + 32 + lane < nch) nextrec = walk[(size_t)img * nch + c0 + 32 + lane];
        __syncwarp();
        const int nb = min(32, nch - c0);
        for (int k = 0; k < nb; k++) {
            const WalkRec& w = batch[k];
            bool ok = false;
            if (ve != 0 && w.e == ve && w.neg == vneg) {
                const bool odd = ((V - w.sa) & 1) != 0;
                const int S = odd ? w.sb : w.sa, E = odd ? w.eb : w.ea;
                const int LO = odd ? w.lob : w.loa, HI = odd ? w.hib : w.hia;
                const int D = V - S, l = LO + D, h = HI + D;
                ok = LO <= HI && (vneg ? (l >= -OUT && h <= -IN) : (l >= IN && h <= OUT));
                if (ok) V = E + D;
            }
            if (ok) continue;
            // the float value, then the chunk exactly
            if (ve != 0) v = (float)V * pow2f(ve - 24);
            if (isnan(v)) break;  // absorbing for both chains: the result is NaN
            const int c = c0 + k;
            const size_t lo = chunk_lo(sz, nch, c), hi = chunk_lo(sz, nch, c + 1);
            const ChunkRun* sr = w.cross ? sub + ((size_t)img * nch + c) * kSub : nullptr;
            v = warp_segment<KIND>(x + lo, (int)(hi - lo), v, mean, sr, buf);
            float u;
            if (binade(v, ve, u)) {
                vneg = signbit(v) ? 1 : 0;
                V = (int)(v * pow2f(24 - ve));
            } else {
                ve = 0;
            }
        }
    }
    if (ve != 0) v = (float)V * pow2f(ve - 24);
    if (lane == 0) {
        if (KIND == 0) {
            const float m = v / (float)sz;
            means[img] = m;
            out[2 * img] = m;
        } else {
            out[2 * img + 1] = sqrtf(v / (float)sz);
        }
    }
}

int stats_chunks(size_t sz) { return (int)std::max<size_t>(1, sz / kStatsChunk); }

// bytes of the largest chunk staged in shared memory (chunks are below 2 x kStatsChunk)
constexpr int kSegSmemMax = (int)((2 * (size_t)kStatsChunk + 2) * sizeof(float));

}  // namespace

size_t image_stats_scratch_bytes(size_t sz, int nimg) {
    const size_t nch = (size_t)stats_chunks(sz);
    return 256 + (size_t)nimg * nch * (2 * sizeof(double) + sizeof(ChunkRun) * (1 + kSub) + sizeof(WalkRec)) + 64;
}

// Mean and standard deviation of one or two images (im1 may be null when nimg
// is 1) into out[2 * img + 0 / 1], in the reference's float semantics.
cudaError_t launch_image_stats(const float* im0, const float* im1, int nimg, size_t sz, void* scratch, float* out,
                               cudaStream_t s) {
    if (nimg < 1 || nimg > 2 || sz == 0 || !im0 || (nimg == 2 && !im1) || !scratch || !out)
        return cudaErrorInvalidValue;
    const int nch = stats_chunks(sz);
    char* p = static_cast<char*>(scratch);
    float* means = reinterpret_cast<float*>(p);
    p += 256;
    double* sx = reinterpret_cast<double*>(p);
    p += (size_t)nimg * nch * sizeof(double);
    double* sx2 = reinterpret_cast<double*>(p);
    p += (size_t)nimg * nch * sizeof(double);
    ChunkRun* run = reinterpret_cast<ChunkRun*>(p);
    p += (size_t)nimg * nch * sizeof(ChunkRun);
    ChunkRun* sub = reinterpret_cast<ChunkRun*>(p);
    p += (size_t)nimg * nch * kSub * sizeof(ChunkRun);
    WalkRec* walk = reinterpret_cast<WalkRec*>(p);
    if (!im1) im1 = im0;
    // the shared-memory limits are set to the bound on every call, never lowered,
    // so concurrent callers cannot race on them
    const size_t seg_smem = ((size_t)(sz / (size_t)nch) + 2) * sizeof(float);
    cudaError_t e = cudaSuccess;
    for (const void* f : {(const void*)k_stats_stitch<0>, (const void*)k_stats_stitch<1>, (const void*)k_stats_sub<0>,
                          (const void*)k_stats_sub<1>})
        if (e == cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, kSegSmemMax);
    if (e != cudaSuccess) return e;
    const dim3 tgrid((nch + 31) / 32, nimg), cgrid(nch, nimg);
    k_stats_sums<<<cgrid, 256, 0, s>>>(im0, im1, sz, nch, sx, sx2);
    k_stats_starts<0><<<nimg, 1024, 0, s>>>(sz, nch, sx, sx2, run);
    k_stats_traj<0><<<tgrid, 32, 0, s>>>(im0, im1, sz, nch, means, run, walk);
    k_stats_restarts<0><<<nimg, 1024, 0, s>>>(sz, nch, sx, sx2, run);
    k_stats_traj<0><<<tgrid, 32, 0, s>>>(im0, im1, sz, nch, means, run, walk);
    k_stats_sub<0><<<cgrid, 32, seg_smem, s>>>(im0, im1, sz, nch, means, run, sub);
    k_stats_stitch<0><<<nimg, 32, seg_smem, s>>>(im0, im1, sz, nch, run, walk, sub, means, out);
    k_stats_starts<1><<<nimg, 1024, 0, s>>>(sz, nch, sx, sx2, run);
    k_stats_traj<1><<<tgrid, 32, 0, s>>>(im0, im1, sz, nch, means, run, walk);
    k_stats_restarts<1><<<nimg, 1024, 0, s>>>(sz, nch, sx, sx2, run);
    k_stats_traj<1><<<tgrid, 32, 0, s>>>(im0, im1, sz, nch, means, run, walk);
    k_stats_sub<1><<<cgrid, 32, seg_smem, s>>>(im0, im1, sz, nch, means, run, sub);
    k_stats_stitch<1><<<nimg, 32, seg_smem, s>>>(im0, im1, sz, nch, run, walk, sub, means, out);
    count_launches(13);
    return cudaGetLastError();
}

}  // namespace deeds
