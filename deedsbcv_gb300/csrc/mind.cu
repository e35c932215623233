// MIND-SSC descriptor on sm_103a (replaces descriptor(), src/MINDSSCbox.h:127-232).
//
// Layout in HBM: six distance channels D[l][p] (6 x m*n*o float32, context
// scratch) and the output codes C[p] (uint64).  Four launches:
//   1. k_pass_i: per (j,k) line and channel, the shifted squared difference
//      (imshift + distances, src/MINDSSCbox.h:79-124) streamed into the i-axis
//      box sum, through shared-memory tiles so loads and stores are coalesced;
//   2. k_pass_jk (j) / 3. k_pass_jk (k): the j- and k-axis box sums, in place;
//   4. k_quantise: the 12 SSC pairs -> min/mean normalisation -> 5 thresholds
//      -> thermometer code (src/MINDSSCbox.h:175-224).
// Box sums keep the reference's sequential float prefix sum along each line and
// its edge rules (src/MINDSSCbox.h:9-73): one thread owns one line and streams it
// with a lag of r, keeping the last 2r+2 prefix values in a ring; a parallel
// scan would change the rounding and with it codes near thresholds.
// Roofline: HBM-bound; per call ~ 4 B read + 24 B write (pass i), 2 x 48 B
// (passes j, k), 24 B read + 8 B write (quantise) per voxel = 152 B/voxel.
#include <cmath>

#include "common.cuh"
#include "kernels.h"

namespace deeds {

namespace {

constexpr int kRing = 16;  // supports box radius r <= 7 (2r+2 <= 16)

// Shift vectors of the six distance channels (src/MINDSSCbox.h:132-134).
__constant__ int c_dx[6] = {1, 1, -1, 0, 1, 0};
__constant__ int c_dy[6] = {1, -1, 0, -1, 0, 1};
__constant__ int c_dz[6] = {0, 0, 1, 1, 1, 1};

// i-axis pass: CTA = one k slice x TJ consecutive j lines x all 6 channels.
// The image neighbourhood of an i-chunk (rows j-q..j+TJ+q at k and k+q, i-q..i+CH+q)
// is staged in shared memory with coalesced loads; each thread streams one
// (channel, line) through the sequential box sum; outputs go through a shared
// tile so that the six channel planes are written with coalesced stores.
// The radius QS is a compile-time constant and chunks start at multiples of 16,
// so every index into the ring of prefix values is static after unrolling and the
// ring lives in registers (a runtime index would place it in local memory); the
// tail outputs are emitted at the line's last step for the same reason.
constexpr int TJ = 32;  // lines per CTA
constexpr int CH = 32;  // i samples per chunk (a multiple of kRing)
static_assert(CH == 32 && TJ == 32, "one lane per sample; warp l of a CTA is channel l");

template <int QS>
__global__ void __launch_bounds__(6 * TJ) k_pass_i(const float* __restrict__ im, float* __restrict__ D, int m, int n,
                                                   int o) {
    extern __shared__ float sm[];
    constexpr int W = CH + 2 * QS + 1;     // padded row length of the image tile
    constexpr int WL = CH + 2 * QS;        // loaded row length
    constexpr int R = TJ + 2 * QS;         // image rows per k slice
    float* Tbuf = sm;                      // two tiles [2][R][W]: the chunk's, and the next one's in flight
    float* O = sm + 4 * R * W;             // [6][TJ][CH+1]
    const int k = blockIdx.y, j0 = blockIdx.x * TJ;
    const int l = threadIdx.x / TJ, jj = threadIdx.x % TJ, j = j0 + jj;
    const int64_t mn = (int64_t)m * n, sz = mn * o;
    const int dx = c_dx[l] * QS, dy = c_dy[l] * QS, dz = c_dz[l] * QS;
    const bool line_ok = j < n;
    const bool other_ok = j + dx >= 0 && j + dx < n && k + dz < o;
    const int kk = dz ? 1 : 0;
    float* gout = D + l * sz + (int64_t)j * m + (int64_t)k * mn;
    float ring[kRing];
    float P = 0.0f;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int kWarps = 6 * TJ / 32;
    // the image tile of the chunk at i0 into Tb with 4-byte cp.async, one warp per
    // tile row (rows of both k planes); samples outside the volume are zero-filled
    // (no bytes read)
    auto load_tile = [&](int i0, float* Tb) {
        for (int row = warp; row < 2 * R; row += kWarps) {
            const int z = row / R, r = row - z * R;
            const int jr = j0 - QS + r, kz = k + z * QS;
            const bool row_ok = jr >= 0 && jr < n && kz < o;
            const float* src = im + (int64_t)(row_ok ? jr : 0) * m + (int64_t)(row_ok ? kz : 0) * mn;
            float* dst = Tb + row * W;
#pragma unroll
            for (int ip = lane; ip < WL; ip += 32) {
                const int ii = i0 - QS + ip;
                const bool ok = row_ok && ii >= 0 && ii < m;
                const unsigned d = (unsigned)__cvta_generic_to_shared(dst + ip);
                asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(ok ? src + ii : im),
                             "r"(ok ? 4 : 0)
                             : "memory");
            }
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    load_tile(0, Tbuf);
    for (int i0 = 0, c = 0; i0 < m; i0 += CH, c++) {
        float* T = Tbuf + (c & 1) * 2 * R * W;
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        __syncthreads();  // this chunk's tile has landed; the previous chunk's tile is consumed
        if (i0 + CH < m) load_tile(i0 + CH, Tbuf + ((c + 1) & 1) * 2 * R * W);  // in flight during this chunk
        const int cend = min(CH, m - i0);
        // interior chunk: no line start or end, no shifted sample outside the line, all
        // CH samples present; the steps need no index checks
        const bool interior = i0 >= CH && i0 + CH + QS <= m;
        if (line_ok && interior) {
            const float* self = T + (jj + QS) * W + QS;
            // a partner line outside the volume compares the voxel with itself (d = 0)
            const float* oth = other_ok ? T + (kk * R + jj + QS + dx) * W + QS + dy : self;
            float* out = O + (l * TJ + jj) * (CH + 1);
#pragma unroll
            for (int u = 0; u < CH; u++) {
                const float d = oth[u] - self[u];
                P = P + d * d;
                ring[u & (kRing - 1)] = P;  // i0 is a multiple of kRing
                out[u] = P - ring[(u - 2 * QS - 1) & (kRing - 1)];
            }
        } else if (line_ok) {
            const float* self = T + (jj + QS) * W + QS;
            const float* oth = T + (kk * R + jj + QS + dx) * W + QS + dy;
            float* out = O + (l * TJ + jj) * (CH + 1);
#pragma unroll
            for (int u = 0; u < CH; u++) {
                if (u < cend) {
                    const int t = i0 + u;
                    const float s = self[u];
                    const float v = (other_ok && t + dy >= 0 && t + dy < m) ? oth[u] : s;
                    const float d = v - s;
                    const float x = d * d;
                    P = (t == 0) ? x : P + x;
                    ring[u & (kRing - 1)] = P;  // i0 is a multiple of kRing
                    const int i = t - QS;       // output position (lag r = QS)
                    if (i >= 0) out[u] = (i <= QS) ? P : P - ring[(u - 2 * QS - 1) & (kRing - 1)];
                    if (t == m - 1) {
                        // tail: i in [m-QS, m): P[m-1] - P[i-QS-1]
#pragma unroll
                        for (int s2 = 0; s2 < QS; s2++) gout[m - QS + s2] = P - ring[(u - 2 * QS + s2) & (kRing - 1)];
                    }
                }
            }
        }
        __syncwarp();  // a warp stores the output rows its own lanes wrote (warp = channel)
        // coalesced store of outputs i0-QS .. i0+cend-1-QS: the warp of channel l stores
        // its TJ lines, one lane per sample (CH == 32)
        {
            const int i = i0 + lane - QS;
            if (lane < cend && i >= 0) {
                const int nl = min(TJ, n - j0);
                float* dst = D + warp * sz + (int64_t)k * mn + (int64_t)j0 * m + i;
                const float* src = O + warp * TJ * (CH + 1) + lane;
#pragma unroll 8
                for (int jl = 0; jl < nl; jl++) dst[(int64_t)jl * m] = src[jl * (CH + 1)];
            }
        }
    }
}

// In-place box pass along j (axis=1) or k (axis=2); threads over consecutive i.
// Samples are loaded CHUNK at a time before any of the chunk's outputs (which
// lag by r) are stored, so the loads of a chunk are independent; with CHUNK a
// multiple of kRing and QS fixed at compile time the ring stays in registers.
template <int QS>
__global__ void k_pass_jk(float* __restrict__ D, int m, int n, int o, int axis) {
    constexpr int CHUNK = kRing;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y;  // the other coordinate: k for axis 1, j for axis 2
    const int l = blockIdx.z;
    if (i >= m) return;
    const int64_t mn = (int64_t)m * n, sz = mn * o;
    float* base;
    int64_t stride;
    int L;
    if (axis == 1) { base = D + l * sz + i + b * mn; stride = m; L = n; }
    else { base = D + l * sz + i + (int64_t)b * m; stride = mn; L = o; }
    float ring[kRing];
    float P = 0.0f;
    for (int c0 = 0; c0 < L; c0 += CHUNK) {
        float x[CHUNK];
#pragma unroll
        for (int u = 0; u < CHUNK; u++) x[u] = (c0 + u < L) ? base[(c0 + u) * stride] : 0.0f;
#pragma unroll
        for (int u = 0; u < CHUNK; u++) {
            const int t = c0 + u;
            if (t < L) {
                P = (t == 0) ? x[u] : P + x[u];
                ring[u] = P;  // c0 is a multiple of kRing
                const int io = t - QS;
                if (io >= 0) base[io * stride] = (io <= QS) ? P : P - ring[(u - 2 * QS - 1) & (kRing - 1)];
                if (t == L - 1) {
#pragma unroll
                    for (int s2 = 0; s2 < QS; s2++)
                        base[(L - QS + s2) * stride] = P - ring[(u - 2 * QS + s2) & (kRing - 1)];
                }
            }
        }
    }
}

// The five quantisation thresholds and, around each, a window of 2^-20 relative
// width: the product y = v * RN(1/noise) is within 1.5 ulp of the correctly rounded
// quotient RN(v/noise), so a threshold whose window does not hold y compares with
// the quotient as it compares with y.
struct QuantThr {
    float t[5], lo[5], hi[5];
};

// The twelve SSC pairs (src/MINDSSCbox.h:136-140): pair l compares channel l / 2
// at the voxel's neighbour QS away along one axis (0: i, 1: j, 2: k) in direction
// kSign[l]; a neighbour outside the volume reads the voxel itself.  With QS a
// compile-time constant every offset is a constant multiple of the line and
// slice strides and each pair needs one bounds test.
template <int QS, bool LOGTHR>
__global__ void __launch_bounds__(64) k_quantise(const float* __restrict__ D, uint64_t* __restrict__ codes, int m,
                                                 int n, int o, QuantThr th) {
    constexpr int kAxis[12] = {1, 0, 1, 0, 2, 1, 2, 0, 2, 1, 2, 0};
    constexpr int kSign[12] = {-1, -1, -1, 1, -1, 1, -1, 1, -1, -1, -1, -1};
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    const int k = blockIdx.z;
    if (i >= m) return;
    const int64_t mn = (int64_t)m * n, sz = mn * o;
    const int64_t p = i + (int64_t)j * m + k * mn;
    const float* c = D + p;
    const bool lo_ok[3] = {i >= QS, j >= QS, k >= QS};
    const bool hi_ok[3] = {i + QS < m, j + QS < n, k + QS < o};
    const int64_t step[3] = {QS, (int64_t)QS * m, (int64_t)QS * mn};
    float v[12];
#pragma unroll
    for (int l = 0; l < 12; l++) {
        const int ax = kAxis[l];
        const bool ok = kSign[l] < 0 ? lo_ok[ax] : hi_ok[ax];
        const int64_t off = ok ? (kSign[l] < 0 ? -step[ax] : step[ax]) : 0;
        v[l] = __ldg(c + (l >> 1) * sz + off);
    }
    float mn_v = v[0];
#pragma unroll
    for (int l = 1; l < 12; l++) mn_v = v[l] < mn_v ? v[l] : mn_v;
    float noise = 0.0f;
#pragma unroll
    for (int l = 0; l < 12; l++) { v[l] = v[l] - mn_v; noise = noise + v[l]; }
    noise = fmaxf(__fdiv_rn(noise, 12.0f), 1e-6f);
    // The level only counts the thresholds above the correctly rounded quotient
    // RN(v / noise).  v * RN(1 / noise) is within 1.5 ulp of it (two roundings of
    // at most half an ulp each, relative 2^-24, on a quotient whose own rounding is
    // half an ulp), so unless a threshold lies within 2^-20 (relative, ~8 ulp) of
    // that product both give the same count; near a threshold the IEEE division
    // decides.  noise >= 1e-6 (fmaxf drops a NaN sum); NaN, infinite, zero and
    // tiny quotients fall on the same side of every threshold both ways.
    const float rcp = __frcp_rn(noise);
    uint64_t code = 0;
#pragma unroll
    for (int l = 0; l < 12; l++) {
        const float y = __fmul_rn(v[l], rcp);
        int lvl = 0;
        bool exact;
        if (LOGTHR) {
            // thresholds -log((c+1.5)/6), c = 0..4: c counts when c < z = 6 exp(-x) - 1.5,
            // so the level is ceil(z) clamped to [0, 5].  z from y and the fast exponential
            // is within 2^-17 of the z of the quotient and of the float thresholds; within
            // 2^-12 of an integer (or NaN) the IEEE division decides.
            const float z = __fadd_rn(__fmul_rn(6.0f, __expf(-y)), -1.5f);
            exact = !(fabsf(__fsub_rn(z, rintf(z))) >= 0x1p-12f);
            lvl = min(max((int)ceilf(z), 0), 5);
        } else {
            // y outside every threshold's window: each threshold is above or below the
            // quotient as it is above or below y; y inside a window: the IEEE division decides
            int cnt = 0;
#pragma unroll
            for (int q = 0; q < 5; q++) {
                lvl += y < th.lo[q];
                cnt += y <= th.hi[q];
            }
            exact = cnt != lvl;
        }
        if (exact) {
            const float x = __fdiv_rn(v[l], noise);
            lvl = 0;
#pragma unroll
            for (int q = 0; q < 5; q++) lvl += th.t[q] > x;
        }
        code |= (uint64_t)((1u << lvl) - 1u) << (5 * l);  // thermometer {0,1,3,7,15,31}
    }
    codes[p] = code;
}

}  // namespace

template <int QS>
static void mind_passes(const float* d_im, int m, int n, int o, const float thr[5], float* d_scratch,
                        uint64_t* d_codes, cudaStream_t s) {
    const size_t smem = (size_t)(4 * (TJ + 2 * QS) * (CH + 2 * QS + 1) + 6 * TJ * (CH + 1)) * sizeof(float);
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_pass_i<QS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_pass_i<QS><<<dim3((n + TJ - 1) / TJ, o), 6 * TJ, smem, s>>>(d_im, d_scratch, m, n, o);
    // 64 i per block: the usual volume extents are multiples of 64, so no lane idles
    k_pass_jk<QS><<<dim3((m + 63) / 64, o, 6), 64, 0, s>>>(d_scratch, m, n, o, 1);
    k_pass_jk<QS><<<dim3((m + 63) / 64, n, 6), 64, 0, s>>>(d_scratch, m, n, o, 2);
    QuantThr th;
    for (int q = 0; q < 5; q++) {
        // a window of 2^-20 (relative) on either side of the threshold
        const float a = thr[q] * (1.0f - 0x1p-20f), b = thr[q] * (1.0f + 0x1p-20f);
        th.t[q] = thr[q];
        th.lo[q] = a < b ? a : b;
        th.hi[q] = a < b ? b : a;
    }
    // the reference's thresholds -logf((c+1.5)/6) (within 2^-20): the level from one exponential
    bool logthr = true;
    for (int q = 0; q < 5; q++) {
        const double ref = -std::log((q + 1.5) / 6.0);
        logthr = logthr && std::fabs((double)thr[q] - ref) <= 0x1p-20 * ref;
    }
    if (logthr) k_quantise<QS, true><<<dim3((m + 63) / 64, n, o), 64, 0, s>>>(d_scratch, d_codes, m, n, o, th);
    else k_quantise<QS, false><<<dim3((m + 63) / 64, n, o), 64, 0, s>>>(d_scratch, d_codes, m, n, o, th);
}

cudaError_t launch_mind_ssc(const float* d_im, int m, int n, int o, int qs, const float thr[5], float* d_scratch,
                            uint64_t* d_codes, cudaStream_t s) {
    switch (qs) {
        case 1: mind_passes<1>(d_im, m, n, o, thr, d_scratch, d_codes, s); break;
        case 2: mind_passes<2>(d_im, m, n, o, thr, d_scratch, d_codes, s); break;
        case 3: mind_passes<3>(d_im, m, n, o, thr, d_scratch, d_codes, s); break;
        case 4: mind_passes<4>(d_im, m, n, o, thr, d_scratch, d_codes, s); break;
        case 5: mind_passes<5>(d_im, m, n, o, thr, d_scratch, d_codes, s); break;
        case 6: mind_passes<6>(d_im, m, n, o, thr, d_scratch, d_codes, s); break;
        case 7: mind_passes<7>(d_im, m, n, o, thr, d_scratch, d_codes, s); break;
        default: return cudaErrorInvalidValue;
    }
    count_launches(4);
    return cudaGetLastError();
}

}  // namespace deeds
