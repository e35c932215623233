// MIND-SSC descriptor on sm_103a (replaces descriptor(), src/MINDSSCbox.h:127-232).
//
// Layout in HBM: six distance channels D[l][p] (6 x m*n*o float32, context
// scratch) and the output codes C[p] (uint64).  Four launches:
//   1. pass_i: per (j,k,l) line, the shifted squared difference (imshift +
//      distances, src/MINDSSCbox.h:79-124) streamed into the i-axis box sum;
//   2. pass_j / 3. pass_k: the j- and k-axis box sums, in place;
//   4. quantise: the 12 SSC pairs -> min/mean normalisation -> 5 thresholds ->
//      thermometer code (src/MINDSSCbox.h:175-224).
// Box sums keep the reference's sequential float prefix sum along each line and
// its edge rules (src/MINDSSCbox.h:9-73): one thread owns one line and streams
// it with a lag of r, keeping the last 2r+2 prefix values in a ring.  Lines of
// the j and k passes map consecutive i to consecutive lanes (coalesced).
// Roofline: HBM-bound; per call ~ 4 B read + 6x(4 B write) (pass_i),
// 2 x 6 x 8 B (pass_j, pass_k), 6 x 4 B read + 8 B write (quantise) per voxel.
#include "common.cuh"
#include "kernels.h"

namespace deeds {

namespace {

constexpr int kRing = 16;  // supports box radius r <= 7 (2r+2 <= 16)

// Streaming box filter of one line.  get(t) yields the t-th input sample,
// put(t, v) stores the t-th output.  Inputs are consumed strictly before the
// output at the same position is stored (lag r), so in-place use is safe.
template <class Get, class Put>
__device__ __forceinline__ void box_line(int L, int r, Get get, Put put) {
    float ring[kRing];
    float P = 0.0f;
    for (int t = 0; t < L; t++) {
        const float x = get(t);
        P = (t == 0) ? x : P + x;
        ring[t & (kRing - 1)] = P;
        const int i = t - r;
        if (i >= 0) {
            if (i <= r) put(i, P);                                            // i < r+1: P[i+r]
            else put(i, P - ring[(t - 2 * r - 1) & (kRing - 1)]);           // P[i+r] - P[i-r-1]
        }
    }
    const float last = P;
    for (int i = (L - r > 0 ? L - r : 0); i < L; i++) {
        // i >= L-r: P[L-1] - P[i-r-1]  (i-r-1 >= 0 since L >= 2r+1)
        put(i, last - ring[(i - r - 1) & (kRing - 1)]);
    }
}

// Shift vectors of the six distance channels (src/MINDSSCbox.h:132-134).
__constant__ int c_dx[6] = {1, 1, -1, 0, 1, 0};
__constant__ int c_dy[6] = {1, -1, 0, -1, 0, 1};
__constant__ int c_dz[6] = {0, 0, 1, 1, 1, 1};
// The twelve SSC pairs: channel and neighbour offset (src/MINDSSCbox.h:136-140).
__constant__ int c_sx[12] = {-1, 0, -1, 0, 0, 1, 0, 0, 0, -1, 0, 0};
__constant__ int c_sy[12] = {0, -1, 0, 1, 0, 0, 0, 1, 0, 0, 0, -1};
__constant__ int c_sz[12] = {0, 0, 0, 0, -1, 0, -1, 0, -1, 0, -1, 0};

__global__ void k_pass_i(const float* __restrict__ im, float* __restrict__ D, int m, int n, int o, int qs) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    const int l = blockIdx.z;
    if (j >= n) return;
    const int64_t mn = (int64_t)m * n, sz = mn * o;
    const int dx = c_dx[l] * qs, dy = c_dy[l] * qs, dz = c_dz[l] * qs;
    const int jj = j + dx, kk = k + dz;
    const bool line_ok = jj >= 0 && jj < n && kk >= 0 && kk < o;
    const float* self = im + (int64_t)j * m + k * mn;
    const float* other = im + (int64_t)jj * m + (int64_t)kk * mn;
    float* out = D + l * sz + (int64_t)j * m + k * mn;
    box_line(m, qs,
             [&](int i) {
                 const float s = self[i];
                 const int ii = i + dy;
                 const float v = (line_ok && ii >= 0 && ii < m) ? other[ii] : s;
                 const float d = v - s;
                 return d * d;
             },
             [&](int i, float v) { out[i] = v; });
}

// In-place box pass along j (axis=1) or k (axis=2); threads over consecutive i.
__global__ void k_pass_jk(float* __restrict__ D, int m, int n, int o, int qs, int axis) {
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
    box_line(L, qs, [&](int t) { return base[t * stride]; }, [&](int t, float v) { base[t * stride] = v; });
}

__global__ void k_quantise(const float* __restrict__ D, uint64_t* __restrict__ codes, int m, int n, int o, int qs,
                           float t0, float t1, float t2, float t3, float t4) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    const int k = blockIdx.z;
    if (i >= m) return;
    const int64_t mn = (int64_t)m * n, sz = mn * o;
    const int64_t p = i + (int64_t)j * m + k * mn;
    float v[12];
#pragma unroll
    for (int l = 0; l < 12; l++) {
        const int ii = i + c_sy[l] * qs, jj = j + c_sx[l] * qs, kk = k + c_sz[l] * qs;
        const float* Dl = D + (l >> 1) * sz;
        const bool ok = ii >= 0 && ii < m && jj >= 0 && jj < n && kk >= 0 && kk < o;
        v[l] = __ldg(Dl + (ok ? ii + (int64_t)jj * m + kk * mn : p));
    }
    float mn_v = v[0];
#pragma unroll
    for (int l = 1; l < 12; l++) mn_v = v[l] < mn_v ? v[l] : mn_v;
    float noise = 0.0f;
#pragma unroll
    for (int l = 0; l < 12; l++) { v[l] = v[l] - mn_v; noise = noise + v[l]; }
    noise = fmaxf(__fdiv_rn(noise, 12.0f), 1e-6f);
    uint64_t code = 0;
#pragma unroll
    for (int l = 0; l < 12; l++) {
        const float x = __fdiv_rn(v[l], noise);
        const int lvl = (t0 > x) + (t1 > x) + (t2 > x) + (t3 > x) + (t4 > x);
        code |= (uint64_t)((1u << lvl) - 1u) << (5 * l);  // thermometer {0,1,3,7,15,31}
    }
    codes[p] = code;
}

}  // namespace

cudaError_t launch_mind_ssc(const float* d_im, int m, int n, int o, int qs, const float thr[5], float* d_scratch,
                            uint64_t* d_codes, cudaStream_t s) {
    {
        dim3 blk(128), grd((n + 127) / 128, o, 6);
        k_pass_i<<<grd, blk, 0, s>>>(d_im, d_scratch, m, n, o, qs);
    }
    {
        dim3 blk(128), grd((m + 127) / 128, o, 6);
        k_pass_jk<<<grd, blk, 0, s>>>(d_scratch, m, n, o, qs, 1);
    }
    {
        dim3 blk(128), grd((m + 127) / 128, n, 6);
        k_pass_jk<<<grd, blk, 0, s>>>(d_scratch, m, n, o, qs, 2);
    }
    {
        dim3 blk(128), grd((m + 127) / 128, n, o);
        k_quantise<<<grd, blk, 0, s>>>(d_scratch, d_codes, m, n, o, qs, thr[0], thr[1], thr[2], thr[3], thr[4]);
    }
    count_launches(4);
    return cudaGetLastError();
}

}  // namespace deeds
