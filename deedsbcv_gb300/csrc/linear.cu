// linearBCV on sm_103a (replaces the device-sized stages of src/linearBCV.cpp:
// warpAffine of src/affineLTS1.h:39-68, and the cost smoothing and per-node
// statistics of estimateAffine2, src/affineLTS1.h:91-190).  The least-trimmed-
// squares fit itself works on a few thousand points and stays on the host
// (linear_host.cpp).  Same numerics contract as the deeds kernels: IEEE float in
// source order without FMA contraction, double exactly where the reference's
// C++ promotes.
#include "common.cuh"
#include "kernels.h"

namespace deeds {

namespace {

struct Affine12 {
    float x[12];
};

// warpAffine of src/affineLTS1.h:39-68: the affine map alone; a voxel whose floor
// corner leaves [0, dim-2] on any axis is 0.
__global__ void k_lin_warp(const float* __restrict__ in, Affine12 X, float* __restrict__ out, int m, int n, int o) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i >= m) return;
    const int64_t p = i + (int64_t)j * m + (int64_t)k * m * n;
    const float fi = (float)i, fj = (float)j, fk = (float)k;
    const float y1 = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(fi, X.x[0]), __fmul_rn(fj, X.x[1])), __fmul_rn(fk, X.x[2])), X.x[3]);
    const float x1 = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(fi, X.x[4]), __fmul_rn(fj, X.x[5])), __fmul_rn(fk, X.x[6])), X.x[7]);
    const float z1 = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(fi, X.x[8]), __fmul_rn(fj, X.x[9])), __fmul_rn(fk, X.x[10])), X.x[11]);
    int x, y, z;
    float dx, dy, dz;
    split_coord(x1, x, dx);
    split_coord(y1, y, dy);
    split_coord(z1, z, dz);
    if (y < 0 || y >= m - 1 || x < 0 || x >= n - 1 || z < 0 || z >= o - 1) {
        out[p] = 0.0f;
        return;
    }
    out[p] = sample_ff(in, corners(y, x, z, m, n, o), ff_weights(dx, dy, dz), dx, dy, dz);
}

// One smoothing pass of estimateAffine2 (src/affineLTS1.h:124-158) along an axis
// of `len` nodes with node stride `stride`: the reference walks the nodes in
// index order and updates in place, so along each line
//     c'[t] = c[t] + (0.5 c[t+1] + 0.5 c'[t-1])      (double, rounded to float)
// with the neighbours clamped to the line (at t = 0 the lower neighbour is the
// node itself, read before its update).  A thread owns one (line, label) and
// walks the line; consecutive threads hold consecutive labels of the same node
// (coalesced).  blockIdx.y selects one of two volumes.
// The step in float-float (see ff_blend8 in common.cuh for the method): the
// reference evaluates E = cur + (0.5 next + 0.5 prev) with two double roundings,
// so its result is within 2^-52 S of E (S = |cur| + |next|/2 + |prev|/2); the
// float-float sum below (exact halves, exact two-sums, one float rounding of the
// low parts) is within 2^-47 S of E.  When no float midpoint lies within 2^-43 S
// of it, both round to the same float; otherwise the caller takes the double
// expression.
__device__ __forceinline__ bool smooth_step_ff(float cur, float next, float prev, float& out) {
    const float h1 = 0.5f * next, h2 = 0.5f * prev;
    const float S = fabsf(cur) + fabsf(h1) + fabsf(h2);
    if (!(S >= 0x1p-60f && S <= 0x1p+100f)) return false;  // also NaN / infinite values
    const FF s1 = ff_two_sum(h1, h2);
    const FF s2 = ff_two_sum(cur, s1.hi);
    return ff_round_safe(ff_two_sum(s2.hi, __fadd_rn(s2.lo, s1.lo)), S * 0x1p-43f, out);
}

struct SmoothLines {
    int len, stride;           // along the smoothed axis
    int a_len, a_stride;       // first other axis
    int b_stride;              // second other axis
    int64_t lines;
};

__global__ void k_lin_smooth(float* __restrict__ c0, float* __restrict__ c1, SmoothLines L, int len3) {
    float* __restrict__ c = blockIdx.y == 0 ? c0 : c1;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= L.lines * len3) return;
    const int64_t line = t / len3;
    const int lab = (int)(t - line * len3);
    const int a = (int)(line % L.a_len), b = (int)(line / L.a_len);
    const int64_t base = (int64_t)a * L.a_stride + (int64_t)b * L.b_stride;
    float* p = c + base * len3 + lab;
    const int64_t step = (int64_t)L.stride * len3;
    float cur = p[0];
    float prev = cur;  // node 0: the lower neighbour is itself, not yet updated
    for (int s = 0; s < L.len; s++) {
        const float next = s + 1 < L.len ? p[(s + 1) * step] : cur;  // upper neighbour: not yet updated
        float v;
        if (!smooth_step_ff(cur, next, prev, v)) {
            const double add = __dadd_rn(__dmul_rn(0.5, f2d(next)), __dmul_rn(0.5, f2d(prev)));
            v = __double2float_rn(__dadd_rn(f2d(cur), add));
        }
        p[s * step] = v;
        prev = v;
        cur = next;
    }
}

// Per node of a level (src/affineLTS1.h:167-206): the first minimum and its label
// of both smoothed cost volumes, the means of the fixed and moving images over
// the node's g^3 block (float sums in the reference's k, j, i order), and the
// exclusions: a mean below 5 (background) or a node within two of the grid's
// border sets the value to 1e20.  One warp per node.
__global__ void k_lin_node_stats(const float* __restrict__ c0, const float* __restrict__ c1,
                                 const float* __restrict__ fixed, const float* __restrict__ moving, int m, int n, int o,
                                 int g, int len3, float* __restrict__ minval, int* __restrict__ minind) {
    const int warps = blockDim.x >> 5;
    const int node = blockIdx.x * warps + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    const int m1 = m / g, n1 = n / g, o1 = o / g;
    const int sz1 = m1 * n1 * o1;
    if (node >= sz1) return;
    const int z1 = node / (m1 * n1), x1 = (node - z1 * m1 * n1) / m1, y1 = node - z1 * m1 * n1 - x1 * m1;
    float best[2];
    int arg[2];
#pragma unroll
    for (int v = 0; v < 2; v++) {
        const float* row = (v == 0 ? c0 : c1) + (int64_t)node * len3;
        float bv = 3.0e38f;
        int bi = 0x7fffffff;
        for (int l = lane; l < len3; l += 32) {
            const float x = row[l];
            if (x < bv) { bv = x; bi = l; }  // strictly smaller: the first index within a lane
        }
        for (int off = 16; off > 0; off >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, bv, off);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
            if (ov < bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
        }
        best[v] = bv;
        arg[v] = bi;
    }
    // lane 0: fixed-image mean, lane 1: moving-image mean
    float mean = 0.0f;
    if (lane < 2) {
        const float* im = lane == 0 ? fixed : moving;
        const int64_t mn = (int64_t)m * n;
        for (int k1 = 0; k1 < g; k1++)
            for (int j1 = 0; j1 < g; j1++) {
                const float* r = im + (int64_t)y1 * g + (int64_t)(x1 * g + j1) * m + (int64_t)(z1 * g + k1) * mn;
                for (int i1 = 0; i1 < g; i1++) mean = __fadd_rn(mean, r[i1]);
            }
        mean = __fdiv_rn(mean, (float)(g * g * g));
    }
    const float mean_f = __shfl_sync(0xffffffffu, mean, 0), mean_m = __shfl_sync(0xffffffffu, mean, 1);
    if (lane == 0) {
        if (mean_f < 5.0f) best[0] = 1e20f;
        if (mean_m < 5.0f) best[1] = 1e20f;
        if (z1 < 2 || z1 > o1 - 2 || x1 < 2 || x1 > n1 - 2 || y1 < 2 || y1 > m1 - 2) best[0] = best[1] = 1e20f;
        minval[node] = best[0];
        minval[sz1 + node] = best[1];
        minind[node] = arg[0];
        minind[sz1 + node] = arg[1];
    }
}

inline dim3 vol_grid3(int m, int n, int o, int threads) { return dim3((m + threads - 1) / threads, n, o); }

}  // namespace

cudaError_t launch_lin_warp(const float* d_in, const float* X, int m, int n, int o, float* d_out, cudaStream_t s) {
    Affine12 a;
    for (int i = 0; i < 12; i++) a.x[i] = X[i];
    k_lin_warp<<<vol_grid3(m, n, o, 128), 128, 0, s>>>(d_in, a, d_out, m, n, o);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_lin_smooth(float* d_c0, float* d_c1, int m1, int n1, int o1, int len3, cudaStream_t s) {
    const int nvol = d_c1 ? 2 : 1;
    const int64_t sz1 = (int64_t)m1 * n1 * o1;
    // y (stride 1), then x (stride m1), then z (stride m1*n1)
    const SmoothLines passes[3] = {
        {m1, 1, n1, m1, m1 * n1, sz1 / m1},
        {n1, m1, m1, 1, m1 * n1, sz1 / n1},
        {o1, m1 * n1, m1, 1, m1, sz1 / o1},
    };
    for (const SmoothLines& L : passes) {
        const int64_t threads = L.lines * len3;
        const dim3 grid((unsigned)((threads + 255) / 256), nvol);
        k_lin_smooth<<<grid, 256, 0, s>>>(d_c0, d_c1, L, len3);
        count_launches(1);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_lin_node_stats(const float* d_c0, const float* d_c1, const float* d_fixed, const float* d_moving,
                                  int m, int n, int o, int g, int len3, float* d_minval, int* d_minind,
                                  cudaStream_t s) {
    const int sz1 = (m / g) * (n / g) * (o / g);
    k_lin_node_stats<<<(sz1 + 3) / 4, 128, 0, s>>>(d_c0, d_c1, d_fixed, d_moving, m, n, o, g, len3, d_minval,
                                                    d_minind);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace deeds
