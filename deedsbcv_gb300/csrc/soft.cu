// Differentiable soft-min deeds level on sm_103a: forward and hand-written adjoint.
//
// There is no counterpart in the reference; the form relaxes one level of
// src/deedsBCV0.cpp:238-306 so that it is differentiable in both images and in
// the regularisation weight alpha.  With a zero prior field:
//   descriptor  s_l(p) = 6 exp(-(v_l - min v)/max(mean(v - min v), 1e-6)), v_l the
//               12 box-filtered self-similarity distances of MIND-SSC
//               (src/MINDSSCbox.h:127-201; the reference quantises exactly this
//               quantity: code = #{c : s > c + 1.5});
//   cost        C[c][l] = alpha1 sum_{samples p of c} sum_ch phi(sF_ch(p) - sM_ch(p + d(l))),
//               phi(x) = sqrt(x^2 + eps^2) - eps, alpha1 = 0.5 (g/(alpha q))/maxsamp,
//               sampling and clamp-to-edge of src/dataCostD.h:141-200;
//   upward      B_c = C_c + sum_children (M_k - min M_k),
//               M_c(lp) = -tau LSE_l(-(e_c B_c(l) + |lab(l) - lab(lp)|^2)/tau)
//               (src/regularisation.h:190-238 with min -> soft-min);
//   downward    log p_root = log softmax(-B_root/tau),
//               log p_c(l) = -e_c B_c(l)/tau + LSE_lp(log p_p(lp) + M_c(lp)/tau - |lab(l)-lab(lp)|^2/tau);
//   output      E_c = sum_l p_c(l) d(l), d(l) = (label - hw) q per axis (u = x, v = y, w = z).
//
// Both label-space transforms are the same operator S(x)(b) = LSE_a(x(a) - |a-b|^2/tau)
// over the len^3 label grid.  Because |a-b|^2 is a sum over the three axes, S is
// three one-axis passes in the log domain (len^4 terms per pass instead of len^6),
// each pass max-shifted so that nothing under- or overflows.  Its adjoint is three
// passes back, each weighting the incoming gradient with exp(in(a) - |a-b|^2/tau -
// out(b)) <= 1.  One CTA owns one tree node; its label vectors and the pass
// intermediates live in shared memory.  Tree nodes are processed one breadth level
// per launch (children before parents upward, parents before children downward).
//
// Backward recomputes the forward sweeps from the inputs (no message tensors are
// kept between forward and backward) and then runs, per breadth level:
//   marginal adjoint (leaves to root): h_c = dL/dlog p_c = (gE_c . d) p_c + sum_children R_k;
//       Bbar_c = -e_c h_c/tau (root: -(h - p sum h)/tau); R_c = S^T h_c (w.r.t. S's input);
//   message adjoint (root to leaves): Mbar_c = R_c/tau + Bbar_parent;
//       Bbar_c += e_c S^T(Mbar_c) (S taken at -e_c B_c/tau); cbar_c = Bbar_c;
// then the cost, descriptor, box-filter and squared-difference adjoints.  The min
// subtracted from each message shifts B_parent by a constant to which the marginals
// are invariant, so it carries no gradient.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace deeds {

namespace {

__constant__ int s_dx[6] = {1, 1, -1, 0, 1, 0};
__constant__ int s_dy[6] = {1, -1, 0, -1, 0, 1};
__constant__ int s_dz[6] = {0, 0, 1, 1, 1, 1};
__constant__ int s_sx[12] = {-1, 0, -1, 0, 0, 1, 0, 0, 0, -1, 0, 0};
__constant__ int s_sy[12] = {0, -1, 0, 1, 0, 0, 0, 1, 0, 0, 0, -1};
__constant__ int s_sz[12] = {0, 0, 0, 0, -1, 0, -1, 0, -1, 0, -1, 0};

__device__ __forceinline__ bool inside(int i, int j, int k, int m, int n, int o) {
    return i >= 0 && i < m && j >= 0 && j < n && k >= 0 && k < o;
}

inline unsigned blocks_for(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// ---------------------------------------------------------------------------
// Descriptor

// w_l(p) = (I(p + t_l) - I(p))^2, 0 where p + t_l leaves the volume (the reference's
// imshift keeps the voxel itself there, src/MINDSSCbox.h:79-124)
__global__ void k_soft_sqdiff(const float* __restrict__ im, float* __restrict__ w, int m, int n, int o, int qs) {
    const int64_t sz = (int64_t)m * n * o;
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= sz) return;
    const int i = (int)(p % m), j = (int)((p / m) % n), k = (int)(p / ((int64_t)m * n));
    const float c = im[p];
#pragma unroll
    for (int l = 0; l < 6; l++) {
        const int ii = i + s_dy[l] * qs, jj = j + s_dx[l] * qs, kk = k + s_dz[l] * qs;
        float d = 0.0f;
        if (inside(ii, jj, kk, m, n, o)) d = im[ii + (int64_t)jj * m + (int64_t)kk * m * n] - c;
        w[l * sz + p] = d * d;
    }
}

// Windowed sum over [max(0,i-r), min(L-1,i+r)] along one axis, out of place, summed
// directly (no prefix-sum differences, whose cancellation would cost the soft
// descriptor its float32 accuracy).  The operator is symmetric, so the same
// kernel is its own adjoint.  Grid: x over i, y over j (32 x 8 blocks), z over
// (k, channel): no index divisions by runtime sizes.
// R > 0: compile-time radius (window loads unrolled and issued together); R = 0:
// the radius r at run time.
template <int R>
__global__ void k_soft_box(const float* __restrict__ in, float* __restrict__ out, int m, int n, int o, int r, int axis) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= m || j >= n) return;
    const int k = blockIdx.z % o, ch = blockIdx.z / o;
    const int64_t mn = (int64_t)m * n;
    const int64_t p = (int64_t)ch * mn * o + i + (int64_t)j * m + (int64_t)k * mn;
    int L, c;
    int64_t stride;
    if (axis == 0) { L = m; stride = 1; c = i; }
    else if (axis == 1) { L = n; stride = m; c = j; }
    else { L = o; stride = mn; c = k; }
    const float* x = in + (p - (int64_t)c * stride);
    float acc = 0.0f;
    if (R > 0) {
        float v[2 * R + 1];
#pragma unroll
        for (int d = -R; d <= R; d++) {
            const int a = c + d;
            v[d + R] = (a >= 0 && a < L) ? __ldg(x + a * stride) : 0.0f;
        }
#pragma unroll
        for (int d = 0; d <= 2 * R; d++) acc += v[d];
    } else {
        const int a0 = max(0, c - r), a1 = min(L - 1, c + r);
        for (int a = a0; a <= a1; a++) acc += x[a * stride];
    }
    out[p] = acc;
}

struct DescPoint {
    float v[12];
    int64_t q[12];
};

__device__ __forceinline__ void gather_desc(const float* __restrict__ d, int64_t p, int m, int n, int o, int qs,
                                            DescPoint& dp) {
    const int64_t sz = (int64_t)m * n * o;
    const int i = (int)(p % m), j = (int)((p / m) % n), k = (int)(p / ((int64_t)m * n));
#pragma unroll
    for (int l = 0; l < 12; l++) {
        const int ii = i + s_sy[l] * qs, jj = j + s_sx[l] * qs, kk = k + s_sz[l] * qs;
        dp.q[l] = inside(ii, jj, kk, m, n, o) ? ii + (int64_t)jj * m + (int64_t)kk * m * n : p;
        dp.v[l] = d[(l >> 1) * sz + dp.q[l]];
    }
}

// soft descriptor s (12 x sz) from the box-filtered channels d (6 x sz)
__global__ void k_soft_desc(const float* __restrict__ d, float* __restrict__ s, int m, int n, int o, int qs) {
    const int64_t sz = (int64_t)m * n * o;
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= sz) return;
    DescPoint dp;
    gather_desc(d, p, m, n, o, qs, dp);
    float mn = dp.v[0];
#pragma unroll
    for (int l = 1; l < 12; l++) mn = fminf(mn, dp.v[l]);
    float sum = 0.0f;
#pragma unroll
    for (int l = 0; l < 12; l++) sum += dp.v[l] - mn;
    const float noise = fmaxf(sum / 12.0f, 1e-6f);
#pragma unroll
    for (int l = 0; l < 12; l++) s[l * sz + p] = 6.0f * expf(-(dp.v[l] - mn) / noise);
}

// adjoint of k_soft_desc: sbar (12 x sz) -> dbar (6 x sz), accumulated with atomics
// (the twelve gathers of a voxel hit neighbours that other voxels also gather)
__global__ void k_soft_desc_adj(const float* __restrict__ d, const float* __restrict__ sbar, float* __restrict__ dbar,
                                int m, int n, int o, int qs) {
    const int64_t sz = (int64_t)m * n * o;
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= sz) return;
    DescPoint dp;
    gather_desc(d, p, m, n, o, qs, dp);
    float mn = dp.v[0];
    int am = 0;
#pragma unroll
    for (int l = 1; l < 12; l++)
        if (dp.v[l] < mn) { mn = dp.v[l]; am = l; }
    float sum = 0.0f;
#pragma unroll
    for (int l = 0; l < 12; l++) sum += dp.v[l] - mn;
    const bool clamped = sum / 12.0f < 1e-6f;
    const float noise = fmaxf(sum / 12.0f, 1e-6f);
    // x_l = (v_l - mn)/noise, noise = sum_l (v_l - mn)/12 unless clamped, mn = v_am
    float vb[12], nbar = 0.0f;
#pragma unroll
    for (int l = 0; l < 12; l++) {
        const float x = (dp.v[l] - mn) / noise;
        vb[l] = -6.0f * expf(-x) * sbar[l * sz + p];  // dL/dx_l
        nbar -= vb[l] * x / noise;
    }
    float tot = 0.0f;
#pragma unroll
    for (int l = 0; l < 12; l++) {
        vb[l] = vb[l] / noise + (clamped ? 0.0f : nbar / 12.0f);
        tot += vb[l];
    }
#pragma unroll
    for (int l = 0; l < 12; l++) atomicAdd(dbar + (l >> 1) * sz + dp.q[l], l == am ? vb[l] - tot : vb[l]);
}

// adjoint of k_soft_sqdiff: wbar (6 x sz) -> imbar (accumulated)
__global__ void k_soft_sqdiff_adj(const float* __restrict__ im, const float* __restrict__ wbar,
                                  float* __restrict__ imbar, int m, int n, int o, int qs) {
    const int64_t sz = (int64_t)m * n * o;
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= sz) return;
    const int i = (int)(p % m), j = (int)((p / m) % n), k = (int)(p / ((int64_t)m * n));
    const float c = im[p];
    float self = 0.0f;
#pragma unroll
    for (int l = 0; l < 6; l++) {
        const int ii = i + s_dy[l] * qs, jj = j + s_dx[l] * qs, kk = k + s_dz[l] * qs;
        if (inside(ii, jj, kk, m, n, o)) {
            const int64_t t = ii + (int64_t)jj * m + (int64_t)kk * m * n;
            const float gr = 2.0f * (im[t] - c) * wbar[l * sz + p];
            atomicAdd(imbar + t, gr);
            self -= gr;
        }
    }
    atomicAdd(imbar + p, self);
}

// ---------------------------------------------------------------------------
// Cost

// 4-byte asynchronous global->shared copies (cp.async, sm_80+): a thread issues all
// its staging copies back to back and waits once, instead of one load latency per
// element.  The caller waits with cp_async_wait_all() and then a block barrier.
__device__ __forceinline__ void cp_async4(float* smem_dst, const float* gsrc) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

struct SoftGeom {
    int m, n, o, g, hw, q, len, len3, m1, n1, o1, S, nx, nsamp;
    float alpha1, eps;
};

__device__ __forceinline__ float phi_grad(float x, float eps) { return x * rsqrtf(x * x + eps * eps); }

// C[c][l]: one CTA per node, the node's fixed samples in shared memory, threads over labels
__global__ void k_soft_cost(const float* __restrict__ sF, const float* __restrict__ sM, float* __restrict__ cost,
                            SoftGeom G) {
    extern __shared__ float fs[];  // [nsamp][12]
    const int node = blockIdx.x;
    const int y = node % G.m1, x = (node / G.m1) % G.n1, z = node / (G.m1 * G.n1);
    const int64_t mn = (int64_t)G.m * G.n, sz = mn * G.o;
    for (int e = threadIdx.x; e < G.nsamp * 12; e += blockDim.x) {
        const int c = e % 12, s = e / 12;
        const int ii = s % G.g, jj = (s / G.g) % G.nx, kk = s / (G.g * G.nx);
        const int64_t p = (y * G.g + ii) + (int64_t)(x * G.g + jj * G.S) * G.m + (int64_t)(z * G.g + kk * G.S) * mn;
        fs[e] = sF[c * sz + p];
    }
    __syncthreads();
    for (int l = threadIdx.x; l < G.len3; l += blockDim.x) {
        const int dy = (l % G.len - G.hw) * G.q, dx = ((l / G.len) % G.len - G.hw) * G.q,
                  dz = (l / (G.len * G.len) - G.hw) * G.q;
        float acc = 0.0f;
        int s = 0;
        for (int kk = 0; kk < G.nx; kk++) {
            const int qk = clampi(z * G.g + kk * G.S + dz, 0, G.o - 1);
            for (int jj = 0; jj < G.nx; jj++) {
                const int qj = clampi(x * G.g + jj * G.S + dx, 0, G.n - 1);
                for (int ii = 0; ii < G.g; ii++, s++) {
                    const int qi = clampi(y * G.g + ii + dy, 0, G.m - 1);
                    const float* mv = sM + qi + (int64_t)qj * G.m + (int64_t)qk * mn;
                    const float* fv = fs + s * 12;
#pragma unroll
                    for (int c = 0; c < 12; c++) {
                        const float dl = fv[c] - __ldg(mv + c * sz);
                        acc += sqrtf(dl * dl + G.eps * G.eps) - G.eps;
                    }
                }
            }
        }
        cost[(int64_t)node * G.len3 + l] = G.alpha1 * acc;
    }
}

// Adjoint of the cost w.r.t. the fixed descriptor (one CTA per node, one thread per
// (sample, channel); samples of different nodes are disjoint, so plain stores) and
// dot = sum(cbar * C) for the alpha gradient (C = alpha1 f, alpha1 ~ 1/alpha,
// dL/dalpha = -dot/alpha).
__global__ void k_soft_cost_adj_fixed(const float* __restrict__ sF, const float* __restrict__ sM,
                                      const float* __restrict__ cbar, const float* __restrict__ cost,
                                      float* __restrict__ sFbar, double* __restrict__ dot, SoftGeom G) {
    const int node = blockIdx.x;
    const int y = node % G.m1, x = (node / G.m1) % G.n1, z = node / (G.m1 * G.n1);
    const int64_t mn = (int64_t)G.m * G.n, sz = mn * G.o;
    const float* cb = cbar + (int64_t)node * G.len3;
    const float* cn = cost + (int64_t)node * G.len3;
    // The level is invariant to adding a constant to one node's costs, so the exact
    // cbar sums to zero over labels and sum(cbar * C) = sum(cbar * (C - mean C)); the
    // centred form keeps float32 rounding in cbar from being amplified by |mean C|.
    __shared__ double red[32];
    double csum = 0.0;
    for (int l = threadIdx.x; l < G.len3; l += blockDim.x) csum += (double)cn[l];
    for (int off = 16; off > 0; off >>= 1) csum += __shfl_xor_sync(0xffffffffu, csum, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = csum;
    __syncthreads();
    double cmean = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) cmean += red[w];
    cmean /= (double)G.len3;
    double part = 0.0;
    for (int l = threadIdx.x; l < G.len3; l += blockDim.x) part += (double)cb[l] * ((double)cn[l] - cmean);
    for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(dot, part);
    for (int e = threadIdx.x; e < G.nsamp * 12; e += blockDim.x) {
        const int c = e % 12, s = e / 12;
        const int ii = s % G.g, jj = (s / G.g) % G.nx, kk = s / (G.g * G.nx);
        const int pi = y * G.g + ii, pj = x * G.g + jj * G.S, pk = z * G.g + kk * G.S;
        const int64_t p = pi + (int64_t)pj * G.m + (int64_t)pk * mn;
        const float f = sF[c * sz + p];
        const float* mc = sM + c * sz;
        float gF = 0.0f;
        int l = 0;
        for (int lz = 0; lz < G.len; lz++) {
            const int qk = clampi(pk + (lz - G.hw) * G.q, 0, G.o - 1);
            for (int lx = 0; lx < G.len; lx++) {
                const int qj = clampi(pj + (lx - G.hw) * G.q, 0, G.n - 1);
                const float* row = mc + (int64_t)qj * G.m + (int64_t)qk * mn;
                for (int ly = 0; ly < G.len; ly++, l++) {
                    const int qi = clampi(pi + (ly - G.hw) * G.q, 0, G.m - 1);
                    gF += cb[l] * phi_grad(f - row[qi], G.eps);
                }
            }
        }
        sFbar[c * sz + p] = G.alpha1 * gF;
    }
}

// Range of p along one axis with clamp(p + d, 0, dim-1) == qv, intersected with the
// node-covered extent [0, cover) (empty when lo > hi).
__device__ __forceinline__ void preimage(int qv, int d, int dim, int cover, int& lo, int& hi) {
    lo = qv == 0 ? 0 : qv - d;
    hi = qv == dim - 1 ? dim - 1 : qv - d;
    if (qv == 0) hi = min(hi, -d);
    if (qv == dim - 1) lo = max(lo, dim - 1 - d);
    lo = max(lo, 0);
    hi = min(hi, cover - 1);
}

// Adjoint of the cost w.r.t. the moving descriptor as a gather (no atomics): one
// thread per moving voxel q (all 12 channels), over the labels and the samples p
// whose clamped displaced position is q.
__global__ void k_soft_cost_adj_moving(const float* __restrict__ sF, const float* __restrict__ sM,
                                       const float* __restrict__ cbar, float* __restrict__ sMbar, SoftGeom G) {
    const int64_t mn = (int64_t)G.m * G.n, sz = mn * G.o;
    const int64_t qv = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (qv >= sz) return;
    const int qi = (int)(qv % G.m), qj = (int)((qv / G.m) % G.n), qk = (int)(qv / mn);
    float mq[12], acc[12];
#pragma unroll
    for (int c = 0; c < 12; c++) {
        mq[c] = sM[c * sz + qv];
        acc[c] = 0.0f;
    }
    const int ci = G.m1 * G.g, cj = G.n1 * G.g, ck = G.o1 * G.g;
    for (int lz = 0; lz < G.len; lz++) {
        int k0, k1;
        preimage(qk, (lz - G.hw) * G.q, G.o, ck, k0, k1);
        for (int pk = k0; pk <= k1; pk++) {
            if ((pk % G.g) % G.S) continue;
            for (int lx = 0; lx < G.len; lx++) {
                int j0, j1;
                preimage(qj, (lx - G.hw) * G.q, G.n, cj, j0, j1);
                for (int pj = j0; pj <= j1; pj++) {
                    if ((pj % G.g) % G.S) continue;
                    const int nbase = (pj / G.g) * G.m1 + (pk / G.g) * G.m1 * G.n1;
                    const int lbase = lx * G.len + lz * G.len * G.len;
                    for (int ly = 0; ly < G.len; ly++) {
                        int i0, i1;
                        preimage(qi, (ly - G.hw) * G.q, G.m, ci, i0, i1);
                        for (int pi = i0; pi <= i1; pi++) {
                            const float cb = __ldg(cbar + (int64_t)(nbase + pi / G.g) * G.len3 + lbase + ly);
                            const float* fp = sF + pi + (int64_t)pj * G.m + (int64_t)pk * mn;
#pragma unroll
                            for (int c = 0; c < 12; c++) acc[c] += cb * phi_grad(__ldg(fp + c * sz) - mq[c], G.eps);
                        }
                    }
                }
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 12; c++) sMbar[c * sz + qv] = -G.alpha1 * acc[c];
}

// The same gather with the grid spacing, label width and quantisation fixed at
// compile time (the row-form level shapes): the label and sample loops unroll
// and the node and lattice arithmetic uses constants.
template <int G_, int LEN_, int Q_>
__global__ void __launch_bounds__(128) k_soft_cost_adj_moving_t(const float* __restrict__ sF,
                                                               const float* __restrict__ sM,
                                                               const float* __restrict__ cbar,
                                                               float* __restrict__ sMbar, SoftGeom G) {
    constexpr int S = G_ > 4 ? 2 : 1, HW = (LEN_ - 1) / 2, LEN3 = LEN_ * LEN_ * LEN_;
    const int64_t mn = (int64_t)G.m * G.n, sz = mn * G.o;
    const int64_t qv = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (qv >= sz) return;
    const int qi = (int)(qv % G.m), qj = (int)((qv / G.m) % G.n), qk = (int)(qv / mn);
    float mq[12], acc[12];
#pragma unroll
    for (int c = 0; c < 12; c++) {
        mq[c] = sM[c * sz + qv];
        acc[c] = 0.0f;
    }
    const int ci = G.m1 * G_, cj = G.n1 * G_, ck = G.o1 * G_;
    const float eps = G.eps;
    constexpr int R = HW * Q_;
    // away from the y faces every label has exactly one y preimage, qi - dy, inside
    // the node-covered extent: a straight-line path whose loads can be issued together
    const bool yint = qi >= (R > 1 ? R : 1) && qi <= min(ci - 1 - R, G.m - 2);
    for (int lz = 0; lz < LEN_; lz++) {
        int k0, k1;
        preimage(qk, (lz - HW) * Q_, G.o, ck, k0, k1);
        for (int pk = k0; pk <= k1; pk++) {
            if (S > 1 && (pk % G_) % S) continue;
            for (int lx = 0; lx < LEN_; lx++) {
                int j0, j1;
                preimage(qj, (lx - HW) * Q_, G.n, cj, j0, j1);
                for (int pj = j0; pj <= j1; pj++) {
                    if (S > 1 && (pj % G_) % S) continue;
                    const int nbase = (pj / G_) * G.m1 + (pk / G_) * G.m1 * G.n1;
                    const float* cbl = cbar + (int64_t)(lx * LEN_ + lz * LEN_ * LEN_);
                    const float* fpk = sF + (int64_t)pj * G.m + (int64_t)pk * mn;
                    if (yint) {
                        float cbv[LEN_];
#pragma unroll
                        for (int ly = 0; ly < LEN_; ly++) {
                            const int pi = qi - (ly - HW) * Q_;
                            cbv[ly] = __ldg(cbl + (int64_t)(nbase + pi / G_) * LEN3 + ly);
                        }
#pragma unroll
                        for (int ly = 0; ly < LEN_; ly++) {
                            const float* fp = fpk + qi - (ly - HW) * Q_;
#pragma unroll
                            for (int c = 0; c < 12; c++)
                                acc[c] += cbv[ly] * phi_grad(__ldg(fp + c * sz) - mq[c], eps);
                        }
                    } else {
                        for (int ly = 0; ly < LEN_; ly++) {
                            int i0, i1;
                            preimage(qi, (ly - HW) * Q_, G.m, ci, i0, i1);
                            for (int pi = i0; pi <= i1; pi++) {
                                const float cb = __ldg(cbl + (int64_t)(nbase + pi / G_) * LEN3 + ly);
                                const float* fp = fpk + pi;
#pragma unroll
                                for (int c = 0; c < 12; c++)
                                    acc[c] += cb * phi_grad(__ldg(fp + c * sz) - mq[c], eps);
                            }
                        }
                    }
                }
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 12; c++) sMbar[c * sz + qv] = -G.alpha1 * acc[c];
}

template <int G_, int LEN_, int Q_>
static cudaError_t run_adj_moving_t(const SoftGeom& G, const float* sF, const float* sM, const float* cbar,
                                    float* sMbar, cudaStream_t st) {
    const int64_t sz = (int64_t)G.m * G.n * G.o;
    k_soft_cost_adj_moving_t<G_, LEN_, Q_><<<(unsigned)((sz + 127) / 128), 128, 0, st>>>(sF, sM, cbar, sMbar, G);
    return cudaSuccess;
}

// ---------------------------------------------------------------------------
// Halo form of the cost and its adjoint.  The moving descriptor values that one
// node's samples reach under every label form one box (the node block grown by
// hw*q on each side, clipped to the volume: the reference's clamp-to-edge maps
// every displaced position into it).  The box of a group of channels is staged
// in shared memory with coalesced loads, so the len^3 x samples x channels terms
// read shared memory only.  For nodes whose box is not clipped the displaced
// position is a per-sample base plus a per-label offset; clipped (border) nodes
// clamp per axis.

struct Halo {
    int y0, x0, z0, HY, HX, HZ, H3;
    bool interior;
};

__device__ __forceinline__ Halo node_halo(const SoftGeom& G, int y, int x, int z) {
    const int R = G.hw * G.q;
    const int ylo = y * G.g - R, yhi = y * G.g + G.g - 1 + R;
    const int xlo = x * G.g - R, xhi = x * G.g + G.g - 1 + R;
    const int zlo = z * G.g - R, zhi = z * G.g + G.g - 1 + R;
    Halo h;
    h.y0 = max(0, ylo); h.HY = min(G.m - 1, yhi) - h.y0 + 1;
    h.x0 = max(0, xlo); h.HX = min(G.n - 1, xhi) - h.x0 + 1;
    h.z0 = max(0, zlo); h.HZ = min(G.o - 1, zhi) - h.z0 + 1;
    h.H3 = h.HY * h.HX * h.HZ;
    h.interior = ylo >= 0 && yhi < G.m && xlo >= 0 && xhi < G.n && zlo >= 0 && zhi < G.o;
    return h;
}

__device__ __forceinline__ int label_dy(const SoftGeom& G, int l) { return (l % G.len - G.hw) * G.q; }
__device__ __forceinline__ int label_dx(const SoftGeom& G, int l) { return ((l / G.len) % G.len - G.hw) * G.q; }
__device__ __forceinline__ int label_dz(const SoftGeom& G, int l) { return (l / (G.len * G.len) - G.hw) * G.q; }

// sample s of node (y,x,z): voxel coordinates
__device__ __forceinline__ void sample_pos(const SoftGeom& G, int y, int x, int z, int s, int& py, int& px, int& pz) {
    py = y * G.g + s % G.g;
    px = x * G.g + ((s / G.g) % G.nx) * G.S;
    pz = z * G.g + (s / (G.g * G.nx)) * G.S;
}

__device__ __forceinline__ int halo_clamped(const SoftGeom& G, const Halo& h, int py, int px, int pz, int l) {
    const int a = clampi(py + label_dy(G, l), 0, G.m - 1) - h.y0;
    const int b = clampi(px + label_dx(G, l), 0, G.n - 1) - h.x0;
    const int c = clampi(pz + label_dz(G, l), 0, G.o - 1) - h.z0;
    return a + h.HY * (b + h.HX * c);
}

// Stage channels [c0, c0+CG) of the node's halo (coalesced along y).
__device__ __forceinline__ void stage_halo(const SoftGeom& G, const Halo& h, const float* __restrict__ vol, int c0,
                                           int CG, float* hv) {
    const int64_t mn = (int64_t)G.m * G.n, sz = mn * G.o;
    for (int e = threadIdx.x; e < CG * h.H3; e += blockDim.x) {
        const int c = e / h.H3, r = e % h.H3;
        const int a = r % h.HY, b = (r / h.HY) % h.HX, cc = r / (h.HY * h.HX);
        hv[e] = vol[(int64_t)(c0 + c) * sz + (h.y0 + a) + (int64_t)(h.x0 + b) * G.m + (int64_t)(h.z0 + cc) * mn];
    }
}

constexpr int kHaloLPT = 3;  // labels per thread in the halo cost kernel (len^3 <= 3 * 512)

// C[node][l] from shared-memory halos; threads own labels, CG channels per stage.
__global__ void __launch_bounds__(512) k_soft_cost_halo(const float* __restrict__ sF, const float* __restrict__ sM,
                                                        float* __restrict__ cost, SoftGeom G, int CG, int H3max) {
    extern __shared__ float sh[];
    const int node = blockIdx.x;
    const int y = node % G.m1, x = (node / G.m1) % G.n1, z = node / (G.m1 * G.n1);
    const Halo h = node_halo(G, y, x, z);
    const int64_t mn = (int64_t)G.m * G.n, sz = mn * G.o;
    float* hv = sh;                                             // [CG][H3]
    float* fsm = sh + (size_t)CG * H3max;                       // [CG][nsamp]
    int* loff = reinterpret_cast<int*>(fsm + CG * G.nsamp);     // [len3]
    int* sb = loff + G.len3;                                    // [nsamp]
    for (int l = threadIdx.x; l < G.len3; l += blockDim.x)
        loff[l] = label_dy(G, l) + h.HY * (label_dx(G, l) + h.HX * label_dz(G, l));
    for (int s = threadIdx.x; s < G.nsamp; s += blockDim.x) {
        int py, px, pz;
        sample_pos(G, y, x, z, s, py, px, pz);
        sb[s] = (py - h.y0) + h.HY * ((px - h.x0) + h.HX * (pz - h.z0));
    }
    float acc[kHaloLPT];
#pragma unroll
    for (int k = 0; k < kHaloLPT; k++) acc[k] = 0.0f;
    const float eps2 = G.eps * G.eps;
    for (int c0 = 0; c0 < 12; c0 += CG) {
        __syncthreads();
        stage_halo(G, h, sM, c0, CG, hv);
        for (int e = threadIdx.x; e < CG * G.nsamp; e += blockDim.x) {
            const int c = e / G.nsamp, s = e % G.nsamp;
            int py, px, pz;
            sample_pos(G, y, x, z, s, py, px, pz);
            fsm[e] = sF[(int64_t)(c0 + c) * sz + py + (int64_t)px * G.m + (int64_t)pz * mn];
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kHaloLPT; k++) {
            const int l = threadIdx.x + k * blockDim.x;
            if (l >= G.len3) break;
            float a = acc[k];
            if (h.interior) {
                const int lo = loff[l];
                for (int s = 0; s < G.nsamp; s++) {
                    const int base = sb[s] + lo;
                    for (int c = 0; c < CG; c++) {
                        const float d = fsm[c * G.nsamp + s] - hv[c * h.H3 + base];
                        const float x2 = d * d + eps2;
                        a += x2 * rsqrtf(x2);
                    }
                }
            } else {
                for (int s = 0; s < G.nsamp; s++) {
                    int py, px, pz;
                    sample_pos(G, y, x, z, s, py, px, pz);
                    const int base = halo_clamped(G, h, py, px, pz, l);
                    for (int c = 0; c < CG; c++) {
                        const float d = fsm[c * G.nsamp + s] - hv[c * h.H3 + base];
                        const float x2 = d * d + eps2;
                        a += x2 * rsqrtf(x2);
                    }
                }
            }
            acc[k] = a;
        }
    }
#pragma unroll
    for (int k = 0; k < kHaloLPT; k++) {
        const int l = threadIdx.x + k * blockDim.x;
        if (l < G.len3) cost[(int64_t)node * G.len3 + l] = G.alpha1 * (acc[k] - (float)(12 * G.nsamp) * G.eps);
    }
}

// Adjoint of the cost from shared-memory halos: threads own (channel, sample)
// items and walk the labels; each term's gradient goes to the fixed sample (a
// register) and, through a shared-memory atomic, to the halo position it read;
// the halo gradients are then added to the moving descriptor's gradient
// (neighbouring nodes' halos overlap).  Also dot = sum(cbar * C) for alpha.
__global__ void __launch_bounds__(256) k_soft_cost_adj_halo(const float* __restrict__ sF,
                                                            const float* __restrict__ sM,
                                                            const float* __restrict__ cbar,
                                                            const float* __restrict__ cost, float* __restrict__ sFbar,
                                                            float* __restrict__ sMbar, double* __restrict__ dot,
                                                            SoftGeom G, int CG, int H3max) {
    extern __shared__ float sh[];
    __shared__ double red[32];
    const int node = blockIdx.x;
    const int y = node % G.m1, x = (node / G.m1) % G.n1, z = node / (G.m1 * G.n1);
    const Halo h = node_halo(G, y, x, z);
    const int64_t mn = (int64_t)G.m * G.n, sz = mn * G.o;
    float* hv = sh;                                        // [CG][H3]
    float* hg = sh + (size_t)CG * H3max;                   // [CG][H3]
    float* cb = hg + (size_t)CG * H3max;                   // [len3]
    int* loff = reinterpret_cast<int*>(cb + G.len3);       // [len3]
    int* sb = loff + G.len3;                               // [nsamp]
    const float* cbn = cbar + (int64_t)node * G.len3;
    const float* cn = cost + (int64_t)node * G.len3;
    // alpha: centred dot product (the exact cbar sums to zero over labels)
    double csum = 0.0;
    for (int l = threadIdx.x; l < G.len3; l += blockDim.x) {
        csum += (double)cn[l];
        cb[l] = cbn[l];
        loff[l] = label_dy(G, l) + h.HY * (label_dx(G, l) + h.HX * label_dz(G, l));
    }
    for (int off = 16; off > 0; off >>= 1) csum += __shfl_xor_sync(0xffffffffu, csum, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = csum;
    for (int s = threadIdx.x; s < G.nsamp; s += blockDim.x) {
        int py, px, pz;
        sample_pos(G, y, x, z, s, py, px, pz);
        sb[s] = (py - h.y0) + h.HY * ((px - h.x0) + h.HX * (pz - h.z0));
    }
    __syncthreads();
    double cmean = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) cmean += red[w];
    cmean /= (double)G.len3;
    double part = 0.0;
    for (int l = threadIdx.x; l < G.len3; l += blockDim.x) part += (double)cb[l] * ((double)cn[l] - cmean);
    for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(dot, part);
    const float eps2 = G.eps * G.eps;
    for (int c0 = 0; c0 < 12; c0 += CG) {
        __syncthreads();
        stage_halo(G, h, sM, c0, CG, hv);
        for (int e = threadIdx.x; e < CG * h.H3; e += blockDim.x) hg[e] = 0.0f;
        __syncthreads();
        for (int item = threadIdx.x; item < CG * G.nsamp; item += blockDim.x) {
            const int c = item / G.nsamp, s = item % G.nsamp;
            int py, px, pz;
            sample_pos(G, y, x, z, s, py, px, pz);
            const int64_t p = py + (int64_t)px * G.m + (int64_t)pz * mn;
            const float f = sF[(int64_t)(c0 + c) * sz + p];
            const float* hvc = hv + c * h.H3;
            float* hgc = hg + c * h.H3;
            float gF = 0.0f;
            if (h.interior) {
                const int base = sb[s];
                for (int l = 0; l < G.len3; l++) {
                    const int idx = base + loff[l];
                    const float d = f - hvc[idx];
                    const float gr = cb[l] * d * rsqrtf(d * d + eps2);
                    gF += gr;
                    atomicAdd(hgc + idx, -gr);
                }
            } else {
                for (int l = 0; l < G.len3; l++) {
                    const int idx = halo_clamped(G, h, py, px, pz, l);
                    const float d = f - hvc[idx];
                    const float gr = cb[l] * d * rsqrtf(d * d + eps2);
                    gF += gr;
                    atomicAdd(hgc + idx, -gr);
                }
            }
            sFbar[(int64_t)(c0 + c) * sz + p] = G.alpha1 * gF;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < CG * h.H3; e += blockDim.x) {
            const float v = hg[e];
            if (v == 0.0f) continue;
            const int c = e / h.H3, r = e % h.H3;
            const int a = r % h.HY, b = (r / h.HY) % h.HX, cc = r / (h.HY * h.HX);
            atomicAdd(sMbar + (int64_t)(c0 + c) * sz + (h.y0 + a) + (int64_t)(h.x0 + b) * G.m +
                          (int64_t)(h.z0 + cc) * mn,
                      G.alpha1 * v);
        }
    }
}

// Column form of the two halo kernels, for compile-time grid spacing, label width
// and quantisation.  Each node stages a full NA^3 box (NA = g + 2hw*q) of the
// moving descriptor whose entry (a, b, c) holds the voxel at the clamped
// coordinates (y*g - hw*q + a, ...): the reference's clamp-to-edge is baked into
// the staged data, so every displaced sample position is plain box arithmetic.  A
// thread owns one sampled column of the node (fixed x and z sample offsets, its g
// samples along y) and one (lx, lz) label pair, and walks the len y-labels: the
// displaced y positions i + ly*q of its g samples are NA consecutive box entries,
// loaded once per channel; in the adjoint each entry's gradient is summed in a
// register before one shared-memory atomic (instead of one per term).

// Block size (whole warps, 128..256) that leaves the fewest idle item slots.
constexpr int balanced_block(int items) {
    int best = 256, waste = (items + 255) / 256 * 256 - items;
    for (int b = 224; b >= 128; b -= 32) {
        const int w = (items + b - 1) / b * b - items;
        if (w * 256 < waste * b) { best = b; waste = w; }
    }
    return best;
}

template <int G_, int LEN_, int Q_>
struct ColGeom {
    static constexpr int GS = G_, HW = (LEN_ - 1) / 2, R = HW * Q_, NA = G_ + 2 * R, NA3 = NA * NA * NA;
    static constexpr int S = G_ > 4 ? 2 : 1, NX = (G_ + S - 1) / S, NSAMP = NX * NX * G_;
    static constexpr int ITEMS = NX * NX * LEN_ * LEN_, LEN3 = LEN_ * LEN_ * LEN_;
    // forward items: (channel half, column, lx, lz); adjoint items per channel group: (channel, column, lx)
    static constexpr int FWD_ITEMS = 2 * ITEMS, ADJ_ITEMS = 6 * NX * NX * LEN_;
    static constexpr int FWD_BLOCK = balanced_block(FWD_ITEMS), ADJ_BLOCK = balanced_block(ADJ_ITEMS);
};

// Stage channels [c0, c0+CG) of the node's clamped box and, when fs is given, all
// 12 channels of its fixed samples.
template <class CGm>
__device__ __forceinline__ void stage_box(const SoftGeom& G, int y, int x, int z, const float* __restrict__ sM, int c0,
                                          int CG, float* hv, const float* __restrict__ sF, float* fs) {
    const int64_t mn = (int64_t)G.m * G.n, sz = mn * G.o;
    const int yb = y * G.g - CGm::R, xb = x * G.g - CGm::R, zb = z * G.g - CGm::R;
    // a warp stages 32/NA box rows at a time: lane -> (row within the group, y offset)
    constexpr int RPW = 32 / CGm::NA;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int sub = lane / CGm::NA, a = lane - sub * CGm::NA;
    const int ya = clampi(yb + a, 0, G.m - 1);
    const int nrows = CG * CGm::NA * CGm::NA;
    if (sub < RPW)
        for (int r = warp * RPW + sub; r < nrows; r += nw * RPW) {
            const int b = r % CGm::NA, t = r / CGm::NA, cc = t % CGm::NA, c = t / CGm::NA;
            cp_async4(hv + r * CGm::NA + a, sM + (int64_t)(c0 + c) * sz + ya + (int64_t)clampi(xb + b, 0, G.n - 1) * G.m +
                                                (int64_t)clampi(zb + cc, 0, G.o - 1) * mn);
        }
    if (fs)
        for (int e = threadIdx.x; e < 12 * CGm::NSAMP; e += blockDim.x) {
            const int c = e / CGm::NSAMP, s = e % CGm::NSAMP;
            const int py = y * CGm::GS + s % CGm::GS, px = x * CGm::GS + ((s / CGm::GS) % CGm::NX) * CGm::S,
                      pz = z * CGm::GS + (s / (CGm::GS * CGm::NX)) * CGm::S;
            cp_async4(fs + e, sF + (int64_t)c * sz + py + (int64_t)px * G.m + (int64_t)pz * mn);
        }
    cp_async_wait_all();
}

template <int G_, int LEN_, int Q_>
__global__ void __launch_bounds__(ColGeom<G_, LEN_, Q_>::FWD_BLOCK, 4)
    k_soft_cost_col(const float* __restrict__ sF, const float* __restrict__ sM, float* __restrict__ cost, SoftGeom G) {
    using CGm = ColGeom<G_, LEN_, Q_>;
    extern __shared__ float sh[];
    const int node = blockIdx.x;
    const int y = node % G.m1, x = (node / G.m1) % G.n1, z = node / (G.m1 * G.n1);
    float* hv = sh;                      // [12][NA3]
    float* fs = sh + 12 * CGm::NA3;      // [12][NSAMP]
    float* acc = fs + 12 * CGm::NSAMP;   // [LEN3]
    stage_box<CGm>(G, y, x, z, sM, 0, 12, hv, sF, fs);
    for (int l = threadIdx.x; l < CGm::LEN3; l += blockDim.x) acc[l] = 0.0f;
    __syncthreads();
    const float eps2 = G.eps * G.eps;
    // items are (column, lab, channel half) with the column fastest: the NX^2 = 16
    // columns of one (lab, half) are the 16 lanes of a half-warp (the block is a
    // multiple of 16 threads), whose label sums are reduced with shuffles before
    // one shared-memory add per label
    static_assert(CGm::NX * CGm::NX == 16, "column kernels assume 16 sampled columns per node");
    for (int base = 0; base < CGm::FWD_ITEMS; base += blockDim.x) {
        const int item = base + threadIdx.x;
        const bool valid = item < CGm::FWD_ITEMS;
        const int it = valid ? item : 0;
        const int col = it % 16, lab = (it / 16) % (LEN_ * LEN_);
        const int half = it / CGm::ITEMS;
        const int jj = col % CGm::NX, kk = col / CGm::NX, lx = lab % LEN_, lz = lab / LEN_;
        const int plane = CGm::NA * ((jj * CGm::S + lx * Q_) + CGm::NA * (kk * CGm::S + lz * Q_));
        float sums[LEN_][2];
#pragma unroll
        for (int ly = 0; ly < LEN_; ly++) sums[ly][0] = sums[ly][1] = 0.0f;
        if (valid)
            for (int c = 6 * half; c < 6 * half + 6; c++) {
                const float* hvc = hv + c * CGm::NA3 + plane;
                const float* fsc = fs + c * CGm::NSAMP + G_ * col;
                float v[CGm::NA], f[G_];
#pragma unroll
                for (int a = 0; a < CGm::NA; a++) v[a] = hvc[a];
#pragma unroll
                for (int i = 0; i < G_; i++) f[i] = fsc[i];
#pragma unroll
                for (int ly = 0; ly < LEN_; ly++)
#pragma unroll
                    for (int i = 0; i < G_; i++) {
                        const float d = f[i] - v[i + ly * Q_];
                        const float x2 = d * d + eps2;
                        sums[ly][i & 1] += x2 * rsqrtf(x2);
                    }
            }
#pragma unroll
        for (int ly = 0; ly < LEN_; ly++) {
            float v = sums[ly][0] + sums[ly][1];
#pragma unroll
            for (int off = 8; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            if (valid && col == 0) atomicAdd(acc + ly + LEN_ * lab, v);
        }
    }
    __syncthreads();
    for (int l = threadIdx.x; l < CGm::LEN3; l += blockDim.x)
        cost[(int64_t)node * CGm::LEN3 + l] = G.alpha1 * (acc[l] - (float)(12 * CGm::NSAMP) * G.eps);
}

// Adjoint: an item is one (channel, column, lx) of a channel group; it walks lz
// (different box rows) and, per row, the len y-labels x g samples: the row's
// gradient sums are accumulated in registers and added to a shared row buffer with
// one atomic per entry; the column's fixed-side gradients stay in registers across
// lz and are added once per item.  Channels are processed in two groups of six so
// that the shared footprint allows four CTAs per SM; items divide the block evenly.
constexpr int kAdjCG = 6;

template <int G_, int LEN_, int Q_>
__global__ void __launch_bounds__(ColGeom<G_, LEN_, Q_>::ADJ_BLOCK, 4)
    k_soft_cost_adj_col(const float* __restrict__ sF, const float* __restrict__ sM, const float* __restrict__ cbar,
                        const float* __restrict__ cost, float* __restrict__ sFbar, float* __restrict__ sMbar,
                        double* __restrict__ dot, SoftGeom G) {
    using CGm = ColGeom<G_, LEN_, Q_>;
    extern __shared__ float sh[];
    __shared__ double red[32];
    const int node = blockIdx.x;
    const int y = node % G.m1, x = (node / G.m1) % G.n1, z = node / (G.m1 * G.n1);
    const int64_t mn = (int64_t)G.m * G.n, sz = mn * G.o;
    float* hv = sh;                           // [CG][NA3]
    float* hg = sh + kAdjCG * CGm::NA3;       // [CG][NA3]
    float* fs = hg + kAdjCG * CGm::NA3;       // [12][NSAMP]
    float* gfs = fs + 12 * CGm::NSAMP;        // [12][NSAMP]
    float* cb = gfs + 12 * CGm::NSAMP;        // [LEN3]
    const float* cbn = cbar + (int64_t)node * CGm::LEN3;
    const float* cn = cost + (int64_t)node * CGm::LEN3;
    // alpha: centred dot product (the exact cbar sums to zero over labels)
    double csum = 0.0;
    for (int l = threadIdx.x; l < CGm::LEN3; l += blockDim.x) {
        csum += (double)cn[l];
        cb[l] = cbn[l];
    }
    for (int off = 16; off > 0; off >>= 1) csum += __shfl_xor_sync(0xffffffffu, csum, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = csum;
    for (int e = threadIdx.x; e < 12 * CGm::NSAMP; e += blockDim.x) gfs[e] = 0.0f;
    __syncthreads();
    double cmean = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) cmean += red[w];
    cmean /= (double)CGm::LEN3;
    double part = 0.0;
    for (int l = threadIdx.x; l < CGm::LEN3; l += blockDim.x) part += (double)cb[l] * ((double)cn[l] - cmean);
    for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(dot, part);
    const float eps2 = G.eps * G.eps;
    const int yb = y * G.g - CGm::R, xb = x * G.g - CGm::R, zb = z * G.g - CGm::R;
    for (int c0 = 0; c0 < 12; c0 += kAdjCG) {
        __syncthreads();
        stage_box<CGm>(G, y, x, z, sM, c0, kAdjCG, hv, sF, c0 == 0 ? fs : nullptr);
        for (int e = threadIdx.x; e < kAdjCG * CGm::NA3; e += blockDim.x) hg[e] = 0.0f;
        __syncthreads();
        // items (column, channel, lx) with the column fastest: a half-warp holds the 16
        // columns of one (channel, lx), whose box rows (jj + lx, kk + lz) are distinct,
        // so the row atomics of a warp never collide on an address
        for (int item = threadIdx.x; item < CGm::ADJ_ITEMS; item += blockDim.x) {
            const int col = item % (CGm::NX * CGm::NX);
            const int cl = (item / (CGm::NX * CGm::NX)) % kAdjCG;
            const int lx = item / (CGm::NX * CGm::NX * kAdjCG);
            const int jj = col % CGm::NX, kk = col / CGm::NX;
            const float* fsc = fs + (c0 + cl) * CGm::NSAMP + G_ * col;
            float f[G_], gf[G_];
#pragma unroll
            for (int i = 0; i < G_; i++) {
                f[i] = fsc[i];
                gf[i] = 0.0f;
            }
            for (int lz = 0; lz < LEN_; lz++) {
                const int plane = CGm::NA * ((jj * CGm::S + lx * Q_) + CGm::NA * (kk * CGm::S + lz * Q_));
                const float* hvr = hv + cl * CGm::NA3 + plane;
                float* hgr = hg + cl * CGm::NA3 + plane;
                const float* cbl = cb + LEN_ * (lx + LEN_ * lz);
                float v[CGm::NA], gm[CGm::NA];
#pragma unroll
                for (int a = 0; a < CGm::NA; a++) {
                    v[a] = hvr[a];
                    gm[a] = 0.0f;
                }
#pragma unroll
                for (int ly = 0; ly < LEN_; ly++) {
                    const float w = cbl[ly], nw = -w;
#pragma unroll
                    for (int i = 0; i < G_; i++) {
                        const float d = f[i] - v[i + ly * Q_];
                        const float t = d * rsqrtf(d * d + eps2);  // phi'(d)
                        gf[i] = fmaf(w, t, gf[i]);
                        gm[i + ly * Q_] = fmaf(nw, t, gm[i + ly * Q_]);
                    }
                }
#pragma unroll
                for (int a = 0; a < CGm::NA; a++) atomicAdd(hgr + a, gm[a]);
            }
#pragma unroll
            for (int i = 0; i < G_; i++) atomicAdd(gfs + (c0 + cl) * CGm::NSAMP + G_ * col + i, gf[i]);
        }
        __syncthreads();
        for (int e = threadIdx.x; e < kAdjCG * CGm::NA3; e += blockDim.x) {
            const float gv = hg[e];
            if (gv == 0.0f) continue;
            const int cl = e / CGm::NA3, r = e % CGm::NA3;
            const int a = r % CGm::NA, b = (r / CGm::NA) % CGm::NA, cc = r / (CGm::NA * CGm::NA);
            atomicAdd(sMbar + (int64_t)(c0 + cl) * sz + clampi(yb + a, 0, G.m - 1) +
                          (int64_t)clampi(xb + b, 0, G.n - 1) * G.m + (int64_t)clampi(zb + cc, 0, G.o - 1) * mn,
                      G.alpha1 * gv);
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 12 * CGm::NSAMP; e += blockDim.x) {
        const int c = e / CGm::NSAMP, s = e % CGm::NSAMP;
        const int py = y * G_ + s % G_, px = x * G_ + ((s / G_) % CGm::NX) * CGm::S,
                  pz = z * G_ + (s / (G_ * CGm::NX)) * CGm::S;
        sFbar[(int64_t)c * sz + py + (int64_t)px * G.m + (int64_t)pz * mn] = G.alpha1 * gfs[e];
    }
}

// ---------------------------------------------------------------------------
// Row form for the coarser levels (grid > 4: nine sampled columns per node, and
// label quantisation > 1).  An item is one label pair (lx, lz) of one sampled
// column; its displaced samples read one row of the moving descriptor: NA = g +
// (len-1) q consecutive voxels along y at clamped (x, z).  At these shapes no
// two items of a node read the same row, so a node's rows are staged compactly,
// row t at slot t with an odd pitch: the staging copies are coalesced along y
// (a warp per row, cp.async) and each thread then reads its own row from shared
// memory without bank conflicts (consecutive threads, rows PY apart, PY odd).  A thread keeps its item's len sums (forward)
// or the label weights (adjoint) in registers across all channel groups.  The
// moving-side gradient is the gather kernel k_soft_cost_adj_moving.

struct RowPlan {
    int PY, CG;  // row pitch (floats, odd), channels per stage
};

template <int G_, int LEN_, int Q_>
struct RowGeom {
    static constexpr int S = G_ > 4 ? 2 : 1, NX = (G_ + S - 1) / S, NCOL = NX * NX, NSAMP = NCOL * G_;
    static constexpr int NA = G_ + (LEN_ - 1) * Q_, LEN2 = LEN_ * LEN_, LEN3 = LEN2 * LEN_;
    static constexpr int ITEMS = LEN2 * NCOL;
    static constexpr int BLOCK = (ITEMS + 31) / 32 * 32;
    static constexpr int PY = NA | 1;
    static_assert(ITEMS <= 1024 && NA <= 32, "one item per thread, one row per warp");
};

// Item t of a node: label pair (lab = lx + len*lz) and sampled column (jj, kk).
// Label-fastest order (forward: a warp's items share a column, its label sums go
// to distinct addresses) or column-fastest order (adjoint: a warp's items spread
// over the nine columns, so its sample-gradient atomics hit a column <= 4 times).
template <class RG, int LEN_, int Q_, bool COL_FAST>
__device__ __forceinline__ void row_item(int t, int& lab, int& col, int& bx, int& bz) {
    lab = COL_FAST ? t / RG::NCOL : t % RG::LEN2;
    col = COL_FAST ? t % RG::NCOL : t / RG::LEN2;
    const int lx = lab % LEN_, lz = lab / LEN_, jj = col % RG::NX, kk = col / RG::NX;
    bx = jj * RG::S + lx * Q_;
    bz = kk * RG::S + lz * Q_;
}

// Stage channels [c0, c0+CG) of the node's item rows: rows[c][t][a], pitch PY.
// goff[t] holds item t's clamped (x, z) offset in one channel.
template <class RG>
__device__ __forceinline__ void stage_rows(const SoftGeom& G, int yb, const float* __restrict__ sM, int c0, int CG,
                                           const int* goff, float* rows) {
    const int64_t sz = (int64_t)G.m * G.n * G.o;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int ya = clampi(yb + lane, 0, G.m - 1);
    if (lane < RG::NA)
        for (int c = 0; c < CG; c++) {
            const float* src = sM + (int64_t)(c0 + c) * sz + ya;
            float* dst = rows + c * (RG::ITEMS * RG::PY) + lane;
            for (int r = warp; r < RG::ITEMS; r += nw) cp_async4(dst + r * RG::PY, src + goff[r]);
        }
    cp_async_wait_all();
}

template <class RG>
__device__ __forceinline__ void stage_fixed_samples(const SoftGeom& G, int y, int x, int z,
                                                    const float* __restrict__ sF, float* fs) {
    const int64_t mn = (int64_t)G.m * G.n, sz = mn * G.o;
    for (int e = threadIdx.x; e < 12 * RG::NSAMP; e += blockDim.x) {
        const int c = e / RG::NSAMP, s = e % RG::NSAMP;
        const int col = s / G.g, i = s % G.g;
        const int py = y * G.g + i, px = x * G.g + (col % RG::NX) * RG::S, pz = z * G.g + (col / RG::NX) * RG::S;
        cp_async4(fs + e, sF + (int64_t)c * sz + py + (int64_t)px * G.m + (int64_t)pz * mn);
    }
    cp_async_wait_all();
}

// Each thread writes its item's clamped (x, z) row offset; returns the box's y origin.
template <class RG, int LEN_, int Q_, bool COL_FAST>
__device__ __forceinline__ int row_offsets(const SoftGeom& G, int y, int x, int z, int* goff) {
    const int R = (RG::NA - G.g) / 2;
    const int t = threadIdx.x;
    if (t < RG::ITEMS) {
        int lab, col, bx, bz;
        row_item<RG, LEN_, Q_, COL_FAST>(t, lab, col, bx, bz);
        goff[t] = clampi(x * G.g - R + bx, 0, G.n - 1) * G.m + clampi(z * G.g - R + bz, 0, G.o - 1) * G.m * G.n;
    }
    return y * G.g - R;
}

template <int G_, int LEN_, int Q_>
__global__ void __launch_bounds__(RowGeom<G_, LEN_, Q_>::BLOCK, 2)
    k_soft_cost_rows(const float* __restrict__ sF, const float* __restrict__ sM, float* __restrict__ cost, SoftGeom G,
                     RowPlan P) {
    using RG = RowGeom<G_, LEN_, Q_>;
    extern __shared__ float sh[];
    const int node = blockIdx.x;
    const int y = node % G.m1, x = (node / G.m1) % G.n1, z = node / (G.m1 * G.n1);
    float* rows = sh;                                  // [CG][ITEMS][PY]
    float* fs = rows + P.CG * RG::ITEMS * RG::PY;      // [12][NSAMP]
    float* acc = fs + 12 * RG::NSAMP;                  // [LEN3]
    int* goff = reinterpret_cast<int*>(acc + RG::LEN3);  // [ITEMS]
    const int yb = row_offsets<RG, LEN_, Q_, false>(G, y, x, z, goff);
    for (int l = threadIdx.x; l < RG::LEN3; l += blockDim.x) acc[l] = 0.0f;
    stage_fixed_samples<RG>(G, y, x, z, sF, fs);
    const float eps2 = G.eps * G.eps;
    const int t = threadIdx.x;
    const bool active = t < RG::ITEMS;
    int lab = 0, col = 0, bx, bz;
    row_item<RG, LEN_, Q_, false>(active ? t : 0, lab, col, bx, bz);
    float sums[LEN_];
#pragma unroll
    for (int ly = 0; ly < LEN_; ly++) sums[ly] = 0.0f;
    for (int c0 = 0; c0 < 12; c0 += P.CG) {
        __syncthreads();  // goff written / previous rows consumed
        stage_rows<RG>(G, yb, sM, c0, P.CG, goff, rows);
        __syncthreads();
        if (active)
            for (int c = 0; c < P.CG; c++) {
                const float* row = rows + (c * RG::ITEMS + t) * RG::PY;
                const float* fc = fs + (c0 + c) * RG::NSAMP + col * G_;
                float v[RG::NA], f[G_];
#pragma unroll
                for (int a = 0; a < RG::NA; a++) v[a] = row[a];
#pragma unroll
                for (int i = 0; i < G_; i++) f[i] = fc[i];
#pragma unroll
                for (int ly = 0; ly < LEN_; ly++)
#pragma unroll
                    for (int i = 0; i < G_; i++) {
                        const float d = f[i] - v[i + ly * Q_];
                        const float x2 = d * d + eps2;
                        sums[ly] += x2 * rsqrtf(x2);
                    }
            }
    }
    if (active)
#pragma unroll
        for (int ly = 0; ly < LEN_; ly++) atomicAdd(acc + ly + LEN_ * lab, sums[ly]);
    __syncthreads();
    for (int l = threadIdx.x; l < RG::LEN3; l += blockDim.x)
        cost[(int64_t)node * RG::LEN3 + l] = G.alpha1 * (acc[l] - (float)(12 * RG::NSAMP) * G.eps);
}

// Fixed-side adjoint and the alpha dot product in row form: an item's len label
// weights stay in registers, its g sample gradients are summed over its labels
// per channel and added to the node's shared sample gradients.
template <int G_, int LEN_, int Q_>
__global__ void __launch_bounds__(RowGeom<G_, LEN_, Q_>::BLOCK, 2)
    k_soft_cost_adjF_rows(const float* __restrict__ sF, const float* __restrict__ sM, const float* __restrict__ cbar,
                          const float* __restrict__ cost, float* __restrict__ sFbar, double* __restrict__ dot,
                          SoftGeom G, RowPlan P) {
    using RG = RowGeom<G_, LEN_, Q_>;
    extern __shared__ float sh[];
    __shared__ double red[32];
    const int node = blockIdx.x;
    const int y = node % G.m1, x = (node / G.m1) % G.n1, z = node / (G.m1 * G.n1);
    const int64_t mn = (int64_t)G.m * G.n, sz = mn * G.o;
    float* rows = sh;                                  // [CG][ITEMS][PY]
    float* fs = rows + P.CG * RG::ITEMS * RG::PY;      // [12][NSAMP]
    float* gfs = fs + 12 * RG::NSAMP;                  // [12][NSAMP]
    float* cb = gfs + 12 * RG::NSAMP;                  // [LEN3]
    int* goff = reinterpret_cast<int*>(cb + RG::LEN3);  // [ITEMS]
    const float* cbn = cbar + (int64_t)node * RG::LEN3;
    const float* cn = cost + (int64_t)node * RG::LEN3;
    const int yb = row_offsets<RG, LEN_, Q_, true>(G, y, x, z, goff);
    // alpha: centred dot product (the exact cbar sums to zero over labels)
    double csum = 0.0;
    for (int l = threadIdx.x; l < RG::LEN3; l += blockDim.x) {
        csum += (double)cn[l];
        cb[l] = cbn[l];
    }
    for (int off = 16; off > 0; off >>= 1) csum += __shfl_xor_sync(0xffffffffu, csum, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = csum;
    for (int e = threadIdx.x; e < 12 * RG::NSAMP; e += blockDim.x) gfs[e] = 0.0f;
    stage_fixed_samples<RG>(G, y, x, z, sF, fs);
    __syncthreads();
    double cmean = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) cmean += red[w];
    cmean /= (double)RG::LEN3;
    double part = 0.0;
    for (int l = threadIdx.x; l < RG::LEN3; l += blockDim.x) part += (double)cb[l] * ((double)cn[l] - cmean);
    for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(dot, part);
    const float eps2 = G.eps * G.eps;
    const int t = threadIdx.x;
    const bool active = t < RG::ITEMS;
    int lab = 0, col = 0, bx, bz;
    row_item<RG, LEN_, Q_, true>(active ? t : 0, lab, col, bx, bz);
    float w[LEN_];
#pragma unroll
    for (int ly = 0; ly < LEN_; ly++) w[ly] = cb[ly + LEN_ * lab];
    for (int c0 = 0; c0 < 12; c0 += P.CG) {
        __syncthreads();
        stage_rows<RG>(G, yb, sM, c0, P.CG, goff, rows);
        __syncthreads();
        if (active)
            for (int c = 0; c < P.CG; c++) {
                const float* row = rows + (c * RG::ITEMS + t) * RG::PY;
                const float* fc = fs + (c0 + c) * RG::NSAMP + col * G_;
                float* gfc = gfs + (c0 + c) * RG::NSAMP + col * G_;
                float v[RG::NA], f[G_], gf[G_];
#pragma unroll
                for (int a = 0; a < RG::NA; a++) v[a] = row[a];
#pragma unroll
                for (int i = 0; i < G_; i++) {
                    f[i] = fc[i];
                    gf[i] = 0.0f;
                }
#pragma unroll
                for (int ly = 0; ly < LEN_; ly++)
#pragma unroll
                    for (int i = 0; i < G_; i++) {
                        const float d = f[i] - v[i + ly * Q_];
                        gf[i] += w[ly] * d * rsqrtf(d * d + eps2);
                    }
#pragma unroll
                for (int i = 0; i < G_; i++) atomicAdd(gfc + i, gf[i]);
            }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 12 * RG::NSAMP; e += blockDim.x) {
        const int c = e / RG::NSAMP, s = e % RG::NSAMP;
        const int cl = s / G.g, i = s % G.g;
        const int py = y * G.g + i, px = x * G.g + (cl % RG::NX) * RG::S, pz = z * G.g + (cl / RG::NX) * RG::S;
        sFbar[(int64_t)c * sz + py + (int64_t)px * G.m + (int64_t)pz * mn] = G.alpha1 * gfs[e];
    }
}

// ---------------------------------------------------------------------------
// Tree sweeps

struct SoftTree {
    int len, len3, hw, sz, root, q;
    float tau, itau;
    const int* parents;
    const float* edgemst;
    const int* child_ptr;
    const int* children;
    const float* off;  // nullable: (3, sz) label-unit offsets x|y|z of each node's edge, (prior[parent]-prior[node])/q
    float* offbar;     // nullable (backward): dL/doff, (3, sz)
};

// The offset of node c's edge along label axis s (stride 1 = y, len = x, len^2 = z).
__device__ __forceinline__ float edge_off(const SoftTree& t, int c, int axis) {
    if (!t.off) return 0.0f;
    const int comp = axis == 0 ? 1 : (axis == 1 ? 0 : 2);  // off is stored x|y|z
    return t.off[comp * t.sz + c];
}

__device__ float block_max(float v, float* red) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    float r = -INFINITY;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) r = fmaxf(r, red[w]);
    __syncthreads();
    return r;
}

// (max, sum exp(x - max)) of the block's values in one reduction; returns the LSE.
// red needs 64 floats.
__device__ float block_lse(float mx, float se, float* red) {
    for (int o = 16; o > 0; o >>= 1) {
        const float om = __shfl_xor_sync(0xffffffffu, mx, o), os = __shfl_xor_sync(0xffffffffu, se, o);
        const float nm = fmaxf(mx, om);
        se = (mx == -INFINITY ? 0.0f : se * __expf(mx - nm)) + (om == -INFINITY ? 0.0f : os * __expf(om - nm));
        mx = nm;
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
        red[threadIdx.x >> 5] = mx;
        red[32 + (threadIdx.x >> 5)] = se;
    }
    __syncthreads();
    float m = -INFINITY;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) m = fmaxf(m, red[w]);
    float t = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++)
        if (red[w] != -INFINITY) t += red[32 + w] * __expf(red[w] - m);
    __syncthreads();
    return m + __logf(t);
}

// three sums in one reduction; red needs 96 floats
__device__ void block_sum3(float& a, float& b, float& c, float* red) {
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
        c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
        red[threadIdx.x >> 5] = a;
        red[32 + (threadIdx.x >> 5)] = b;
        red[64 + (threadIdx.x >> 5)] = c;
    }
    __syncthreads();
    a = b = c = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
        a += red[w];
        b += red[32 + w];
        c += red[64 + w];
    }
    __syncthreads();
}

__device__ float block_sum(float v, float* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    float r = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) r += red[w];
    __syncthreads();
    return r;
}

// out(o) = LSE_a in(line(o), a) - d(a, b)^2/tau along the axis of stride s, with b =
// o's coordinate on that axis and d = sgn (b - a) + off (the prior field's offset of
// the edge; sgn = +1 when b indexes the parent label, -1 when it indexes the child's).
// Ends with a barrier.
__device__ void lse_axis(const float* in, float* out, int len, int len3, int s, float itau, float off, float sgn) {
    for (int o = threadIdx.x; o < len3; o += blockDim.x) {
        const int b = (o / s) % len;
        const float* line = in + (o - b * s);
        float mx = -INFINITY;
        for (int a = 0; a < len; a++) {
            const float d = sgn * (float)(b - a) + off;
            mx = fmaxf(mx, line[a * s] - d * d * itau);
        }
        float acc = 0.0f;
        for (int a = 0; a < len; a++) {
            const float d = sgn * (float)(b - a) + off;
            acc += __expf(line[a * s] - d * d * itau - mx);
        }
        out[o] = mx + __logf(acc);
    }
    __syncthreads();
}

// adjoint of one pass: inbar(a) = sum_b outbar(b) w(a, b), w = exp(in(a) - d^2/tau - out(b));
// returns this thread's part of dL/doff = sum_{a,b} outbar(b) w(a, b) (-2 d / tau).
__device__ float lse_axis_adj(const float* in, const float* out, const float* outbar, float* inbar, int len, int len3,
                              int s, float itau, float off, float sgn) {
    float dof = 0.0f;
    for (int o = threadIdx.x; o < len3; o += blockDim.x) {
        const int a = (o / s) % len;
        const int base = o - a * s;
        const float x = in[o];
        float acc = 0.0f;
        for (int b = 0; b < len; b++) {
            const float d = sgn * (float)(b - a) + off;
            const float wb = outbar[base + b * s] * __expf(x - d * d * itau - out[base + b * s]);
            acc += wb;
            dof += wb * d;
        }
        inbar[o] = acc;
    }
    __syncthreads();
    return -2.0f * itau * dof;
}

// S = pass z o pass x o pass y; keeps t1, t2 for the adjoint (out may alias in).
// off3 = (y, x, z) offsets of the node's edge.
__device__ __forceinline__ void sep_lse(const float* in, float* t1, float* t2, float* out, int len, int len3,
                                        float itau, const float* off3, float sgn) {
    lse_axis(in, t1, len, len3, 1, itau, off3[0], sgn);
    lse_axis(t1, t2, len, len3, len, itau, off3[1], sgn);
    lse_axis(t2, out, len, len3, len * len, itau, off3[2], sgn);
}

// inbar = S^T outbar.  wa is scratch; wb may alias outbar and inbar may alias wa.
// dof3 (y, x, z) receives this thread's parts of dL/doff.
__device__ __forceinline__ void sep_lse_adj(const float* in, const float* t1, const float* t2, const float* out,
                                            const float* outbar, float* wa, float* wb, float* inbar, int len,
                                            int len3, float itau, const float* off3, float sgn, float* dof3) {
    dof3[2] = lse_axis_adj(t2, out, outbar, wa, len, len3, len * len, itau, off3[2], sgn);
    dof3[1] = lse_axis_adj(t1, t2, wa, wb, len, len3, len, itau, off3[1], sgn);
    dof3[0] = lse_axis_adj(in, t1, wb, inbar, len, len3, 1, itau, off3[0], sgn);
}

// Adds this block's dL/doff of node c (scaled) into t.offbar (x|y|z layout); red: 96 floats.
__device__ void add_offbar(const SoftTree& t, int c, float* dof3, float scale, float* red) {
    if (!t.offbar) return;
    block_sum3(dof3[0], dof3[1], dof3[2], red);
    if (threadIdx.x == 0) {
        t.offbar[t.sz + c] += scale * dof3[0];      // y
        t.offbar[c] += scale * dof3[1];             // x
        t.offbar[2 * t.sz + c] += scale * dof3[2];  // z
    }
}

// ---- per-node bodies (one CTA per node; data of other nodes written in the same
// sweep is read with __ldcg, after the producer's release has been observed)
//
// What a node reads that does not come from this sweep (its own rows from the
// forward or earlier sweeps, its child list) is loaded before the dependency
// wait into NodePre — one label per thread, the label threadIdx.x — so that after
// the wait only the rows produced in this sweep remain on the critical path, and
// the children's rows are then loaded together rather than one child after another.

constexpr int kMaxChildren = 6;  // a 6-connected grid tree: at most 6 children (the root)

struct NodePre {
    float v0, v1, v2;  // own values at label threadIdx.x (meaning depends on the sweep)
    int nch;
    int ch[kMaxChildren];
};

// Own value at label l: prefetched for the thread's first label, else loaded.
__device__ __forceinline__ float own(int l, float pre, const float* __restrict__ row) {
    return l == (int)threadIdx.x ? pre : row[l];
}

__device__ __forceinline__ void load_children(const SoftTree& t, int c, NodePre& pre) {
    const int k0 = t.child_ptr[c], k1 = t.child_ptr[c + 1];
    pre.nch = k1 - k0;
#pragma unroll
    for (int i = 0; i < kMaxChildren; i++) pre.ch[i] = i < pre.nch ? t.children[k0 + i] : 0;
}

// v + sum over children in child order of (X[k][l] - xmin[k]) (xmin may be null):
// all children's values are loaded before the in-order sum.
__device__ __forceinline__ float add_children(const SoftTree& t, int c, const NodePre& pre, int l, float v,
                                              const float* __restrict__ X, const float* __restrict__ xmin) {
    const int L3 = t.len3;
    if (pre.nch <= kMaxChildren) {
        float xs[kMaxChildren], ms[kMaxChildren];
#pragma unroll
        for (int i = 0; i < kMaxChildren; i++) {
            xs[i] = i < pre.nch ? __ldcg(X + (int64_t)pre.ch[i] * L3 + l) : 0.0f;
            ms[i] = (xmin && i < pre.nch) ? __ldcg(xmin + pre.ch[i]) : 0.0f;
        }
#pragma unroll
        for (int i = 0; i < kMaxChildren; i++)
            if (i < pre.nch) v += xmin ? xs[i] - ms[i] : xs[i];
        return v;
    }
    for (int ci = t.child_ptr[c]; ci < t.child_ptr[c + 1]; ci++) {
        const int k = t.children[ci];
        v += xmin ? __ldcg(X + (int64_t)k * L3 + l) - __ldcg(xmin + k) : __ldcg(X + (int64_t)k * L3 + l);
    }
    return v;
}

// Upward: B_c = C_c + sum_children (M_k - min M_k), stored minus its minimum (the
// marginals and the parent's (message - min) are invariant to a constant shift of
// B_c, and the centred values keep the exponents of the label-space transforms
// small where the probability mass is); M_c = -tau S(-e_c B_c / tau).
__device__ void node_up(const SoftTree& t, int c, const NodePre& pre, const float* __restrict__ cost,
                        float* __restrict__ B, float* __restrict__ M, float* __restrict__ Mmin, float* sh) {
    const int L3 = t.len3;
    float* f = sh;
    float* t1 = sh + L3;
    float* t2 = sh + 2 * L3;
    float* red = sh + 3 * L3;
    const float e = c == t.root ? 0.0f : t.edgemst[c];
    float bmin = INFINITY;
    for (int l = threadIdx.x; l < L3; l += blockDim.x) {
        const float v = add_children(t, c, pre, l, own(l, pre.v0, cost + (int64_t)c * L3), M, Mmin);
        f[l] = v;
        bmin = fminf(bmin, v);
    }
    bmin = -block_max(-bmin, red);
    for (int l = threadIdx.x; l < L3; l += blockDim.x) {
        const float v = f[l] - bmin;
        B[(int64_t)c * L3 + l] = v;
        f[l] = -e * v * t.itau;
    }
    __syncthreads();
    if (c == t.root) return;
    const float off3[3] = {edge_off(t, c, 0), edge_off(t, c, 1), edge_off(t, c, 2)};
    sep_lse(f, t1, t2, f, t.len, L3, t.itau, off3, 1.0f);  // output index = parent label
    float mn = INFINITY;
    for (int lp = threadIdx.x; lp < L3; lp += blockDim.x) {
        const float msg = -t.tau * f[lp];
        M[(int64_t)c * L3 + lp] = msg;
        mn = fminf(mn, msg);
    }
    mn = -block_max(-mn, red);
    if (threadIdx.x == 0) Mmin[c] = mn;
}

// Downward marginals; writes log p_c and the expected displacement.  log p_c is
// normalised in exact arithmetic; renormalising stops float rounding from drifting
// along root-to-leaf paths (no effect on the exact gradient, whose parameter
// derivatives are tangent to the normalised set).
__device__ void node_down(const SoftTree& t, int c, const NodePre& pre, const float* __restrict__ B,
                          const float* __restrict__ M, float* __restrict__ logp, float* __restrict__ disp, float* sh) {
    const int L3 = t.len3, len = t.len;
    float* r = sh;
    float* t1 = sh + L3;
    float* t2 = sh + 2 * L3;
    float* red = sh + 3 * L3;
    float* lc = logp + (int64_t)c * L3;
    const float* bc = B + (int64_t)c * L3;
    if (c == t.root) {
        for (int l = threadIdx.x; l < L3; l += blockDim.x) r[l] = -own(l, pre.v1, bc) * t.itau;
    } else {
        const int p = t.parents[c];
        const float e = t.edgemst[c];
        for (int lp = threadIdx.x; lp < L3; lp += blockDim.x)
            r[lp] = __ldcg(logp + (int64_t)p * L3 + lp) + own(lp, pre.v0, M + (int64_t)c * L3) * t.itau;
        __syncthreads();
        const float off3[3] = {edge_off(t, c, 0), edge_off(t, c, 1), edge_off(t, c, 2)};
        sep_lse(r, t1, t2, r, len, L3, t.itau, off3, -1.0f);  // output index = child label
        for (int l = threadIdx.x; l < L3; l += blockDim.x) r[l] += -e * own(l, pre.v1, bc) * t.itau;
    }
    float mx = -INFINITY;
    for (int l = threadIdx.x; l < L3; l += blockDim.x) mx = fmaxf(mx, r[l]);
    float se = 0.0f;
    for (int l = threadIdx.x; l < L3; l += blockDim.x) se += __expf(r[l] - mx);
    const float lz = block_lse(mx, se, red);
    float eu = 0.0f, ev = 0.0f, ew = 0.0f;
    for (int l = threadIdx.x; l < L3; l += blockDim.x) {
        const float lp = r[l] - lz;
        lc[l] = lp;
        const float pl = __expf(lp);
        eu += pl * (float)(((l / len) % len - t.hw) * t.q);
        ev += pl * (float)((l % len - t.hw) * t.q);
        ew += pl * (float)((l / (len * len) - t.hw) * t.q);
    }
    block_sum3(eu, ev, ew, red);
    if (threadIdx.x == 0) {
        disp[c] = eu;
        disp[t.sz + c] = ev;
        disp[2 * t.sz + c] = ew;
    }
}

// Adjoint of the marginals (leaves to root):
//   h(l) = gE_c . d(l) p_c(l) + sum_children R_k(l)    (= dL/dlog p_c)
//   Bbar_c = -e h/tau (root: -(h - p sum h)/tau, projected to zero mean);  R_c = S^T h w.r.t. r
__device__ void node_down_adj(const SoftTree& t, int c, const NodePre& pre, const float* __restrict__ M,
                              const float* __restrict__ logp, const float* __restrict__ gdisp, float* __restrict__ R,
                              float* __restrict__ Bbar, float* sh) {
    const int L3 = t.len3, len = t.len;
    float* r = sh;
    float* t1 = sh + L3;
    float* t2 = sh + 2 * L3;
    float* G = sh + 3 * L3;
    float* h = sh + 4 * L3;
    float* wa = sh + 5 * L3;
    float* red = sh + 6 * L3;
    const float* lc = logp + (int64_t)c * L3;
    const float gu = gdisp[c], gv = gdisp[t.sz + c], gw = gdisp[2 * t.sz + c];
    float tot = 0.0f;
    for (int l = threadIdx.x; l < L3; l += blockDim.x) {
        const float du = (float)(((l / len) % len - t.hw) * t.q), dv = (float)((l % len - t.hw) * t.q),
                    dw = (float)((l / (len * len) - t.hw) * t.q);
        const float v = add_children(t, c, pre, l, (gu * du + gv * dv + gw * dw) * __expf(own(l, pre.v0, lc)), R,
                                     nullptr);
        h[l] = v;
        tot += v;
    }
    float* bb = Bbar + (int64_t)c * L3;
    if (c == t.root) {
        tot = block_sum(tot, red);
        float mean = 0.0f;
        for (int l = threadIdx.x; l < L3; l += blockDim.x) {
            wa[l] = -(h[l] - __expf(own(l, pre.v0, lc)) * tot) * t.itau;
            mean += wa[l];
        }
        mean = block_sum(mean, red) / (float)L3;
        for (int l = threadIdx.x; l < L3; l += blockDim.x) bb[l] = wa[l] - mean;
        return;
    }
    const int p = t.parents[c];
    const float e = t.edgemst[c];
    for (int l = threadIdx.x; l < L3; l += blockDim.x) {
        bb[l] = -e * t.itau * h[l];
        r[l] = own(l, pre.v2, logp + (int64_t)p * L3) + own(l, pre.v1, M + (int64_t)c * L3) * t.itau;
    }
    __syncthreads();
    const float off3[3] = {edge_off(t, c, 0), edge_off(t, c, 1), edge_off(t, c, 2)};
    float dof3[3];
    sep_lse(r, t1, t2, G, len, L3, t.itau, off3, -1.0f);
    sep_lse_adj(r, t1, t2, G, h, wa, h, wa, len, L3, t.itau, off3, -1.0f, dof3);
    float* rc = R + (int64_t)c * L3;
    for (int l = threadIdx.x; l < L3; l += blockDim.x) rc[l] = wa[l];
    add_offbar(t, c, dof3, 1.0f, red);
}

// Adjoint of the upward recursion (root to leaves, root excluded):
//   Mbar_c = R_c/tau + Bbar_parent; M_c = -tau S(f), f = -e B_c/tau, so
//   dL/dB_c += -e/tau S^T(-tau Mbar_c) = e S^T(Mbar_c).  Bbar_c is final afterwards
// (= dL/dC_c); the exact value sums to zero over labels (shift invariance), and
// projecting keeps rounding from accumulating as a common mode down the tree.
__device__ void node_up_adj(const SoftTree& t, int c, const NodePre& pre, const float* __restrict__ B,
                            const float* __restrict__ R, float* __restrict__ Bbar, float* sh) {
    if (c == t.root) return;
    const int L3 = t.len3, len = t.len;
    float* f = sh;
    float* t1 = sh + L3;
    float* t2 = sh + 2 * L3;
    float* out = sh + 3 * L3;
    float* mb = sh + 4 * L3;
    float* wa = sh + 5 * L3;
    float* red = sh + 6 * L3;
    const int p = t.parents[c];
    const float e = t.edgemst[c];
    for (int l = threadIdx.x; l < L3; l += blockDim.x) {
        f[l] = -e * own(l, pre.v0, B + (int64_t)c * L3) * t.itau;
        mb[l] = own(l, pre.v1, R + (int64_t)c * L3) * t.itau + __ldcg(Bbar + (int64_t)p * L3 + l);
    }
    __syncthreads();
    const float off3[3] = {edge_off(t, c, 0), edge_off(t, c, 1), edge_off(t, c, 2)};
    float dof3[3];
    sep_lse(f, t1, t2, out, len, L3, t.itau, off3, 1.0f);
    sep_lse_adj(f, t1, t2, out, mb, wa, mb, wa, len, L3, t.itau, off3, 1.0f, dof3);
    // M = -tau out: dL/dout = -tau Mbar, so the offset gradient computed with Mbar scales by -tau
    add_offbar(t, c, dof3, -t.tau, red);
    float* bb = Bbar + (int64_t)c * L3;
    float mean = 0.0f;
    for (int l = threadIdx.x; l < L3; l += blockDim.x) {
        wa[l] = own(l, pre.v2, bb) + e * wa[l];
        mean += wa[l];
    }
    mean = block_sum(mean, red) / (float)L3;
    for (int l = threadIdx.x; l < L3; l += blockDim.x) bb[l] = wa[l] - mean;
}

// ---- persistent sweeps
//
// One launch per sweep.  CTAs claim nodes with a global ticket in breadth order
// (top-down sweeps) or reverse breadth order (bottom-up sweeps), wait until the
// node's parent (top-down) or all of its children (bottom-up) are finished, run the
// node body and release it.  A node only waits on nodes with smaller tickets,
// which were claimed by CTAs that are running and wait only on smaller tickets
// still, so the sweep always progresses; there are no per-level launches.  Each
// wait is bounded: on expiry the sweep records an error (reported as a timeout by
// the host) and carries on without further waits, so no CTA can hang.  (A
// wait-free variant for the bottom-up sweeps, in which the CTA completing a
// node's children continues with the node, measured 6-9 % slower: claiming in
// breadth order keeps each level's nodes in flight together.)


struct SweepState {
    int* ticket;  // next ticket
    int* done;    // top-down: 1 when the node is finished; bottom-up: children finished
    int* err;     // set when a wait gave up
};

__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

enum SweepKind { kSweepUp = 0, kSweepDown = 1, kSweepDownAdj = 2, kSweepUpAdj = 3 };

// Publishing a finished node: a release store (top-down: the node is done) or a
// release reduction (bottom-up: one more child of the parent has arrived) at GPU
// scope; the preceding block barrier makes every thread's writes of the node part
// of what is released, and waiters read the flag with ld.acquire.
__device__ __forceinline__ void st_release(int* p, int v) {
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void red_release_add(int* p, int v) {
    asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

constexpr long long kSweepSpinLimitV = 1LL << 21;  // ~0.13 s of 64 ns sleeps

// Bounded wait of one thread until *flag >= need; on expiry sets *err and returns
// false (the caller then skips every further wait).
__device__ __forceinline__ bool bounded_wait_geq(const int* flag, int need, int* err) {
    long long it = 0;
    while (ld_acquire(flag) < need) {
        if (++it > kSweepSpinLimitV) {
            atomicExch(err, 1);
            return false;
        }
        __nanosleep(64);
    }
    return true;
}

struct SweepArgs {
    const float* cost;
    float* B;
    float* M;
    float* Mmin;
    float* logp;
    float* disp;
    const float* gdisp;
    float* R;
    float* Bbar;
};

template <int KIND>
__device__ __forceinline__ void run_node(const SoftTree& t, int c, const NodePre& pre, const SweepArgs& a,
                                         float* sh) {
    if (KIND == kSweepUp) node_up(t, c, pre, a.cost, a.B, a.M, a.Mmin, sh);
    else if (KIND == kSweepDown) node_down(t, c, pre, a.B, a.M, a.logp, a.disp, sh);
    else if (KIND == kSweepDownAdj) node_down_adj(t, c, pre, a.M, a.logp, a.gdisp, a.R, a.Bbar, sh);
    else node_up_adj(t, c, pre, a.B, a.R, a.Bbar, sh);
}

// The node's inputs that precede this sweep (see NodePre), loaded before the wait.
template <int KIND>
__device__ __forceinline__ NodePre prefetch_node(const SoftTree& t, int c, const SweepArgs& a) {
    NodePre pre;
    pre.v0 = pre.v1 = pre.v2 = 0.0f;
    pre.nch = 0;
    const int l = threadIdx.x;
    const bool in = l < t.len3;
    const int64_t row = (int64_t)c * t.len3 + l;
    const bool root = c == t.root;
    if (KIND == kSweepUp) {
        if (in) pre.v0 = a.cost[row];
        load_children(t, c, pre);
    } else if (KIND == kSweepDown) {
        if (in) {
            if (!root) pre.v0 = a.M[row];
            pre.v1 = a.B[row];
        }
    } else if (KIND == kSweepDownAdj) {
        if (in) {
            pre.v0 = a.logp[row];
            if (!root) {
                pre.v1 = a.M[row];
                pre.v2 = a.logp[(int64_t)t.parents[c] * t.len3 + l];
            }
        }
        load_children(t, c, pre);
    } else if (!root && in) {
        pre.v0 = a.B[row];
        pre.v1 = a.R[row];
        pre.v2 = a.Bbar[row];
    }
    return pre;
}

template <int KIND>
__global__ void k_soft_sweep(SoftTree t, const int* __restrict__ ordered, SweepArgs a, SweepState st) {
    extern __shared__ float sh[];
    __shared__ int s_tk;
    constexpr bool kTopDown = KIND == kSweepDown || KIND == kSweepUpAdj;
    for (;;) {
        if (threadIdx.x == 0) s_tk = atomicAdd(st.ticket, 1);
        __syncthreads();
        const int tk = s_tk;
        if (tk >= t.sz) break;
        const int c = ordered[kTopDown ? tk : t.sz - 1 - tk];
        const NodePre pre = prefetch_node<KIND>(t, c, a);
        if (threadIdx.x == 0 && ld_acquire(st.err) == 0) {
            // top-down: the parent is released (done = 1); bottom-up: every child has arrived
            const int* flag = kTopDown ? (c == t.root ? nullptr : st.done + t.parents[c]) : st.done + c;
            const int need = kTopDown ? 1 : t.child_ptr[c + 1] - t.child_ptr[c];
            if (flag && need > 0) bounded_wait_geq(flag, need, st.err);
        }
        __syncthreads();
        run_node<KIND>(t, c, pre, a, sh);
        __syncthreads();
        if (threadIdx.x == 0) {
            if (kTopDown) st_release(st.done + c, 1);
            else if (c != t.root) red_release_add(st.done + t.parents[c], 1);
        }
    }
}

int soft_threads(int len) { return len * len * len <= 343 ? 128 : 256; }

// one thread per label (rounded to whole warps): the per-node passes are latency bound
int tree_threads(int len) { return std::min(1024, (len * len * len + 31) / 32 * 32); }

SoftGeom make_geom(int m, int n, int o, int g, int hw, int q, float alpha1, float eps) {
    SoftGeom G;
    G.m = m; G.n = n; G.o = o; G.g = g; G.hw = hw; G.q = q;
    G.len = 2 * hw + 1; G.len3 = G.len * G.len * G.len;
    G.m1 = m / g; G.n1 = n / g; G.o1 = o / g;
    G.S = g > 4 ? 2 : 1;
    G.nx = (g + G.S - 1) / G.S;
    G.nsamp = G.nx * G.nx * g;
    G.alpha1 = alpha1;
    G.eps = eps;
    return G;
}

SoftTree make_tree(const SoftTreeDev& d) {
    SoftTree t;
    t.len = d.len; t.len3 = d.len * d.len * d.len; t.hw = (d.len - 1) / 2; t.sz = d.sz; t.root = d.root;
    t.q = d.q; t.tau = d.tau; t.itau = 1.0f / d.tau;
    t.parents = d.parents; t.edgemst = d.edgemst; t.child_ptr = d.child_ptr; t.children = d.children;
    t.off = d.off; t.offbar = d.offbar;
    return t;
}

}  // namespace

// off (x|y|z) of node c's edge = (prior[parent] - prior[c]) / q; the root has none
__global__ void k_soft_offsets(const float* __restrict__ prior, const int* __restrict__ parents, int root, int sz,
                               float q, float* __restrict__ off) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= sz) return;
    const int p = c == root ? c : parents[c];
#pragma unroll
    for (int a = 0; a < 3; a++) off[a * sz + c] = (prior[a * sz + p] - prior[a * sz + c]) / q;
}

// dL/dprior from dL/doff: each edge's offset depends on its two end nodes
__global__ void k_soft_offbar_to_prior(const float* __restrict__ offbar, const int* __restrict__ parents, int root,
                                       int sz, float q, float* __restrict__ gprior) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= sz || c == root) return;
    const int p = parents[c];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float g = offbar[a * sz + c] / q;
        atomicAdd(gprior + a * sz + p, g);
        atomicAdd(gprior + a * sz + c, -g);
    }
}

// ---------------------------------------------------------------------------
// Host drivers

// three box passes a -> b -> a -> b; the result is in b
template <int R>
static void box3_r(float* a, float* b, int m, int n, int o, int r, cudaStream_t st) {
    const dim3 blk(32, 8), grid(blocks_for(m, 32), blocks_for(n, 8), 6 * o);
    k_soft_box<R><<<grid, blk, 0, st>>>(a, b, m, n, o, r, 0);
    k_soft_box<R><<<grid, blk, 0, st>>>(b, a, m, n, o, r, 1);
    k_soft_box<R><<<grid, blk, 0, st>>>(a, b, m, n, o, r, 2);
}

static void box3(float* a, float* b, int m, int n, int o, int r, cudaStream_t st) {
    switch (r) {
        case 1: box3_r<1>(a, b, m, n, o, r, st); break;
        case 2: box3_r<2>(a, b, m, n, o, r, st); break;
        case 3: box3_r<3>(a, b, m, n, o, r, st); break;
        default: box3_r<0>(a, b, m, n, o, r, st); break;
    }
}

cudaError_t launch_soft_offsets(const float* prior, const int* parents, int root, int sz, float q, float* off,
                                cudaStream_t st) {
    k_soft_offsets<<<blocks_for(sz, 256), 256, 0, st>>>(prior, parents, root, sz, q, off);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_soft_offbar_to_prior(const float* offbar, const int* parents, int root, int sz, float q,
                                        float* gprior, cudaStream_t st) {
    k_soft_offbar_to_prior<<<blocks_for(sz, 256), 256, 0, st>>>(offbar, parents, root, sz, q, gprior);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_soft_descriptor(const float* d_im, float* w6a, float* w6b, float* s12, int m, int n, int o, int qs,
                                   cudaStream_t st) {
    const int64_t sz = (int64_t)m * n * o;
    k_soft_sqdiff<<<blocks_for(sz, 256), 256, 0, st>>>(d_im, w6a, m, n, o, qs);
    box3(w6a, w6b, m, n, o, qs, st);
    k_soft_desc<<<blocks_for(sz, 256), 256, 0, st>>>(w6b, s12, m, n, o, qs);
    count_launches(5);
    return cudaGetLastError();
}

cudaError_t launch_soft_descriptor_adj(const float* d_im, float* w6a, float* w6b, const float* sbar12, float* dbar6,
                                       float* imbar, int m, int n, int o, int qs, cudaStream_t st) {
    const int64_t sz = (int64_t)m * n * o;
    k_soft_sqdiff<<<blocks_for(sz, 256), 256, 0, st>>>(d_im, w6a, m, n, o, qs);
    box3(w6a, w6b, m, n, o, qs, st);
    cudaError_t err = cudaMemsetAsync(dbar6, 0, sizeof(float) * 6 * sz, st);
    if (err != cudaSuccess) return err;
    k_soft_desc_adj<<<blocks_for(sz, 256), 256, 0, st>>>(w6b, sbar12, dbar6, m, n, o, qs);
    box3(dbar6, w6b, m, n, o, qs, st);  // adjoint of the box filter: the same operator
    k_soft_sqdiff_adj<<<blocks_for(sz, 256), 256, 0, st>>>(d_im, w6b, imbar, m, n, o, qs);
    count_launches(9);
    return cudaGetLastError();
}

// Channels per halo stage so that the kernel's shared memory stays within ~110 KB
// (two CTAs per SM); 0 when even one channel does not fit (generic kernels).
static int halo_channels(const SoftGeom& G, int H3max, int arrays, size_t extra_bytes) {
    static const int cands[6] = {12, 6, 4, 3, 2, 1};
    for (int c : cands)
        if ((size_t)arrays * c * H3max * sizeof(float) + extra_bytes + (arrays == 1 ? (size_t)c * G.nsamp * 4 : 0) <=
            110 * 1024)
            return c;
    return 0;
}

static int halo_h3max(const SoftGeom& G) {
    const int R = G.hw * G.q;
    return std::min(G.g + 2 * R, G.m) * std::min(G.g + 2 * R, G.n) * std::min(G.g + 2 * R, G.o);
}

// Column kernels are instantiated for the finest-level shapes (grid 4, quant 1,
// label widths 5/7/9); other shapes use the generic halo kernels.
template <int G_, int LEN_, int Q_>
static cudaError_t run_cost_col(const SoftGeom& G, const float* sF, const float* sM, float* cost, cudaStream_t st) {
    using CGm = ColGeom<G_, LEN_, Q_>;
    const size_t smem = sizeof(float) * (12 * (size_t)CGm::NA3 + 12 * CGm::NSAMP + CGm::LEN3);
    if (smem > 200 * 1024) return cudaErrorNotSupported;
    cudaError_t e = cudaFuncSetAttribute(k_soft_cost_col<G_, LEN_, Q_>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    k_soft_cost_col<G_, LEN_, Q_><<<G.m1 * G.n1 * G.o1, CGm::FWD_BLOCK, smem, st>>>(sF, sM, cost, G);
    return cudaSuccess;
}

template <int G_, int LEN_, int Q_>
static cudaError_t run_cost_adj_col(const SoftGeom& G, const float* sF, const float* sM, const float* cbar,
                                    const float* cost, float* sFbar, float* sMbar, double* dot, cudaStream_t st) {
    using CGm = ColGeom<G_, LEN_, Q_>;
    const size_t smem = sizeof(float) * (2 * kAdjCG * (size_t)CGm::NA3 + 24 * CGm::NSAMP + CGm::LEN3);
    if (smem > 200 * 1024) return cudaErrorNotSupported;
    cudaError_t e = cudaFuncSetAttribute(k_soft_cost_adj_col<G_, LEN_, Q_>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_soft_cost_adj_col<G_, LEN_, Q_><<<G.m1 * G.n1 * G.o1, CGm::ADJ_BLOCK, smem, st>>>(sF, sM, cbar, cost, sFbar,
                                                                                         sMbar, dot, G);
    return cudaSuccess;
}

// Channels per stage of the row kernels: as many as fit in 64 KB of rows.
template <int G_, int LEN_, int Q_>
static RowPlan row_plan() {
    using RG = RowGeom<G_, LEN_, Q_>;
    static const int cands[6] = {12, 6, 4, 3, 2, 1};
    RowPlan P{RG::PY, 1};
    for (int c : cands)
        if ((size_t)c * RG::ITEMS * RG::PY * sizeof(float) <= 64 * 1024) { P.CG = c; break; }
    return P;
}

template <int G_, int LEN_, int Q_>
static cudaError_t run_cost_rows(const SoftGeom& G, const float* sF, const float* sM, float* cost, cudaStream_t st) {
    using RG = RowGeom<G_, LEN_, Q_>;
    const RowPlan P = row_plan<G_, LEN_, Q_>();
    const size_t smem = sizeof(float) * ((size_t)P.CG * RG::ITEMS * RG::PY + 12 * RG::NSAMP + RG::LEN3) +
                        sizeof(int) * RG::ITEMS;
    cudaError_t e = cudaFuncSetAttribute(k_soft_cost_rows<G_, LEN_, Q_>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    k_soft_cost_rows<G_, LEN_, Q_><<<G.m1 * G.n1 * G.o1, RG::BLOCK, smem, st>>>(sF, sM, cost, G, P);
    return cudaSuccess;
}

template <int G_, int LEN_, int Q_>
static cudaError_t run_cost_adjF_rows(const SoftGeom& G, const float* sF, const float* sM, const float* cbar,
                                      const float* cost, float* sFbar, double* dot, cudaStream_t st) {
    using RG = RowGeom<G_, LEN_, Q_>;
    const RowPlan P = row_plan<G_, LEN_, Q_>();
    const size_t smem = sizeof(float) * ((size_t)P.CG * RG::ITEMS * RG::PY + 24 * RG::NSAMP + RG::LEN3) +
                        sizeof(int) * RG::ITEMS;
    cudaError_t e = cudaFuncSetAttribute(k_soft_cost_adjF_rows<G_, LEN_, Q_>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_soft_cost_adjF_rows<G_, LEN_, Q_><<<G.m1 * G.n1 * G.o1, RG::BLOCK, smem, st>>>(sF, sM, cbar, cost, sFbar,
                                                                                      dot, G, P);
    return cudaSuccess;
}

// Row kernels are instantiated for the coarse soft levels in use (grid 6 / quant
// 3 or 2, grid 5 / quant 2, label widths 5 and 7).  Every item stages its own
// row; where two items of a node read the same row (quant 2: x offsets 2jj + 2lx
// repeat) that row is simply staged twice.
static int row_shape(const SoftGeom& G) {
    if (G.len != 5 && G.len != 7) return 0;
    if (G.g == 6 && G.q == 3) return 60 + G.len;
    if (G.g == 6 && G.q == 2) return 600 + G.len;
    if (G.g == 5 && G.q == 2) return 50 + G.len;
    return 0;
}

#define DEEDS_ROW_CASES(FN, ...)                                                   \
    case 65: e = FN<6, 5, 3>(__VA_ARGS__); break;                                  \
    case 67: e = FN<6, 7, 3>(__VA_ARGS__); break;                                  \
    case 605: e = FN<6, 5, 2>(__VA_ARGS__); break;                                 \
    case 607: e = FN<6, 7, 2>(__VA_ARGS__); break;                                 \
    case 55: e = FN<5, 5, 2>(__VA_ARGS__); break;                                  \
    case 57: e = FN<5, 7, 2>(__VA_ARGS__); break;

static int col_shape(const SoftGeom& G) {
    if (G.g != 4 || G.q != 1) return 0;
    return G.len == 5 || G.len == 7 || G.len == 9 ? G.len : 0;
}

cudaError_t launch_soft_cost(const float* sF, const float* sM, float* cost, int m, int n, int o, int g, int hw, int q,
                             float alpha1, float eps, cudaStream_t st) {
    const SoftGeom G = make_geom(m, n, o, g, hw, q, alpha1, eps);
    const int H3max = halo_h3max(G);
    {
        cudaError_t e = cudaErrorNotSupported;
        switch (col_shape(G)) {
            case 5: e = run_cost_col<4, 5, 1>(G, sF, sM, cost, st); break;
            case 7: e = run_cost_col<4, 7, 1>(G, sF, sM, cost, st); break;
            case 9: e = run_cost_col<4, 9, 1>(G, sF, sM, cost, st); break;
            default: break;
        }
        if (e == cudaSuccess) {
            count_launches(1);
            return cudaGetLastError();
        }
        if (e != cudaErrorNotSupported) return e;
    }
    if (const int rs = row_shape(G)) {
        cudaError_t e = cudaErrorNotSupported;
        switch (rs) { DEEDS_ROW_CASES(run_cost_rows, G, sF, sM, cost, st) default: break; }
        if (e != cudaSuccess) return e;
        count_launches(1);
        return cudaGetLastError();
    }
    const size_t extra = sizeof(int) * (size_t)(G.len3 + G.nsamp);
    const int CG = G.len3 <= kHaloLPT * 512 ? halo_channels(G, H3max, 1, extra) : 0;
    if (CG > 0) {
        const size_t smem = sizeof(float) * ((size_t)CG * H3max + (size_t)CG * G.nsamp) + extra;
        cudaError_t e = cudaFuncSetAttribute(k_soft_cost_halo, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        const int threads = std::min(512, (G.len3 + 31) / 32 * 32);
        k_soft_cost_halo<<<G.m1 * G.n1 * G.o1, threads, smem, st>>>(sF, sM, cost, G, CG, H3max);
    } else {
        k_soft_cost<<<G.m1 * G.n1 * G.o1, soft_threads(G.len), sizeof(float) * G.nsamp * 12, st>>>(sF, sM, cost, G);
    }
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_soft_cost_adj(const float* sF, const float* sM, const float* cbar, const float* cost, float* sFbar,
                                 float* sMbar, double* dot, int m, int n, int o, int g, int hw, int q, float alpha1,
                                 float eps, cudaStream_t st) {
    const SoftGeom G = make_geom(m, n, o, g, hw, q, alpha1, eps);
    const int64_t sz = (int64_t)m * n * o;
    cudaError_t err = cudaMemsetAsync(sFbar, 0, sizeof(float) * 12 * sz, st);
    if (err == cudaSuccess) err = cudaMemsetAsync(dot, 0, sizeof(double), st);
    if (err != cudaSuccess) return err;
    if (const int rs = row_shape(G)) {  // fixed side in row form, moving side as a gather (no atomics)
        cudaError_t e = cudaErrorNotSupported;
        switch (rs) { DEEDS_ROW_CASES(run_cost_adjF_rows, G, sF, sM, cbar, cost, sFbar, dot, st) default: break; }
        if (e != cudaSuccess) return e;
        switch (rs) { DEEDS_ROW_CASES(run_adj_moving_t, G, sF, sM, cbar, sMbar, st) default: break; }
        if (e != cudaSuccess) return e;
        count_launches(2);
        return cudaGetLastError();
    }
    const int H3max = halo_h3max(G);
    const size_t extra = sizeof(float) * (size_t)G.len3 + sizeof(int) * (size_t)(G.len3 + G.nsamp);
    const int CG = halo_channels(G, H3max, 2, extra);
    if (col_shape(G) || CG > 0) {
        err = cudaMemsetAsync(sMbar, 0, sizeof(float) * 12 * sz, st);
        if (err != cudaSuccess) return err;
    }
    {
        cudaError_t e = cudaErrorNotSupported;
        switch (col_shape(G)) {
            case 5: e = run_cost_adj_col<4, 5, 1>(G, sF, sM, cbar, cost, sFbar, sMbar, dot, st); break;
            case 7: e = run_cost_adj_col<4, 7, 1>(G, sF, sM, cbar, cost, sFbar, sMbar, dot, st); break;
            case 9: e = run_cost_adj_col<4, 9, 1>(G, sF, sM, cbar, cost, sFbar, sMbar, dot, st); break;
            default: break;
        }
        if (e == cudaSuccess) {
            count_launches(1);
            return cudaGetLastError();
        }
        if (e != cudaErrorNotSupported) return e;
    }
    if (CG > 0) {
        const size_t smem = sizeof(float) * 2 * (size_t)CG * H3max + extra;
        err = cudaFuncSetAttribute(k_soft_cost_adj_halo, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return err;
        k_soft_cost_adj_halo<<<G.m1 * G.n1 * G.o1, 256, smem, st>>>(sF, sM, cbar, cost, sFbar, sMbar, dot, G, CG,
                                                                     H3max);
        count_launches(1);
    } else {
        k_soft_cost_adj_fixed<<<G.m1 * G.n1 * G.o1, 256, 0, st>>>(sF, sM, cbar, cost, sFbar, dot, G);
        k_soft_cost_adj_moving<<<blocks_for(sz, 128), 128, 0, st>>>(sF, sM, cbar, sMbar, G);
        count_launches(2);
    }
    return cudaGetLastError();
}

// Resident sweep CTAs per SM.  A sweep is bound by the latency along the
// deepest root-leaf path (hundreds of nodes at grid 4), and most of its CTAs wait;
// two per SM keep the sweep as fast as a full grid (measured 1-2 % faster at
// 160x160x192, label set 7^3) and leave the rest of each SM to kernels of other
// pairs running on other streams.
constexpr int kSweepCtasPerSm = 2;

size_t soft_tree_smem(int len) { return sizeof(float) * (6 * (size_t)len * len * len + 96); }

template <int KIND>
static cudaError_t run_sweep(const SoftTree& t, const int* ordered, const SweepArgs& a, const SweepState& st,
                             int* sweep_mem, cudaStream_t s) {
    const int threads = tree_threads(t.len);
    const size_t smem = sizeof(float) * ((KIND == kSweepUp || KIND == kSweepDown ? 3 : 6) * (size_t)t.len3 + 96);
    cudaError_t e = cudaFuncSetAttribute(k_soft_sweep<KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, per_sm = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_soft_sweep<KIND>, threads, smem)) != cudaSuccess)
        return e;
    per_sm = std::min(per_sm, kSweepCtasPerSm);
    const int grid = std::max(1, std::min(t.sz, sms * std::max(per_sm, 1)));
    // ticket + per-node flags start at zero (the error word is cleared by the caller)
    if ((e = cudaMemsetAsync(sweep_mem, 0, sizeof(int) * ((size_t)t.sz + 1), s)) != cudaSuccess) return e;
    k_soft_sweep<KIND><<<grid, threads, smem, s>>>(t, ordered, a, st);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_soft_tree_forward(const SoftTreeDev& d, int* sweep_mem, const float* cost, float* B, float* M,
                                     float* Mmin, float* logp, float* disp, cudaStream_t s) {
    const SoftTree t = make_tree(d);
    SweepArgs a{cost, B, M, Mmin, logp, disp, nullptr, nullptr, nullptr};
    const SweepState st{sweep_mem, sweep_mem + 1, sweep_mem + t.sz + 1};
    cudaError_t e = run_sweep<kSweepUp>(t, d.ordered, a, st, sweep_mem, s);
    if (e == cudaSuccess) e = run_sweep<kSweepDown>(t, d.ordered, a, st, sweep_mem, s);
    return e;
}

cudaError_t launch_soft_tree_backward(const SoftTreeDev& d, int* sweep_mem, const float* B, const float* M,
                                      const float* logp, const float* gdisp, float* R, float* Bbar, cudaStream_t s) {
    const SoftTree t = make_tree(d);
    SweepArgs a{nullptr, const_cast<float*>(B), const_cast<float*>(M), nullptr, const_cast<float*>(logp), nullptr,
                gdisp, R, Bbar};
    const SweepState st{sweep_mem, sweep_mem + 1, sweep_mem + t.sz + 1};
    cudaError_t e = run_sweep<kSweepDownAdj>(t, d.ordered, a, st, sweep_mem, s);
    if (e == cudaSuccess) e = run_sweep<kSweepUpAdj>(t, d.ordered, a, st, sweep_mem, s);
    return e;
}

// Self-test of the sweeps' bounded wait: one thread waits on a flag that nothing
// sets; status = 1 if the wait gave up and set the error word, 2 otherwise.
__global__ void k_selftest_flag_wait(const int* flag, int* err, int* status) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *status = bounded_wait_geq(flag, 1, err) ? 2 : 1;
}

cudaError_t launch_selftest_flag_wait(const int* flag, int* err, int* status, cudaStream_t s) {
    k_selftest_flag_wait<<<1, 32, 0, s>>>(flag, err, status);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace deeds
