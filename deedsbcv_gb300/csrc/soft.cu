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
// kernel is its own adjoint.
__global__ void k_soft_box(const float* __restrict__ in, float* __restrict__ out, int m, int n, int o, int r, int axis) {
    const int64_t mn = (int64_t)m * n, sz = mn * o;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 6 * sz) return;
    const int64_t p = t % sz;
    int L, i;
    int64_t stride;
    if (axis == 0) { L = m; stride = 1; i = (int)(p % m); }
    else if (axis == 1) { L = n; stride = m; i = (int)((p / m) % n); }
    else { L = o; stride = mn; i = (int)(p / mn); }
    const float* x = in + (t - (int64_t)i * stride);
    const int a0 = max(0, i - r), a1 = min(L - 1, i + r);
    float acc = 0.0f;
    for (int a = a0; a <= a1; a++) acc += x[a * stride];
    out[t] = acc;
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

// ---------------------------------------------------------------------------
// Tree sweeps

struct SoftTree {
    int len, len3, hw, sz, root, q;
    float tau, itau;
    const int* parents;
    const float* edgemst;
    const int* child_ptr;
    const int* children;
};

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

// out(o) = LSE_a in(line(o), a) - (a - b)^2/tau along the axis of stride s (b = o's
// coordinate on that axis).  Ends with a barrier.
__device__ void lse_axis(const float* in, float* out, int len, int len3, int s, float itau) {
    for (int o = threadIdx.x; o < len3; o += blockDim.x) {
        const int b = (o / s) % len;
        const float* line = in + (o - b * s);
        float mx = -INFINITY;
        for (int a = 0; a < len; a++) {
            const float d = (float)(a - b);
            mx = fmaxf(mx, line[a * s] - d * d * itau);
        }
        float acc = 0.0f;
        for (int a = 0; a < len; a++) {
            const float d = (float)(a - b);
            acc += expf(line[a * s] - d * d * itau - mx);
        }
        out[o] = mx + logf(acc);
    }
    __syncthreads();
}

// adjoint of one pass: inbar(a) = sum_b outbar(b) exp(in(a) - (a-b)^2/tau - out(b))
__device__ void lse_axis_adj(const float* in, const float* out, const float* outbar, float* inbar, int len, int len3,
                             int s, float itau) {
    for (int o = threadIdx.x; o < len3; o += blockDim.x) {
        const int a = (o / s) % len;
        const int base = o - a * s;
        const float x = in[o];
        float acc = 0.0f;
        for (int b = 0; b < len; b++) {
            const float d = (float)(a - b);
            acc += outbar[base + b * s] * expf(x - d * d * itau - out[base + b * s]);
        }
        inbar[o] = acc;
    }
    __syncthreads();
}

// S = pass z o pass x o pass y; keeps t1, t2 for the adjoint (out may alias in)
__device__ __forceinline__ void sep_lse(const float* in, float* t1, float* t2, float* out, int len, int len3,
                                        float itau) {
    lse_axis(in, t1, len, len3, 1, itau);
    lse_axis(t1, t2, len, len3, len, itau);
    lse_axis(t2, out, len, len3, len * len, itau);
}

// inbar = S^T outbar.  wa is scratch; wb may alias outbar and inbar may alias wa.
__device__ __forceinline__ void sep_lse_adj(const float* in, const float* t1, const float* t2, const float* out,
                                            const float* outbar, float* wa, float* wb, float* inbar, int len,
                                            int len3, float itau) {
    lse_axis_adj(t2, out, outbar, wa, len, len3, len * len, itau);
    lse_axis_adj(t1, t2, wa, wb, len, len3, len, itau);
    lse_axis_adj(in, t1, wb, inbar, len, len3, 1, itau);
}

// Upward sweep over one breadth level (one CTA per node).
__global__ void k_soft_up_level(SoftTree t, const int* __restrict__ nodes, const float* __restrict__ cost,
                                float* __restrict__ B, float* __restrict__ M, float* __restrict__ Mmin) {
    extern __shared__ float sh[];
    const int L3 = t.len3;
    float* f = sh;
    float* t1 = sh + L3;
    float* t2 = sh + 2 * L3;
    float* red = sh + 3 * L3;
    const int c = nodes[blockIdx.x];
    const float e = c == t.root ? 0.0f : t.edgemst[c];
    const int k0 = t.child_ptr[c], k1 = t.child_ptr[c + 1];
    float bmin = INFINITY;
    for (int l = threadIdx.x; l < L3; l += blockDim.x) {
        float v = cost[(int64_t)c * L3 + l];
        for (int ci = k0; ci < k1; ci++) {
            const int k = t.children[ci];
            v += M[(int64_t)k * L3 + l] - Mmin[k];
        }
        f[l] = v;
        bmin = fminf(bmin, v);
    }
    // Beliefs are stored minus their minimum: the marginals and the parent's
    // (message - min) are invariant to a constant shift of B_c, and the centred
    // values keep the exponents of the label-space transforms small where the
    // probability mass is.
    bmin = -block_max(-bmin, red);
    for (int l = threadIdx.x; l < L3; l += blockDim.x) {
        const float v = f[l] - bmin;
        B[(int64_t)c * L3 + l] = v;
        f[l] = -e * v * t.itau;
    }
    __syncthreads();
    if (c == t.root) return;
    sep_lse(f, t1, t2, f, t.len, L3, t.itau);
    float mn = INFINITY;
    for (int lp = threadIdx.x; lp < L3; lp += blockDim.x) {
        const float msg = -t.tau * f[lp];
        M[(int64_t)c * L3 + lp] = msg;
        mn = fminf(mn, msg);
    }
    mn = -block_max(-mn, red);
    if (threadIdx.x == 0) Mmin[c] = mn;
}

// Downward marginals over one breadth level; writes log p and the expected displacement.
__global__ void k_soft_down_level(SoftTree t, const int* __restrict__ nodes, const float* __restrict__ B,
                                  const float* __restrict__ M, float* __restrict__ logp, float* __restrict__ disp) {
    extern __shared__ float sh[];
    const int L3 = t.len3, len = t.len;
    float* r = sh;
    float* t1 = sh + L3;
    float* t2 = sh + 2 * L3;
    float* red = sh + 3 * L3;
    const int c = nodes[blockIdx.x];
    float* lc = logp + (int64_t)c * L3;
    const float* bc = B + (int64_t)c * L3;
    if (c == t.root) {
        float mx = -INFINITY;
        for (int l = threadIdx.x; l < L3; l += blockDim.x) mx = fmaxf(mx, -bc[l] * t.itau);
        mx = block_max(mx, red);
        float s = 0.0f;
        for (int l = threadIdx.x; l < L3; l += blockDim.x) s += expf(-bc[l] * t.itau - mx);
        s = block_sum(s, red);
        const float lz = mx + logf(s);
        for (int l = threadIdx.x; l < L3; l += blockDim.x) r[l] = -bc[l] * t.itau - lz;
        __syncthreads();
    } else {
        const int p = t.parents[c];
        const float e = t.edgemst[c];
        for (int lp = threadIdx.x; lp < L3; lp += blockDim.x)
            r[lp] = logp[(int64_t)p * L3 + lp] + M[(int64_t)c * L3 + lp] * t.itau;
        __syncthreads();
        sep_lse(r, t1, t2, r, len, L3, t.itau);
        // log p_c is normalised in exact arithmetic; renormalising stops float
        // rounding from drifting along root-to-leaf paths (no effect on the exact
        // gradient, whose parameter derivatives are tangent to the normalised set)
        float mx = -INFINITY;
        for (int l = threadIdx.x; l < L3; l += blockDim.x) {
            r[l] += -e * bc[l] * t.itau;
            mx = fmaxf(mx, r[l]);
        }
        mx = block_max(mx, red);
        float s = 0.0f;
        for (int l = threadIdx.x; l < L3; l += blockDim.x) s += expf(r[l] - mx);
        s = block_sum(s, red);
        const float lz = mx + logf(s);
        for (int l = threadIdx.x; l < L3; l += blockDim.x) r[l] -= lz;
        __syncthreads();
    }
    float eu = 0.0f, ev = 0.0f, ew = 0.0f;
    for (int l = threadIdx.x; l < L3; l += blockDim.x) {
        lc[l] = r[l];
        const float pl = expf(r[l]);
        eu += pl * (float)(((l / len) % len - t.hw) * t.q);
        ev += pl * (float)((l % len - t.hw) * t.q);
        ew += pl * (float)((l / (len * len) - t.hw) * t.q);
    }
    eu = block_sum(eu, red);
    ev = block_sum(ev, red);
    ew = block_sum(ew, red);
    if (threadIdx.x == 0) {
        disp[c] = eu;
        disp[t.sz + c] = ev;
        disp[2 * t.sz + c] = ew;
    }
}

// Adjoint of the marginals over one breadth level (run leaves to root).
//   h(l) = gE_c . d(l) p_c(l) + sum_children R_k(l)    (= dL/dlog p_c)
//   Bbar_c = -e h/tau (root: -(h - p sum h)/tau);  R_c = S^T h w.r.t. r
__global__ void k_soft_down_adj_level(SoftTree t, const int* __restrict__ nodes, const float* __restrict__ M,
                                      const float* __restrict__ logp, const float* __restrict__ gdisp,
                                      float* __restrict__ R, float* __restrict__ Bbar) {
    extern __shared__ float sh[];
    const int L3 = t.len3, len = t.len;
    float* r = sh;
    float* t1 = sh + L3;
    float* t2 = sh + 2 * L3;
    float* G = sh + 3 * L3;
    float* h = sh + 4 * L3;
    float* wa = sh + 5 * L3;
    float* red = sh + 6 * L3;
    const int c = nodes[blockIdx.x];
    const float* lc = logp + (int64_t)c * L3;
    const float gu = gdisp[c], gv = gdisp[t.sz + c], gw = gdisp[2 * t.sz + c];
    const int k0 = t.child_ptr[c], k1 = t.child_ptr[c + 1];
    float tot = 0.0f;
    for (int l = threadIdx.x; l < L3; l += blockDim.x) {
        const float du = (float)(((l / len) % len - t.hw) * t.q), dv = (float)((l % len - t.hw) * t.q),
                    dw = (float)((l / (len * len) - t.hw) * t.q);
        float v = (gu * du + gv * dv + gw * dw) * expf(lc[l]);
        for (int ci = k0; ci < k1; ci++) v += R[(int64_t)t.children[ci] * L3 + l];
        h[l] = v;
        tot += v;
    }
    float* bb = Bbar + (int64_t)c * L3;
    if (c == t.root) {
        tot = block_sum(tot, red);
        float mean = 0.0f;
        for (int l = threadIdx.x; l < L3; l += blockDim.x) {
            wa[l] = -(h[l] - expf(lc[l]) * tot) * t.itau;
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
        r[l] = logp[(int64_t)p * L3 + l] + M[(int64_t)c * L3 + l] * t.itau;
    }
    __syncthreads();
    sep_lse(r, t1, t2, G, len, L3, t.itau);
    sep_lse_adj(r, t1, t2, G, h, wa, h, wa, len, L3, t.itau);
    float* rc = R + (int64_t)c * L3;
    for (int l = threadIdx.x; l < L3; l += blockDim.x) rc[l] = wa[l];
}

// Adjoint of the upward recursion over one breadth level (run root to leaves, root
// excluded): Mbar_c = R_c/tau + Bbar_parent; M_c = -tau S(f), f = -e B_c/tau, so
// dL/dB_c += -e/tau S^T(-tau Mbar_c) = e S^T(Mbar_c).  Bbar_c is final afterwards (= cbar_c).
__global__ void k_soft_up_adj_level(SoftTree t, const int* __restrict__ nodes, const float* __restrict__ B,
                                    const float* __restrict__ R, float* __restrict__ Bbar) {
    extern __shared__ float sh[];
    const int L3 = t.len3, len = t.len;
    float* f = sh;
    float* t1 = sh + L3;
    float* t2 = sh + 2 * L3;
    float* out = sh + 3 * L3;
    float* mb = sh + 4 * L3;
    float* wa = sh + 5 * L3;
    float* red = sh + 6 * L3;
    const int c = nodes[blockIdx.x];
    const int p = t.parents[c];
    const float e = t.edgemst[c];
    for (int l = threadIdx.x; l < L3; l += blockDim.x) {
        f[l] = -e * B[(int64_t)c * L3 + l] * t.itau;
        mb[l] = R[(int64_t)c * L3 + l] * t.itau + Bbar[(int64_t)p * L3 + l];
    }
    __syncthreads();
    sep_lse(f, t1, t2, out, len, L3, t.itau);
    sep_lse_adj(f, t1, t2, out, mb, wa, mb, wa, len, L3, t.itau);
    // the exact dL/dB_c sums to zero over labels (shift invariance); projecting
    // keeps rounding from accumulating as a common mode down the tree
    float* bb = Bbar + (int64_t)c * L3;
    float mean = 0.0f;
    for (int l = threadIdx.x; l < L3; l += blockDim.x) {
        wa[l] = bb[l] + e * wa[l];
        mean += wa[l];
    }
    mean = block_sum(mean, red) / (float)L3;
    for (int l = threadIdx.x; l < L3; l += blockDim.x) bb[l] = wa[l] - mean;
}

int soft_threads(int len) { return len * len * len <= 343 ? 128 : 256; }

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
    return t;
}

}  // namespace

// ---------------------------------------------------------------------------
// Host drivers

// three box passes a -> b -> a -> b; the result is in b
static void box3(float* a, float* b, int m, int n, int o, int r, cudaStream_t st) {
    const int64_t n6 = (int64_t)6 * m * n * o;
    k_soft_box<<<blocks_for(n6, 256), 256, 0, st>>>(a, b, m, n, o, r, 0);
    k_soft_box<<<blocks_for(n6, 256), 256, 0, st>>>(b, a, m, n, o, r, 1);
    k_soft_box<<<blocks_for(n6, 256), 256, 0, st>>>(a, b, m, n, o, r, 2);
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

cudaError_t launch_soft_cost(const float* sF, const float* sM, float* cost, int m, int n, int o, int g, int hw, int q,
                             float alpha1, float eps, cudaStream_t st) {
    const SoftGeom G = make_geom(m, n, o, g, hw, q, alpha1, eps);
    k_soft_cost<<<G.m1 * G.n1 * G.o1, soft_threads(G.len), sizeof(float) * G.nsamp * 12, st>>>(sF, sM, cost, G);
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
    k_soft_cost_adj_fixed<<<G.m1 * G.n1 * G.o1, 256, 0, st>>>(sF, sM, cbar, cost, sFbar, dot, G);
    k_soft_cost_adj_moving<<<blocks_for(sz, 128), 128, 0, st>>>(sF, sM, cbar, sMbar, G);
    count_launches(2);
    return cudaGetLastError();
}

size_t soft_tree_smem(int len) { return sizeof(float) * (6 * (size_t)len * len * len + 32); }

cudaError_t launch_soft_tree_forward(const SoftTreeDev& d, const int* h_level_start, int n_levels, const float* cost,
                                     float* B, float* M, float* Mmin, float* logp, float* disp, cudaStream_t st) {
    const SoftTree t = make_tree(d);
    const size_t smem = sizeof(float) * (3 * (size_t)t.len3 + 32);
    const int nt = soft_threads(t.len);
    for (int lev = n_levels - 1; lev >= 0; lev--) {
        const int b = h_level_start[lev], e = h_level_start[lev + 1];
        k_soft_up_level<<<e - b, nt, smem, st>>>(t, d.ordered + b, cost, B, M, Mmin);
    }
    for (int lev = 0; lev < n_levels; lev++) {
        const int b = h_level_start[lev], e = h_level_start[lev + 1];
        k_soft_down_level<<<e - b, nt, smem, st>>>(t, d.ordered + b, B, M, logp, disp);
    }
    count_launches(2 * n_levels);
    return cudaGetLastError();
}

cudaError_t launch_soft_tree_backward(const SoftTreeDev& d, const int* h_level_start, int n_levels, const float* B,
                                      const float* M, const float* logp, const float* gdisp, float* R, float* Bbar,
                                      cudaStream_t st) {
    const SoftTree t = make_tree(d);
    const size_t smem = soft_tree_smem(t.len);
    const int nt = soft_threads(t.len);
    for (int lev = n_levels - 1; lev >= 0; lev--) {
        const int b = h_level_start[lev], e = h_level_start[lev + 1];
        k_soft_down_adj_level<<<e - b, nt, smem, st>>>(t, d.ordered + b, M, logp, gdisp, R, Bbar);
    }
    for (int lev = 1; lev < n_levels; lev++) {
        const int b = h_level_start[lev], e = h_level_start[lev + 1];
        k_soft_up_adj_level<<<e - b, nt, smem, st>>>(t, d.ordered + b, B, R, Bbar);
    }
    count_launches(2 * n_levels - 1);
    return cudaGetLastError();
}

}  // namespace deeds
