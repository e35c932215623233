// Tree belief propagation on sm_103a (replaces regularisationCL + messageDT,
// src/regularisation.h:6-303).
//
// Upward sweep (leaves to root).  The reference walks breadth levels from the
// deepest up; per level it scales each child's row by its edge weight, runs the
// separable quadratic min-convolution (messageDT) and then, serially in MST
// ordering order, adds (message - min(message)) into the parent's row
// (:190-238).  Here one work item is one PARENT: a persistent grid claims items
// in deepest-first order with an atomic counter; an item first waits (bounded
// spin) until every child that is itself a parent has been finished, then
// processes its children in ordering order entirely in shared memory — scale,
// y/x/z min-convolution passes with the reference's strict '<' (first minimiser
// wins), block min, and the in-order accumulation into the parent's row — and
// finally publishes its own row.  Because a parent only waits on items claimed
// before it by CTAs that are already running, the schedule cannot deadlock at
// any grid size.  Children's rows are left holding their messages, as the
// reference leaves costall.
//
// Downward pass (root to leaves, :258-293): one CTA per tree picks the root's
// first minimum and then resolves one breadth level per step from the argmin
// tables (allinds).
//
// Roofline: dependency/latency bound; algorithmic traffic is one read and one
// write of the cost volume plus the int16 argmin tables.
#include "common.cuh"
#include "kernels.h"

namespace deeds {

namespace {

constexpr int kBpThreads = 256;
constexpr long long kSpinLimit = 1LL << 22;  // x ~256 ns sleep ~= 1 s before giving up

__device__ __forceinline__ float ld_cg(const float* p) { return __ldcg(p); }

// One axis pass of the min-convolution over a len^3 block held in shared memory.
// For every output position, the minimum over source positions s along the axis
// of in[base + s*stride] + zt[pos - s + len], first minimiser kept.
// `idx_in` maps a source position to the label chain so far (nullptr for the
// first pass, whose chain is the position itself).
__device__ __forceinline__ void dt_pass(const float* in, float* out, const short* idx_in, short* idx_out,
                                        const float* zt, int len, int axis) {
    const int len2 = len * len, len3 = len2 * len;
    const int stride = axis == 0 ? 1 : (axis == 1 ? len : len2);
    for (int l = threadIdx.x; l < len3; l += blockDim.x) {
        const int pos = axis == 0 ? l % len : (axis == 1 ? (l / len) % len : l / len2);
        const int base = l - pos * stride;
        float best = in[base] + zt[pos + len];
        int bs = 0;
        for (int s = 0; s < len; s++) {
            const float c = in[base + s * stride] + zt[pos - s + len];
            if (c < best) { best = c; bs = s; }
        }
        out[l] = best;
        idx_out[l] = idx_in ? idx_in[base + bs * stride] : (short)(base + bs * stride);
    }
}

__device__ __forceinline__ void fill_parabola(float* zt, int len, float off) {
    for (int t = threadIdx.x; t < 2 * len; t += blockDim.x) {
        const float d = (float)(t - len) + off;
        zt[t] = d * d;
    }
}

__device__ float block_min(float v, float* red) {
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < (int)(blockDim.x >> 5) ? red[lane] : INFINITY;
        for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0) red[0] = v;
    }
    __syncthreads();
    const float r = red[0];
    return r;
}

__global__ void __launch_bounds__(kBpThreads) k_bp_up(BpTree t, float* __restrict__ cost, short* __restrict__ allinds,
                                                      int* __restrict__ work, int* __restrict__ flags, int epoch,
                                                      int* __restrict__ err) {
    extern __shared__ float smem[];
    const int len = t.len, len2 = len * len, len3 = len2 * len;
    float* prow = smem;
    float* A = prow + len3;
    float* B = A + len3;
    float* zt = B + len3;            // 2*len
    float* red = zt + 2 * len + 2;   // 32
    short* ia = reinterpret_cast<short*>(red + 32);
    short* ib = ia + len3;
    __shared__ int s_item;
    __shared__ int s_abort;
    for (;;) {
        if (threadIdx.x == 0) {
            s_item = atomicAdd(work, 1);
            s_abort = *(volatile int*)err != 0;
        }
        __syncthreads();
        const int it = s_item;
        if (it >= t.n_up || s_abort) return;
        const int p = t.up_nodes[it];
        const float up0 = t.u0[p], vp0 = t.v0[p], wp0 = t.w0[p];
        for (int l = threadIdx.x; l < len3; l += blockDim.x) prow[l] = ld_cg(cost + (int64_t)p * len3 + l);
        for (int ci = t.child_ptr[it]; ci < t.child_ptr[it + 1]; ci++) {
            const int c = t.children[ci];
            const int wi = t.wait_idx[c];
            if (threadIdx.x == 0 && wi >= 0) {
                long long spins = 0;
                while (*(volatile int*)(flags + wi) != epoch) {
                    if (++spins > kSpinLimit || *(volatile int*)err != 0) {
                        atomicCAS(err, 0, 1);
                        s_abort = 1;
                        break;
                    }
                    __nanosleep(256);
                }
                __threadfence();
            }
            __syncthreads();
            if (s_abort) return;
            const float e = t.edgemst[c];
            const float* crow = cost + (int64_t)c * len3;
            for (int l = threadIdx.x; l < len3; l += blockDim.x) A[l] = __fmul_rn(ld_cg(crow + l), e);
            const float ox = __fdiv_rn(up0 - t.u0[c], t.q);
            const float oy = __fdiv_rn(vp0 - t.v0[c], t.q);
            const float oz = __fdiv_rn(wp0 - t.w0[c], t.q);
            fill_parabola(zt, len, oy);
            __syncthreads();
            dt_pass(A, B, nullptr, ia, zt, len, 0);
            __syncthreads();
            fill_parabola(zt, len, ox);
            __syncthreads();
            dt_pass(B, A, ia, ib, zt, len, 1);
            __syncthreads();
            fill_parabola(zt, len, oz);
            __syncthreads();
            dt_pass(A, B, ib, ia, zt, len, 2);  // message in B, argmin chain in ia
            __syncthreads();
            float mn = INFINITY;
            for (int l = threadIdx.x; l < len3; l += blockDim.x) {
                const float v = B[l];
                mn = fminf(mn, v);
                cost[(int64_t)c * len3 + l] = v;
                allinds[(int64_t)c * len3 + l] = ia[l];
            }
            mn = block_min(mn, red);
            for (int l = threadIdx.x; l < len3; l += blockDim.x) prow[l] = prow[l] + (B[l] - mn);
            // the next child's passes overwrite A/B/ia/zt only after this barrier
            __syncthreads();
        }
        for (int l = threadIdx.x; l < len3; l += blockDim.x) cost[(int64_t)p * len3 + l] = prow[l];
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            atomicExch(flags + it, epoch);
        }
    }
}

// Root argmin (first minimum) and breadth-level backtrack for one tree per CTA.
__global__ void __launch_bounds__(1024) k_bp_down(BpTree t, const float* __restrict__ cost,
                                                 short* __restrict__ allinds, int* __restrict__ sel,
                                                 float* __restrict__ u1, float* __restrict__ v1,
                                                 float* __restrict__ w1, int* __restrict__ err) {
    __shared__ float s_val[32];
    __shared__ int s_idx[32];
    // the argmin tables are only valid if the upward pass completed
    if (*(volatile int*)err != 0) return;
    const int len = t.len, len3 = len * len * len, hw = (len - 1) / 2;
    const int root = t.ordered[0];
    const float* rr = cost + (int64_t)root * len3;
    float bv = INFINITY;
    int bi = 0x7fffffff;
    for (int l = threadIdx.x; l < len3; l += blockDim.x) {
        const float v = __ldcg(rr + l);
        if (v < bv || (v == bv && l < bi)) { bv = v; bi = l; }
        allinds[(int64_t)root * len3 + l] = (short)l;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov < bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { s_val[w] = bv; s_idx[w] = bi; }
    __syncthreads();
    if (w == 0) {
        bv = lane < (int)(blockDim.x >> 5) ? s_val[lane] : INFINITY;
        bi = lane < (int)(blockDim.x >> 5) ? s_idx[lane] : 0x7fffffff;
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov < bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
        }
        if (lane == 0) {
            sel[root] = bi;
            const int i = bi % len, j = (bi / len) % len, k = bi / (len * len);
            u1[root] = (float)(j - hw) * t.q + t.u0[root];
            v1[root] = (float)(i - hw) * t.q + t.v0[root];
            w1[root] = (float)(k - hw) * t.q + t.w0[root];
        }
    }
    __syncthreads();
    for (int lev = 1; lev < t.n_levels; lev++) {
        const int b = t.level_start[lev], e = t.level_start[lev + 1];
        for (int ti = b + threadIdx.x; ti < e; ti += blockDim.x) {
            const int c = t.ordered[ti];
            const int p = t.parents[c];
            int l = allinds[(int64_t)c * len3 + sel[p]];
            if (l < 0 || l >= len3) {  // never for a completed upward pass; keeps reads in bounds
                atomicCAS(err, 0, 2);
                l = 0;
            }
            sel[c] = l;
            const int i = l % len, j = (l / len) % len, k = l / (len * len);
            u1[c] = (float)(j - hw) * t.q + t.u0[c];
            v1[c] = (float)(i - hw) * t.q + t.v0[c];
            w1[c] = (float)(k - hw) * t.q + t.w0[c];
        }
        __syncthreads();
    }
}

}  // namespace

size_t bp_up_smem_bytes(int len) {
    const size_t len3 = (size_t)len * len * len;
    return (3 * len3 + 2 * len + 2 + 32) * sizeof(float) + 2 * len3 * sizeof(short);
}

cudaError_t launch_bp_up(const BpTree& t, float* d_cost, short* d_allinds, int* d_work, int* d_flags, int epoch,
                         int* d_err, int max_ctas, cudaStream_t s) {
    if (t.n_up <= 0) return cudaSuccess;
    const size_t smem = bp_up_smem_bytes(t.len);
    cudaError_t e = cudaFuncSetAttribute(k_bp_up, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(d_work, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    const int ctas = t.n_up < max_ctas ? t.n_up : max_ctas;
    k_bp_up<<<ctas, kBpThreads, smem, s>>>(t, d_cost, d_allinds, d_work, d_flags, epoch, d_err);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_bp_down(const BpTree& t, const float* d_cost, short* d_allinds, int* d_sel, float* d_u1,
                           float* d_v1, float* d_w1, int* d_err, cudaStream_t s) {
    k_bp_down<<<1, 1024, 0, s>>>(t, d_cost, d_allinds, d_sel, d_u1, d_v1, d_w1, d_err);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace deeds
