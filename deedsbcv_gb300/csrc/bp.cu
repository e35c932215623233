// Tree belief propagation on sm_103a (replaces regularisationCL + messageDT,
// src/regularisation.h:6-303).
//
// Upward sweep (leaves to root).  The reference walks breadth levels from the
// deepest up: per level it scales each node's row by its edge weight, runs the
// separable quadratic min-convolution (messageDT, :6-113) and then, serially in
// MST ordering order, adds (message - min(message)) into the parent's row
// (:190-238).  The same arithmetic is scheduled here as a wait-free bottom-up
// reduction: a persistent grid claims leaves (deepest first) from an atomic
// counter; a CTA computes its node's message entirely in shared memory, stores
// it with its minimum, and increments the parent's arrival counter.  The CTA
// that completes a parent's set of children — the last arriver — builds the
// parent's row from its data cost plus every child's (message - min) in MST
// ordering order (the reference's rounding sequence) and continues upward with
// the parent's own message.  No CTA ever waits for another, so there is no
// spin loop and no deadlock at any grid size; the critical path is one
// message per tree level.  Children's rows are left holding their messages and
// the root row its total, as the reference leaves costall.
//
// The distance transform of a len^3 block is three axis passes; a thread owns
// a run of consecutive outputs of one line, holds the line's len values and the
// parabola values it needs in registers and scans all len candidates per output
// (fully unrolled for the compile-time label width), keeping the reference's
// strict '<' so the first minimiser wins.
//
// Downward pass (root to leaves, :258-293): warps across the GPU walk heavy-path
// chains (each follows the child with the deepest subtree) from the argmin
// tables staged ahead in shared memory, publishing every node's label for the
// chains that branch off it; no barrier per breadth level.
//
// Roofline: dependency bound (tree depth 265-987 per tree at 192x160x256).
// Algorithmic traffic: one read + one write of the cost volume and one write of
// the int16 argmin tables per tree.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace deeds {

namespace {

__device__ __forceinline__ float ld_cg(const float* p) { return __ldcg(p); }

// Loads issued where they stand: volatile asm with a memory clobber is not moved
// by the compiler, so a load meant to run ahead (its value used steps or passes
// later) is not sunk next to its use.  .nc for the tree arrays (read-only for the
// whole kernel), .cg for cost rows (written by other CTAs of the kernel).
__device__ __forceinline__ int ld_ahead(const int* p) {
    int v;
    asm volatile("ld.global.nc.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ float ld_ahead(const float* p) {
    float v;
    asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ float ld_ahead_cg(const float* p) {
    float v;
    asm volatile("ld.global.cg.f32 %0, [%1];" : "=f"(v) : "l"(p) : "memory");
    return v;
}

// Arrival counter increment with release and acquire semantics at GPU scope: the
// CTA's earlier writes (made visible to this thread by the preceding barrier) are
// released to whoever later observes the count, and this thread acquires every
// sibling's released writes; a following barrier passes them on to the CTA.
__device__ __forceinline__ int atom_add_acq_rel(int* p, int v) {
    int old;
    asm volatile("atom.add.acq_rel.gpu.s32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

// A pass's LEN^2 lines are split into bp_parts(LEN) parts of consecutive
// outputs, one thread per (line, part): one thread per line left a single warp
// per scheduler at small label widths, and the passes ran latency-bound along
// each line's compare chains.  Parts occupy separate whole-warp ranges of the
// block, so the part index is warp-uniform and each part's output range is a
// compile-time constant (its parabola values stay in registers).
// Children of a parent held in registers by the chain step (a node of the
// 6-connected grid has at most 6 children; more would be read from memory).
constexpr int kKidRegs = 6;

constexpr int bp_line_slots(int len) { return (len * len + 31) / 32 * 32; }

constexpr int bp_parts(int len) {
    // about three outputs per thread, at most 768 threads (registers); one part
    // above 17 and below 7 labels per axis
    return len >= 19 || len < 7
               ? 1
               : ((len + 2) / 3 < 768 / bp_line_slots(len) ? (len + 2) / 3 : 768 / bp_line_slots(len));
}

constexpr int bp_threads(int len) {
    return bp_parts(len) * bp_line_slots(len) < 64 ? 64 : bp_parts(len) * bp_line_slots(len);
}

// Outputs [I0, I1) of one line: out[i] = min_s in[s] + (i - s + off)^2, the
// first minimiser on ties (strict '<', as the reference).
template <int LEN, int AXIS, int I0, int I1>
__device__ __forceinline__ void dt_part(const float* in, float* out, const short* idx_in, short* idx_out, float off,
                                        int base) {
    constexpr int STRIDE = AXIS == 0 ? 1 : (AXIS == 1 ? LEN : LEN * LEN);
    float v[LEN];
#pragma unroll
    for (int s = 0; s < LEN; s++) v[s] = in[base + s * STRIDE];
    float z[2 * LEN];  // z[u] = (u - LEN + off)^2 for the u = i - s + LEN this part reads
#pragma unroll
    for (int u = I0 + 1; u < I1 + LEN; u++) {
        const float d = (float)(u - LEN) + off;
        z[u] = d * d;
    }
#pragma unroll
    for (int i = I0; i < I1; i++) {
        float best = v[0] + z[i + LEN];
        int bs = 0;
#pragma unroll
        for (int s = 1; s < LEN; s++) {
            const float c = v[s] + z[i - s + LEN];
            if (c < best) { best = c; bs = s; }
        }
        out[base + i * STRIDE] = best;
        idx_out[base + i * STRIDE] = idx_in ? idx_in[base + bs * STRIDE] : (short)(base + bs * STRIDE);
    }
}

template <int LEN, int AXIS, int P>
__device__ __forceinline__ void dt_dispatch(int part, const float* in, float* out, const short* idx_in,
                                            short* idx_out, float off, int base) {
    constexpr int K = bp_parts(LEN), OPP = (LEN + K - 1) / K;
    if constexpr (P < K) {
        if (part == P) {
            constexpr int I0 = P * OPP, I1 = (P + 1) * OPP < LEN ? (P + 1) * OPP : LEN;
            if constexpr (I0 < I1) dt_part<LEN, AXIS, I0, I1>(in, out, idx_in, idx_out, off, base);
            return;
        }
        dt_dispatch<LEN, AXIS, P + 1>(part, in, out, idx_in, idx_out, off, base);
    }
}

// One axis pass of the min-convolution: out[line, i] = min_s in[line, s] + (i - s + off)^2.
template <int LEN, int AXIS>
__device__ __forceinline__ void dt_lines(const float* in, float* out, const short* idx_in, short* idx_out,
                                         float off) {
    constexpr int LEN2 = LEN * LEN, LP = bp_line_slots(LEN);
    const int part = threadIdx.x / LP, line = threadIdx.x - part * LP;
    if (line >= LEN2) return;
    const int base = AXIS == 0 ? line * LEN : (AXIS == 1 ? (line % LEN) + (line / LEN) * LEN2 : line);
    dt_dispatch<LEN, AXIS, 0>(part, in, out, idx_in, idx_out, off, base);
}

// Three-input minimum (PTX min.f32 with three sources, sm_100 and later): like
// fminf, a NaN source is ignored unless all are NaN.
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Minimum of N values as a tree of three-input minima (depth log3 N instead of
// the N-long compare chain of a sequential scan).
template <int N>
__device__ __forceinline__ float min_all(const float* c) {
    if constexpr (N == 1) {
        return c[0];
    } else if constexpr (N == 2) {
        return fminf(c[0], c[1]);
    } else {
        constexpr int M = (N + 2) / 3;
        float t[M];
#pragma unroll
        for (int g = 0; g < M; g++) {
            if (3 * g + 2 < N) t[g] = fmin3(c[3 * g], c[3 * g + 1], c[3 * g + 2]);
            else if (3 * g + 1 < N) t[g] = fminf(c[3 * g], c[3 * g + 1]);
            else t[g] = c[3 * g];
        }
        return min_all<M>(t);
    }
}

// Outputs [I0, I1) of one line, values only: out[i] = min_s in[s] + (i - s + off)^2.
// The minimum of the candidates is the value the reference's strict-'<' scan ends
// with (which candidate attains it does not change the value; costs are never
// -0).  NaN: the scan starts from candidate 0 and never replaces a NaN start, so a
// NaN candidate 0 is the result; later NaN candidates never win (as in fminf).
template <int LEN, int AXIS, int I0, int I1>
__device__ __forceinline__ void dt_part_val(const float* in, float* out, float off, int base) {
    constexpr int STRIDE = AXIS == 0 ? 1 : (AXIS == 1 ? LEN : LEN * LEN);
    float v[LEN];
#pragma unroll
    for (int s = 0; s < LEN; s++) v[s] = in[base + s * STRIDE];
    float z[2 * LEN];
#pragma unroll
    for (int u = I0 + 1; u < I1 + LEN; u++) {
        const float d = (float)(u - LEN) + off;
        z[u] = d * d;
    }
#pragma unroll
    for (int i = I0; i < I1; i++) {
        float c[LEN];
#pragma unroll
        for (int s = 0; s < LEN; s++) c[s] = v[s] + z[i - s + LEN];
        const float m = min_all<LEN>(c);
        out[base + i * STRIDE] = c[0] != c[0] ? c[0] : m;
    }
}

template <int LEN, int AXIS, int P>
__device__ __forceinline__ void dt_dispatch_val(int part, const float* in, float* out, float off, int base) {
    constexpr int K = bp_parts(LEN), OPP = (LEN + K - 1) / K;
    if constexpr (P < K) {
        if (part == P) {
            constexpr int I0 = P * OPP, I1 = (P + 1) * OPP < LEN ? (P + 1) * OPP : LEN;
            if constexpr (I0 < I1) dt_part_val<LEN, AXIS, I0, I1>(in, out, off, base);
            return;
        }
        dt_dispatch_val<LEN, AXIS, P + 1>(part, in, out, off, base);
    }
}

template <int LEN, int AXIS>
__device__ __forceinline__ void dt_lines_val(const float* in, float* out, float off) {
    constexpr int LEN2 = LEN * LEN, LP = bp_line_slots(LEN);
    const int part = threadIdx.x / LP, line = threadIdx.x - part * LP;
    if (line >= LEN2) return;
    const int base = AXIS == 0 ? line * LEN : (AXIS == 1 ? (line % LEN) + (line / LEN) * LEN2 : line);
    dt_dispatch_val<LEN, AXIS, 0>(part, in, out, off, base);
}

// Block-wide minimum with one barrier: warps reduce by shuffles, then every thread
// reduces the per-warp values.  `red` must not be rewritten before every thread has
// read it (the caller's next barrier).
__device__ __forceinline__ float block_min1(float v, float* red) {
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    const int nw = (int)(blockDim.x >> 5);
    v = red[0];
    for (int w = 1; w < nw; w++) v = fminf(v, red[w]);
    return v;
}

// Argmin table of one node (allinds, src/regularisation.h:37-107).  The sweep
// computes message values only; a node's three passes are run again here from
// its stored scaled row (`pre`, the transforms' input) with the reference's
// strict-'<' first-minimiser scans, which reproduce the sweep's values bit for
// bit and record, per parent label, the child label.  Uses A, B, ia, ib; the
// caller's barrier precedes (shared memory free) and follows.
template <int LEN>
__device__ __forceinline__ void node_argmin(const BpTree& t, int node, const float* __restrict__ pre,
                                            const float* __restrict__ off, short* __restrict__ allinds, float* A,
                                            float* B, short* ia, short* ib) {
    constexpr int LEN3 = LEN * LEN * LEN;
    constexpr int T = bp_threads(LEN);
    const float* prow = pre + (int64_t)node * LEN3;
    for (int l = threadIdx.x; l < LEN3; l += T) A[l] = ld_cg(prow + l);
    const float ox = off[node], oy = off[t.sz + node], oz = off[2 * t.sz + node];
    __syncthreads();
    dt_lines<LEN, 0>(A, B, nullptr, ia, oy);
    __syncthreads();
    dt_lines<LEN, 1>(B, A, ia, ib, ox);
    __syncthreads();
    dt_lines<LEN, 2>(A, B, ib, ia, oz);
    __syncthreads();
    short* arow = allinds + (int64_t)node * LEN3;
    for (int l = threadIdx.x; l < LEN3; l += T) arow[l] = ia[l];
}

// Slots of the sweep's shared-memory list of a chain's finished nodes (flushed
// to the global list when full).
constexpr int kChainSlots = 1024;

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_gpu(int* p, int v) {
    asm volatile("st.relaxed.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_relaxed_gpu(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Children (by position among the parent's children) whose rows a chain step may
// hold in registers when every sibling has already arrived: within the register
// budget of the sweep's thread count and its other state, and leaving room on the
// SM for the argmin kernel that runs beside the other direction's sweep.
constexpr int sweep_sibling_regs(int len) { return len <= 9 ? 3 : (len == 13 ? 2 : (len <= 15 ? 1 : 0)); }

constexpr long long kArgminSpinLimit = 1LL << 21;  // polls of a 256 ns sleep: ~0.5 s, far beyond a sweep

// Takes the next entry of the list of finished nodes by ticket (work[1]: tickets
// handed out, work[2]: entries reserved; `done`: the entries, -1 until written).
// Used after the sweep, when every reserved entry is written; the wait for it
// is bounded all the same (error 4).  Returns -1 when the entries are exhausted.
// One thread.
__device__ __forceinline__ int take_finished(const BpTree& t, int* work, int* done, int* err) {
    const int k = atomicAdd(work + 1, 1);
    if (k >= ld_acquire_gpu(work + 2)) return -1;
    int v;
    long long it = 0;
    while ((v = ld_acquire_gpu(done + k)) < 0) {
        if (++it > kArgminSpinLimit || ld_acquire_gpu(err) != 0) {
            atomicCAS(err, 0, 4);
            return -1;
        }
        __nanosleep(256);
    }
    return v;
}

template <int LEN>
__global__ void __launch_bounds__(bp_threads(LEN)) k_bp_up(BpTree t, float* __restrict__ cost,
                                                           float* __restrict__ pre, float* __restrict__ mins,
                                                           const float* __restrict__ off,
                                                           int* __restrict__ arrived, int* __restrict__ work,
                                                           int* __restrict__ done, int lists,
                                                           int* __restrict__ err) {
    constexpr int LEN3 = LEN * LEN * LEN;
    constexpr int T = bp_threads(LEN);
    constexpr int NL = (LEN3 + T - 1) / T;
    extern __shared__ float smem[];
    float* A = smem;
    float* B = A + LEN3;
    int* s_chain = reinterpret_cast<int*>(B + LEN3);  // this chain's finished nodes
    __shared__ float red[32];
    __shared__ int s_node, s_last, s_ready;
    // A thread with no line in the transform passes (the line slots are padded past
    // LEN^2) probes, during the passes, whether the parent's other children have
    // all arrived already.
    constexpr int kProbe = bp_line_slots(LEN) - 1;
    static_assert(kProbe >= LEN * LEN && kProbe < T, "the probe thread has no transform line");
    constexpr int KS = sweep_sibling_regs(LEN);
    static_assert(KS <= kKidRegs, "sibling rows are held by child position");
    const int tid = threadIdx.x;
    __shared__ int s_nchain;  // entries of s_chain (written by thread 0)
    if (tid == 0) s_nchain = 0;
    // The argmin tables (only when they are wanted, `lists`; the registration's
    // downward pass evaluates the one entry per node it reads from the stored
    // scaled rows instead): every chain appends its nodes to the list of finished
    // nodes (`done`, work[2] counts entries) when it ends (at a sibling, or at the
    // root) or its shared-memory list is full, and k_bp_argmin_rest makes their
    // tables across the GPU after the sweep, from the stored scaled rows.  The
    // barrier before an append makes every thread's rows visible to thread 0, whose
    // GPU-scope fence orders them before its relaxed list stores.
    auto publish_list = [&]() {  // thread 0
        __threadfence();
        const int slot = atomicAdd(work + 2, s_nchain);
        for (int k = 0; k < s_nchain; k++) st_relaxed_gpu(done + slot + k, s_chain[k]);
        s_nchain = 0;
    };
    for (;;) {
        __syncthreads();  // previous chain finished with s_node / smem
        if (tid == 0) {
            const int it = atomicAdd(work, 1);
            s_node = it < t.n_leaves ? t.leaves[it] : -1;
        }
        __syncthreads();
        int node = s_node;
        if (node < 0) return;
        {
            const float e = t.edgemst[node];
            const float* row = cost + (int64_t)node * LEN3;
            float* prow = pre + (int64_t)node * LEN3;
            for (int l = tid; l < LEN3; l += T) {
                const float a = __fmul_rn(ld_cg(row + l), e);
                A[l] = a;
                prow[l] = a;
            }
        }
        // The chain's static tree data is pipelined: the grandparent's id is known
        // one step ahead and everything else about it (child range, the parent's
        // edge offsets) is loaded during the step before it is needed, so no load
        // of a step waits for another load of the same step.
        int p = t.parents[node];
        int c0 = t.child_ptr[p], c1 = t.child_ptr[p + 1];
        float on_x = off[node], on_y = off[t.sz + node], on_z = off[2 * t.sz + node];
        int gp = p != t.root ? t.parents[p] : p;  // stays a valid node id at the root
        for (;;) {
            // the parent's row still holds its data cost (it is only written after its
            // own message): load it now, its latency hides behind the transform
            float acc[NL];
            const float* prow = cost + (int64_t)p * LEN3;
#pragma unroll
            for (int k = 0; k < NL; k++) {
                const int l = tid + k * T;
                acc[k] = 0.0f;
                if (l < LEN3) acc[k] = ld_ahead_cg(prow + l);
            }
            // the parent's children (the siblings this step may accumulate)
            int kid[kKidRegs];
#pragma unroll
            for (int k = 0; k < kKidRegs; k++) {
                kid[k] = -1;
                if (c0 + k < c1) kid[k] = ld_ahead(t.children + c0 + k);
            }
            const float ox = on_x, oy = on_y, oz = on_z;
            // next step: the parent's edge weight and the grandparent's data, all from
            // ids already in registers; the step after next: the great-grandparent's id
            const float ep = ld_ahead(t.edgemst + p);
            const int gc0 = ld_ahead(t.child_ptr + gp), gc1 = ld_ahead(t.child_ptr + gp + 1);
            const float opx = ld_ahead(off + p), opy = ld_ahead(off + t.sz + p), opz = ld_ahead(off + 2 * t.sz + p);
            int ggp = gp;
            if (gp != t.root) ggp = ld_ahead(t.parents + gp);
            // The parent's other children may all have arrived before this step: then
            // this CTA is the last arriver without the arrival atomic, and their rows
            // are loaded during the last pass instead of after the message.  The probe
            // reads the count relaxed (no wait) and, when it is complete, a fence makes
            // it an acquire of every sibling's release; the barrier after the second
            // pass passes that on to the CTA's loads.
            int probe = -1;
            if (KS > 0 && tid == kProbe && c1 - c0 > 1) probe = ld_relaxed_gpu(arrived + p);
            __syncthreads();
            dt_lines_val<LEN, 0>(A, B, oy);
            __syncthreads();
            if (KS > 0 && tid == kProbe) {
                const bool all = c1 - c0 > 1 && probe == c1 - c0 - 1;
                if (all) asm volatile("fence.acq_rel.gpu;" ::: "memory");
                s_ready = all;
            }
            dt_lines_val<LEN, 1>(B, A, ox);
            __syncthreads();
            const bool ready = KS > 0 && c1 - c0 > 1 && s_ready;
            float sib[KS > 0 ? KS : 1][NL], sibm[KS > 0 ? KS : 1];
#pragma unroll
            for (int k = 0; k < KS; k++) {
                if (ready && c0 + k < c1 && kid[k] != node) {
                    const float* chrow = cost + (int64_t)kid[k] * LEN3;
                    sibm[k] = ld_cg(mins + kid[k]);
#pragma unroll
                    for (int q = 0; q < NL; q++) {
                        const int l = tid + q * T;
                        sib[k][q] = l < LEN3 ? ld_cg(chrow + l) : 0.0f;
                    }
                }
            }
            dt_lines_val<LEN, 2>(A, B, oz);  // message in B (its argmins: k_bp_argmin, from `pre`)
            __syncthreads();
            float mn = INFINITY;
            float* crow = cost + (int64_t)node * LEN3;
            for (int l = tid; l < LEN3; l += T) {
                const float v = B[l];
                mn = fminf(mn, v);
                crow[l] = v;
            }
            mn = block_min1(mn, red);  // its barrier orders all stores of this CTA before the arrival
            // *std::min_element (src/regularisation.h:222) starts from element 0 and only
            // replaces it on '<': a NaN first element is the result, later NaNs are skipped
            if (isnan(B[0])) mn = B[0];
            if (tid == 0 && lists) {
                if (s_nchain == kChainSlots) publish_list();
                s_chain[s_nchain++] = node;
            }
            if (c1 - c0 > 1 && !ready) {
                // siblings exist: the last of them to arrive continues with the parent
                if (tid == 0) {
                    mins[node] = mn;
                    s_last = atom_add_acq_rel(arrived + p, 1) == c1 - c0 - 1;
                }
                __syncthreads();
                if (!s_last) {
                    // the chain ends at a sibling: its nodes' argmin tables are made after
                    // the sweep (made here, that work would share the SMs with the other
                    // chains' steps: two concurrent sweeps ran at about half speed)
                    if (tid == 0 && lists) publish_list();
                    break;
                }
            }
            // the parent's row = data cost + sum over children in MST ordering
            // order of (message - min); this CTA's own message is still in B
            auto add_child = [&](int ch) {
                if (ch == node) {
#pragma unroll
                    for (int k = 0; k < NL; k++) {
                        const int l = tid + k * T;
                        if (l < LEN3) acc[k] = acc[k] + (B[l] - mn);
                    }
                } else {
                    const float mch = ld_cg(mins + ch);
                    const float* chrow = cost + (int64_t)ch * LEN3;
#pragma unroll
                    for (int k = 0; k < NL; k++) {
                        const int l = tid + k * T;
                        if (l < LEN3) acc[k] = acc[k] + (ld_cg(chrow + l) - mch);
                    }
                }
            };
#pragma unroll
            for (int k = 0; k < kKidRegs; k++) {
                if (c0 + k < c1) {
                    if (k < KS && ready && kid[k] != node) {  // the row loaded during the last pass
#pragma unroll
                        for (int q = 0; q < NL; q++) {
                            const int l = tid + q * T;
                            if (l < LEN3) acc[q] = acc[q] + (sib[k < KS ? k : 0][q] - sibm[k < KS ? k : 0]);
                        }
                    } else {
                        add_child(kid[k]);
                    }
                }
            }
            for (int ci = c0 + kKidRegs; ci < c1; ci++) add_child(t.children[ci]);
            if (p == t.root) {
                float* rrow = cost + (int64_t)p * LEN3;
#pragma unroll
                for (int k = 0; k < NL; k++) {
                    const int l = tid + k * T;
                    if (l < LEN3) rrow[l] = acc[k];
                }
                __syncthreads();
                if (tid == 0 && lists) publish_list();
                break;
            }
            __syncthreads();  // B (this message) has been consumed by every thread
            float* pprow = pre + (int64_t)p * LEN3;
#pragma unroll
            for (int k = 0; k < NL; k++) {
                const int l = tid + k * T;
                if (l < LEN3) {
                    const float a = __fmul_rn(acc[k], ep);
                    A[l] = a;
                    pprow[l] = a;
                }
            }
            node = p;
            on_x = opx; on_y = opy; on_z = opz;
            p = gp; c0 = gc0; c1 = gc1;
            gp = ggp;
        }
    }
}

// ---- downward pass (src/regularisation.h:258-293)
//
// The root takes the first minimum of its cost row; every other node takes
// allinds[node][label of its parent].  Nodes are walked along heavy-path chains
// (from a chain's first node down through the child with the deepest subtree to
// a leaf), one warp per chain.  A node's label is all that the chains starting at
// its other children need: its walker publishes it in lbl[node] (-1 until then)
// and the walker of such a chain waits for that entry.  Chains are numbered in
// breadth order of their starts and taken by ticket in that order, so the chain
// holding a waited-for node was taken earlier by a running warp and every wait
// ends.  Ticket 0 is the root's chain (the longest root-leaf path): its warp
// first takes the root's label.
//
// A step's only dependency is the gather allinds[node][label of the node above].
// The warp copies the whole argmin rows of the next D nodes of its chain into a
// shared-memory ring, one bulk copy per row completing on the slot's mbarrier (a
// row's contents do not depend on labels), so the gather reads shared memory and a
// chain advances at about one shared-memory round trip per node instead of one L2
// or HBM round trip.  Rows start at 2-byte offsets: a row's copy covers the
// 16-byte-aligned span around it, except that the few bytes of the table's last
// partial 16-byte chunk are copied with plain loads, so nothing outside the table
// is read.  Node ids and u0/v0/w0 are loaded 32 nodes at a time, a window ahead.
// Waits are bounded (error 4 on expiry; the other walkers see the abort flag); a
// label or table entry out of range records error 2 and reads label 0 instead.
constexpr long long kDownSpinLimit = 1LL << 22;  // polls of a 32 ns sleep: > 0.13 s, far beyond a pass
constexpr int kDownWarps = 4;                    // walkers per CTA

__device__ __forceinline__ int ld_label(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
// Bulk copy global -> shared memory completing on an mbarrier (16-byte-aligned
// addresses, a multiple of 16 bytes).
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Bytes of one ring slot: the widest 16-byte-aligned span of a row of `len3`
// elements of `elem` bytes.
__host__ __device__ constexpr int down_slot_bytes(int len3, int elem) {
    return ((len3 * elem + 15) / 16 + 1) * 16;
}

// The child label for parent label lp from a node's scaled row `in` (LEN^3 floats,
// the input of its three transform passes) and edge offsets: the one entry of its
// argmin table that the downward pass reads, evaluated the way the full passes
// compute every entry (src/regularisation.h:37-107, node_argmin above): pass 0 at
// output Ly on every (x, z) line, pass 1 at output Lx on the (Ly, z) lines, pass 2
// at output Lz, each a strict-'<' first-minimiser scan with the same float sums,
// carrying the input index.  LEN^3 + LEN^2 + LEN candidates instead of 3 LEN^4.
// The warp's lanes share pass 0; sv/si (LEN^2) and sv2/si2 (LEN) are its scratch.
template <int LEN>
__device__ __forceinline__ int lazy_argmin(const float* in, int lp, float ox, float oy, float oz, float* sv,
                                           int* si, float* sv2, int* si2, int lane) {
    const int Ly = lp % LEN, Lx = (lp / LEN) % LEN, Lz = lp / (LEN * LEN);
    auto zz = [](int k, float off) {
        const float d = (float)k + off;
        return d * d;
    };
    float zy[LEN];  // the parabola values of each pass, once per node
#pragma unroll
    for (int u = 0; u < LEN; u++) zy[u] = zz(Ly - u, oy);
    for (int q = lane; q < LEN * LEN; q += 32) {  // pass 0 (y): line q = x + z LEN
        const float* line = in + q * LEN;
        float best = line[0] + zy[0];
        int bu = 0;
#pragma unroll
        for (int u = 1; u < LEN; u++) {
            const float c = line[u] + zy[u];
            if (c < best) { best = c; bu = u; }
        }
        sv[q] = best;
        si[q] = q * LEN + bu;
    }
    float zx[LEN];
#pragma unroll
    for (int x = 0; x < LEN; x++) zx[x] = zz(Lx - x, ox);
    __syncwarp();
    if (lane < LEN) {  // pass 1 (x): the (Ly, z = lane) line
        const int z = lane;
        float best = sv[z * LEN] + zx[0];
        int bt = 0;
#pragma unroll
        for (int x = 1; x < LEN; x++) {
            const float c = sv[x + z * LEN] + zx[x];
            if (c < best) { best = c; bt = x; }
        }
        sv2[z] = best;
        si2[z] = si[bt + z * LEN];
    }
    float zzz[LEN];
#pragma unroll
    for (int z = 0; z < LEN; z++) zzz[z] = zz(Lz - z, oz);
    __syncwarp();
    float best = sv2[0] + zzz[0];  // pass 2 (z): the (Ly, Lx) line, every lane alike
    int bs = 0;
#pragma unroll
    for (int z = 1; z < LEN; z++) {
        const float c = sv2[z] + zzz[z];
        if (c < best) { best = c; bs = z; }
    }
    const int l = si2[bs];
    __syncwarp();  // sv, sv2 are rewritten by the next node's passes
    return l;
}

// lbl: [sz] labels (-1 = not yet known); ctl[0]: tickets handed out, ctl[1]: abort flag.
// LEN = 0: rows of the argmin tables (allinds, int16) are gathered; LEN > 0: rows of
// the stored scaled inputs (pre, float) and the edge offsets (off: x | y | z) give
// the child label through lazy_argmin, and no argmin table is read or written.
template <int D, int LEN>
__global__ void __launch_bounds__(32 * kDownWarps) k_bp_down(BpTree t, const float* __restrict__ cost,
                                                            short* __restrict__ allinds,
                                                            const float* __restrict__ pre,
                                                            const float* __restrict__ off, int* __restrict__ lbl,
                                                            int* __restrict__ ctl, int* __restrict__ err) {
    static_assert(D >= 1 && D <= 16 && (D & (D - 1)) == 0, "ring depth: a power of two, at most half a window");
    constexpr bool kLazy = LEN > 0;
    constexpr int kElem = kLazy ? 4 : 2;
    extern __shared__ __align__(16) unsigned char down_smem[];
    const int len = kLazy ? LEN : t.len, len3 = len * len * len;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int slot_bytes = down_slot_bytes(len3, kElem);
    unsigned char* ring = down_smem + (size_t)wid * D * slot_bytes;
    uint64_t* bars = reinterpret_cast<uint64_t*>(down_smem + (size_t)kDownWarps * D * slot_bytes) + wid * D;
    // lazy scratch per warp: sv, si [LEN^2], sv2, si2 [LEN]
    constexpr int kScratch = kLazy ? 2 * (LEN * LEN + LEN) : 1;
    float* sv = reinterpret_cast<float*>(down_smem + (size_t)kDownWarps * D * (slot_bytes + 8)) + wid * kScratch;
    int* si = reinterpret_cast<int*>(sv + (kLazy ? LEN * LEN : 0));
    float* sv2 = reinterpret_cast<float*>(si + (kLazy ? LEN * LEN : 0));
    int* si2 = reinterpret_cast<int*>(sv2 + (kLazy ? LEN : 0));
    const char* table = kLazy ? reinterpret_cast<const char*>(pre) : reinterpret_cast<const char*>(allinds);
    const long long table_bytes = (long long)t.sz * len3 * kElem;
    if (lane == 0) {
        for (int k = 0; k < D; k++) mbar_init(bars + k, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    // per slot (bit s): the parity of its next phase, and whether a copy into it is
    // in flight (warp-uniform)
    uint32_t phase = 0, pending = 0;
    // copies the row of node nd into ring slot s (nothing for nd < 0)
    auto fetch = [&](int nd, int s) {
        if (nd < 0) return;
        pending |= 1u << s;
        if (lane == 0) {
            const long long a = (long long)nd * len3 * kElem, a0 = a & ~15LL, e = a + (long long)kElem * len3;
            long long bulk = ((e - a0 + 15) >> 4) << 4;
            if (a0 + bulk > table_bytes) bulk = (table_bytes - a0) & ~15LL;  // the table's last partial chunk
            unsigned char* dst = ring + s * slot_bytes;
            // the slot's earlier contents were read (generic proxy) before this copy
            // (async proxy) overwrites them
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_expect_tx(bars + s, (uint32_t)bulk);
            if (bulk > 0) bulk_load(dst, table + a0, (uint32_t)bulk, bars + s);
            for (long long g = a0 + bulk; g < e; g += 2)
                *reinterpret_cast<short*>(dst + (g - a0)) = *reinterpret_cast<const short*>(table + g);
        }
    };
    // waits for the copy into slot s; false if the bounded wait expired
    auto wait_slot = [&](int s) {
        const bool ok = mbar_wait_bounded(bars + s, (phase >> s) & 1u);
        phase ^= 1u << s;
        pending &= ~(1u << s);
        return __all_sync(0xffffffffu, ok);
    };
    auto drain = [&]() {
        for (int k = 0; k < D; k++)
            if (pending & (1u << k)) wait_slot(k);
    };
    for (;;) {
        int tk = 0;
        if (lane == 0) tk = atomicAdd(ctl, 1);
        const int c = __shfl_sync(0xffffffffu, tk, 0);
        if (c >= t.n_chains) break;
        const int s0 = ld_ahead(t.chain_ptr + c), n = ld_ahead(t.chain_ptr + c + 1) - s0;
        // node ids: lane j of w_node holds node s0 + 32 W + j of the current window W,
        // x_node the next window's; in lazy mode the nodes' edge offsets likewise
        // (the next window's loaded half a window later)
        int w_node = lane < n ? ld_ahead(t.chain_nodes + s0 + lane) : -1;
        int x_node = 32 + lane < n ? ld_ahead(t.chain_nodes + s0 + 32 + lane) : -1;
        float w_ox = 0.0f, w_oy = 0.0f, w_oz = 0.0f, x_ox = 0.0f, x_oy = 0.0f, x_oz = 0.0f;
        if (kLazy && w_node >= 0) {
            w_ox = ld_ahead(off + w_node); w_oy = ld_ahead(off + t.sz + w_node); w_oz = ld_ahead(off + 2 * t.sz + w_node);
        }
        const int first = __shfl_sync(0xffffffffu, w_node, 0);
        const bool root_chain = first == t.root;
#pragma unroll
        for (int k = 0; k < D; k++) {
            const int nd = __shfl_sync(0xffffffffu, w_node, k);
            fetch(k < n && !(root_chain && k == 0) ? nd : -1, k);
        }
        int lp;  // label of the node above the next one
        if (root_chain) {
            // first minimum of the root's cost row; the reference scans with value=cost[0],
            // index=0 and '<' (src/regularisation.h:258-279): a NaN at 0 keeps index 0, NaNs
            // elsewhere never win
            const float* rr = cost + (int64_t)first * len3;
            float bv = INFINITY;
            int bi = 0x7fffffff;
            for (int l = lane; l < len3; l += 32) {
                const float v = __ldcg(rr + l);
                if (v < bv) { bv = v; bi = l; }
                if (!kLazy) allinds[(int64_t)first * len3 + l] = (short)l;
            }
            for (int o = 16; o > 0; o >>= 1) {
                const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ov < bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
            }
            if (isnan(__ldcg(rr)) || bi < 0 || bi >= len3) bi = 0;
            lp = bi;
        } else {
            const int p = ld_ahead(t.parents + first);
            int v = -1;
            if (lane == 0) {
                long long it = 0;
                while ((v = ld_label(lbl + p)) < 0) {
                    if (++it > kDownSpinLimit || ld_label(ctl + 1) != 0) break;
                    __nanosleep(32);
                }
            }
            v = __shfl_sync(0xffffffffu, v, 0);
            if (v < 0) {
                if (lane == 0) {
                    atomicCAS(err, 0, 4);
                    st_relaxed_gpu(ctl + 1, 1);
                }
                drain();
                break;
            }
            lp = v;
        }
        for (int k = 0; k < n; k++) {
            if (k > 0 && (k & 31) == 0) {  // next window
                w_node = x_node;
                w_ox = x_ox; w_oy = x_oy; w_oz = x_oz;
                x_node = k + 32 + lane < n ? ld_ahead(t.chain_nodes + s0 + k + 32 + lane) : -1;
            }
            if (kLazy && (k & 31) == 16 && x_node >= 0) {  // the next window's ids were loaded 16 steps ago
                x_ox = ld_ahead(off + x_node); x_oy = ld_ahead(off + t.sz + x_node); x_oz = ld_ahead(off + 2 * t.sz + x_node);
            }
            const int nd = __shfl_sync(0xffffffffu, w_node, k & 31);
            int l = lp;
            if (!(root_chain && k == 0)) {
                if (!wait_slot(k & (D - 1))) {  // row k has landed (bounded)
                    if (lane == 0) {
                        atomicCAS(err, 0, 4);
                        st_relaxed_gpu(ctl + 1, 1);
                    }
                    drain();
                    return;
                }
                __syncwarp();  // and lane 0's plain-load tail bytes of it are visible
                if (lp < 0 || lp >= len3) {  // never for a completed upward pass; keeps reads in bounds
                    if (lane == 0) atomicCAS(err, 0, 2);
                    lp = 0;
                }
                // the row's offset in its 16-byte-aligned span (low bits of nd * len3 * elem)
                const unsigned char* row =
                    ring + (k & (D - 1)) * slot_bytes + (int)(((unsigned)nd * (unsigned)(kElem * len3)) & 15u);
                if constexpr (kLazy) {
                    const float ox = __shfl_sync(0xffffffffu, w_ox, k & 31);
                    const float oy = __shfl_sync(0xffffffffu, w_oy, k & 31);
                    const float oz = __shfl_sync(0xffffffffu, w_oz, k & 31);
                    l = lazy_argmin<kLazy ? LEN : 1>(reinterpret_cast<const float*>(row), lp, ox, oy, oz, sv, si, sv2,
                                                     si2, lane);
                } else {
                    l = reinterpret_cast<const short*>(row)[lp];
                }
                if (l < 0 || l >= len3) {  // never for a completed upward pass
                    if (lane == 0) atomicCAS(err, 0, 2);
                    l = 0;
                }
            }
            __syncwarp();  // every lane has read the slot before it is refilled
            if (lane == 0) st_relaxed_gpu(lbl + nd, l);
            {
                const int kn = k + D;
                const int a = __shfl_sync(0xffffffffu, w_node, kn & 31);
                const int b = __shfl_sync(0xffffffffu, x_node, kn & 31);
                fetch(kn < n ? ((kn >> 5) == (k >> 5) ? a : b) : -1, kn & (D - 1));
            }
            lp = l;
        }
    }
    drain();  // no copy outlives the CTA
}

// Every node's displacement from its resolved label (src/regularisation.h:275-292),
// all nodes at once after the walk: u1 = (x index - hw) * q + u0, likewise v1 (y)
// and w1 (z).  A label never resolved (only after an aborted walk) records error 2
// and reads label 0.
__global__ void k_bp_field(BpTree t, const int* __restrict__ lbl, float* __restrict__ u1, float* __restrict__ v1,
                           float* __restrict__ w1, int* __restrict__ err) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= t.sz) return;
    const int len = t.len, hw = (len - 1) / 2;
    int l = lbl[v];
    if (l < 0 || l >= len * len * len) {
        atomicCAS(err, 0, 2);
        l = 0;
    }
    const int ii = l % len, jj = (l / len) % len, kk = l / (len * len);
    u1[v] = (float)(jj - hw) * t.q + t.u0[v];
    v1[v] = (float)(ii - hw) * t.q + t.v0[v];
    w1[v] = (float)(kk - hw) * t.q + t.w0[v];
}

// Per node the offset of its edge in label units, (u0[parent] - u0[node]) / q
// (src/regularisation.h:205-208), for x | y | z: constants of the upward pass,
// computed for all nodes at once so that no chain step waits for a division.
__global__ void k_bp_offsets(BpTree t, float* __restrict__ off) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= t.sz) return;
    if (c == t.root) {  // never used: the root has no edge
        off[c] = off[t.sz + c] = off[2 * t.sz + c] = 0.0f;
        return;
    }
    const int p = t.parents[c];
    off[c] = __fdiv_rn(t.u0[p] - t.u0[c], t.q);
    off[t.sz + c] = __fdiv_rn(t.v0[p] - t.v0[c], t.q);
    off[2 * t.sz + c] = __fdiv_rn(t.w0[p] - t.w0[c], t.q);
}

// The argmin tables of the nodes in the list of finished nodes (the chain that
// reached the root, and chains longer than the sweep's shared list), after the
// sweep: every entry is written by then.  Persistent CTAs take entries by ticket.
template <int LEN>
__global__ void __launch_bounds__(bp_threads(LEN)) k_bp_argmin_rest(BpTree t, const float* __restrict__ pre,
                                                                    const float* __restrict__ off,
                                                                    int* __restrict__ work, int* __restrict__ done,
                                                                    short* __restrict__ allinds,
                                                                    int* __restrict__ err) {
    constexpr int LEN3 = LEN * LEN * LEN;
    extern __shared__ float smem[];
    float* A = smem;
    float* B = A + LEN3;
    short* ia = reinterpret_cast<short*>(B + LEN3);
    short* ib = ia + LEN3;
    __shared__ int s_node;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_node = take_finished(t, work, done, err);
        __syncthreads();
        if (s_node < 0) return;
        node_argmin<LEN>(t, s_node, pre, off, allinds, A, B, ia, ib);
    }
}

// dynamic shared memory of the sweep (A, B floats, the chain list) and of the argmin
// kernel (A, B floats, ia, ib shorts)
template <int LEN>
constexpr size_t bp_smem(bool sweep) {
    constexpr size_t LEN3 = (size_t)LEN * LEN * LEN;
    return LEN3 * 2 * sizeof(float) + (sweep ? kChainSlots * sizeof(int) : 2 * LEN3 * sizeof(short));
}

template <int LEN>
cudaError_t launch_up(const BpTree& t, float* cost, short* allinds, float* pre, float* mins, int* arrived,
                      int* work, int* done, int* err, int sm_count, int concurrent, cudaStream_t s) {
    constexpr int T = bp_threads(LEN);
    const size_t smem = bp_smem<LEN>(true);
    cudaError_t e = cudaFuncSetAttribute(k_bp_up<LEN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bp_up<LEN>, T, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    // At most two CTAs per SM: the sweep is bound by its deepest chain, whose steps
    // slow down when more CTAs share its SM, while two per SM still finish the rest
    // of the nodes well within the chain's time.  With `concurrent` sweeps running
    // at once (the two directions of a registration) each takes its share of the
    // SMs' CTA slots: persistent CTAs of a sweep that took every slot would keep the
    // other sweep's CTAs from starting until its own ended (at label widths 13-17 a
    // single CTA fills an SM's registers).
    const int slots = per_sm * sm_count / (concurrent > 1 ? concurrent : 1);
    int ctas = slots < 2 * sm_count ? slots : 2 * sm_count;
    if (ctas < 1) ctas = 1;
    if (ctas > t.n_leaves) ctas = t.n_leaves;
    float* off = mins + t.sz;
    k_bp_offsets<<<(t.sz + 255) / 256, 256, 0, s>>>(t, off);
    k_bp_up<LEN><<<ctas, T, smem, s>>>(t, cost, pre, mins, off, arrived, work, done, allinds ? 1 : 0, err);
    count_launches(2);
    return cudaGetLastError();
}

template <int LEN>
cudaError_t launch_argmin(const BpTree& t, short* allinds, const float* pre, const float* mins, int* work, int* done,
                          int* err, int sm_count, cudaStream_t s) {
    constexpr int T = bp_threads(LEN);
    const float* off = mins + t.sz;
    const size_t smem = bp_smem<LEN>(false);
    cudaError_t e = cudaFuncSetAttribute(k_bp_argmin_rest<LEN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bp_argmin_rest<LEN>, T, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int ctas = per_sm * sm_count;
    if (ctas > t.sz) ctas = t.sz;
    k_bp_argmin_rest<LEN><<<ctas, T, smem, s>>>(t, pre, off, work, done, allinds, err);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_bp_up(const BpTree& t, float* d_cost, short* d_allinds, float* d_pre, float* d_mins, int* d_arrived,
                         int* d_work, int* d_done, int* d_err, int sm_count, int concurrent, cudaStream_t s) {
    if (t.n_leaves <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(d_arrived, 0, sizeof(int) * (size_t)t.sz, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_work, 0, 3 * sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_done, 0xff, sizeof(int) * (size_t)t.sz, s);  // -1: not written
    if (e != cudaSuccess) return e;
    switch (t.len) {
        case 1: return launch_up<1>(t, d_cost, d_allinds, d_pre, d_mins, d_arrived, d_work, d_done, d_err, sm_count, concurrent, s);
        case 3: return launch_up<3>(t, d_cost, d_allinds, d_pre, d_mins, d_arrived, d_work, d_done, d_err, sm_count, concurrent, s);
        case 5: return launch_up<5>(t, d_cost, d_allinds, d_pre, d_mins, d_arrived, d_work, d_done, d_err, sm_count, concurrent, s);
        case 7: return launch_up<7>(t, d_cost, d_allinds, d_pre, d_mins, d_arrived, d_work, d_done, d_err, sm_count, concurrent, s);
        case 9: return launch_up<9>(t, d_cost, d_allinds, d_pre, d_mins, d_arrived, d_work, d_done, d_err, sm_count, concurrent, s);
        case 11: return launch_up<11>(t, d_cost, d_allinds, d_pre, d_mins, d_arrived, d_work, d_done, d_err, sm_count, concurrent, s);
        case 13: return launch_up<13>(t, d_cost, d_allinds, d_pre, d_mins, d_arrived, d_work, d_done, d_err, sm_count, concurrent, s);
        case 15: return launch_up<15>(t, d_cost, d_allinds, d_pre, d_mins, d_arrived, d_work, d_done, d_err, sm_count, concurrent, s);
        case 17: return launch_up<17>(t, d_cost, d_allinds, d_pre, d_mins, d_arrived, d_work, d_done, d_err, sm_count, concurrent, s);
        case 19: return launch_up<19>(t, d_cost, d_allinds, d_pre, d_mins, d_arrived, d_work, d_done, d_err, sm_count, concurrent, s);
        case 21: return launch_up<21>(t, d_cost, d_allinds, d_pre, d_mins, d_arrived, d_work, d_done, d_err, sm_count, concurrent, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_bp_argmin(const BpTree& t, short* d_allinds, const float* d_pre, const float* d_mins, int* d_work,
                             int* d_done, int* d_err, int sm_count, cudaStream_t s) {
    if (t.n_leaves <= 0) return cudaSuccess;
    switch (t.len) {
        case 1: return launch_argmin<1>(t, d_allinds, d_pre, d_mins, d_work, d_done, d_err, sm_count, s);
        case 3: return launch_argmin<3>(t, d_allinds, d_pre, d_mins, d_work, d_done, d_err, sm_count, s);
        case 5: return launch_argmin<5>(t, d_allinds, d_pre, d_mins, d_work, d_done, d_err, sm_count, s);
        case 7: return launch_argmin<7>(t, d_allinds, d_pre, d_mins, d_work, d_done, d_err, sm_count, s);
        case 9: return launch_argmin<9>(t, d_allinds, d_pre, d_mins, d_work, d_done, d_err, sm_count, s);
        case 11: return launch_argmin<11>(t, d_allinds, d_pre, d_mins, d_work, d_done, d_err, sm_count, s);
        case 13: return launch_argmin<13>(t, d_allinds, d_pre, d_mins, d_work, d_done, d_err, sm_count, s);
        case 15: return launch_argmin<15>(t, d_allinds, d_pre, d_mins, d_work, d_done, d_err, sm_count, s);
        case 17: return launch_argmin<17>(t, d_allinds, d_pre, d_mins, d_work, d_done, d_err, sm_count, s);
        case 19: return launch_argmin<19>(t, d_allinds, d_pre, d_mins, d_work, d_done, d_err, sm_count, s);
        case 21: return launch_argmin<21>(t, d_allinds, d_pre, d_mins, d_work, d_done, d_err, sm_count, s);
        default: return cudaErrorInvalidValue;
    }
}

// Ring depth by row size: at most ~200 KB of shared memory per CTA.
constexpr int down_ring(int slot) { return slot <= 3072 ? 8 : (slot <= 12288 ? 4 : (slot <= 20480 ? 2 : 1)); }

template <int D, int LEN>
static cudaError_t launch_down(const BpTree& t, const float* d_cost, short* d_allinds, const float* d_pre,
                               const float* d_off, float* d_u1, float* d_v1, float* d_w1, int* d_lbl, int* d_err,
                               int sm_count, cudaStream_t s) {
    constexpr int kElem = LEN > 0 ? 4 : 2;
    const int len3 = t.len * t.len * t.len;
    const size_t scratch = LEN > 0 ? 2 * (size_t)(LEN * LEN + LEN) * 4 : 4;
    const size_t smem = (size_t)kDownWarps * (D * (down_slot_bytes(len3, kElem) + sizeof(uint64_t)) + scratch);
    cudaError_t e = cudaFuncSetAttribute(k_bp_down<D, LEN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bp_down<D, LEN>, 32 * kDownWarps, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    // every CTA resident at once; no more walkers than chains
    const int ctas = std::max(1, std::min(per_sm * sm_count, (t.n_chains + kDownWarps - 1) / kDownWarps));
    // labels unknown (-1), ticket counter 0, abort flag 0
    e = cudaMemsetAsync(d_lbl, 0xff, sizeof(int) * (size_t)t.sz, s);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(d_lbl + t.sz, 0, 2 * sizeof(int), s);
    if (e != cudaSuccess) return e;
    k_bp_down<D, LEN><<<ctas, 32 * kDownWarps, smem, s>>>(t, d_cost, d_allinds, d_pre, d_off, d_lbl, d_lbl + t.sz,
                                                         d_err);
    k_bp_field<<<(t.sz + 255) / 256, 256, 0, s>>>(t, d_lbl, d_u1, d_v1, d_w1, d_err);
    count_launches(2);
    return cudaGetLastError();
}

template <int LEN>
static cudaError_t launch_down_lazy(const BpTree& t, const float* d_cost, const float* d_pre, const float* d_off,
                                    float* d_u1, float* d_v1, float* d_w1, int* d_lbl, int* d_err, int sm_count,
                                    cudaStream_t s) {
    constexpr int D = down_ring(down_slot_bytes(LEN * LEN * LEN, 4));
    return launch_down<D, LEN>(t, d_cost, nullptr, d_pre, d_off, d_u1, d_v1, d_w1, d_lbl, d_err, sm_count, s);
}

cudaError_t launch_bp_down(const BpTree& t, const float* d_cost, short* d_allinds, const float* d_pre,
                           const float* d_mins, float* d_u1, float* d_v1, float* d_w1, int* d_lbl, int* d_err,
                           int sm_count, cudaStream_t s) {
    if (t.n_chains < 1 || !t.chain_ptr || !t.chain_nodes || sm_count < 1) return cudaErrorInvalidValue;
    if (!d_allinds) {
        // no tables: the one entry per node from the stored scaled rows (16-byte aligned)
        if (!d_pre || !d_mins || (reinterpret_cast<uintptr_t>(d_pre) & 15)) return cudaErrorInvalidValue;
        const float* off = d_mins + t.sz;
#define DEEDS_LAZY(L) \
    case L: return launch_down_lazy<L>(t, d_cost, d_pre, off, d_u1, d_v1, d_w1, d_lbl, d_err, sm_count, s);
        switch (t.len) {
            DEEDS_LAZY(1) DEEDS_LAZY(3) DEEDS_LAZY(5) DEEDS_LAZY(7) DEEDS_LAZY(9) DEEDS_LAZY(11) DEEDS_LAZY(13)
            DEEDS_LAZY(15) DEEDS_LAZY(17) DEEDS_LAZY(19) DEEDS_LAZY(21)
            default: return cudaErrorInvalidValue;
        }
#undef DEEDS_LAZY
    }
    // the rows are copied in 16-byte chunks from a 16-byte-aligned table
    if (reinterpret_cast<uintptr_t>(d_allinds) & 15) return cudaErrorInvalidValue;
    const int slot = down_slot_bytes(t.len * t.len * t.len, 2);
    if (slot <= 3072) return launch_down<8, 0>(t, d_cost, d_allinds, nullptr, nullptr, d_u1, d_v1, d_w1, d_lbl, d_err, sm_count, s);
    if (slot <= 12288) return launch_down<4, 0>(t, d_cost, d_allinds, nullptr, nullptr, d_u1, d_v1, d_w1, d_lbl, d_err, sm_count, s);
    return launch_down<2, 0>(t, d_cost, d_allinds, nullptr, nullptr, d_u1, d_v1, d_w1, d_lbl, d_err, sm_count, s);
}

}  // namespace deeds
