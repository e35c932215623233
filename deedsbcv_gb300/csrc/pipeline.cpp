// libdeeds_gpu host side: the C ABI of include/deeds_gpu.h, the context (device
// scratch, streams, pinned staging) and the per-pair level loop that replaces
// main() of src/deedsBCV0.cpp:183-356.
//
// Per pair, on the caller's stream:
//   shift (+1024) -> affine warp of the moving image (warped0)
//   side stream: block SADs of fixed and warped0 for every level's grid ->
//   host: image statistics, Prim and the BP schedules for all 2*levels trees,
//         on worker threads, overlapped with the GPU level loop;
//   per level, forward then backward: grid upsample -> fused full-res
//   upsample + warp -> MIND-SSC -> Hamming cost volume -> (wait for that tree)
//   upload schedule -> upward BP -> downward BP; then inverse consistency.
// Compiled with -ffp-contract=off (host float arithmetic follows the reference).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <future>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/deeds_gpu.h"
#include "kernels.h"
#include "tree_host.h"
#include "linear_host.h"

using namespace deeds;

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
};
struct HostBuf {
    void* p = nullptr;
    size_t cap = 0;
};

struct SoftKept;

struct deeds_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;  // used by the host-pointer entry points
    cudaStream_t side = nullptr;    // MST edge costs and their copies
    cudaStream_t stream_b = nullptr;  // backward-direction chain of deeds_register*
    cudaStream_t bg = nullptr;        // field-independent work deeds_register* overlaps with tree sweeps
    // per direction: the argmin tables of a sweep at the lowest priority, so that
    // they yield SMs to the other direction's latency-bound sweep
    cudaStream_t low[2] = {nullptr, nullptr};
    cudaEvent_t ev_up[2] = {nullptr, nullptr}, ev_arg[2] = {nullptr, nullptr}, ev_cost[2] = {nullptr, nullptr};
    cudaEvent_t ev_e = nullptr, ev_f = nullptr, ev_g = nullptr;
    cudaEvent_t ev_a = nullptr, ev_b = nullptr, ev_c = nullptr, ev_d = nullptr;
    std::string err;
    std::map<std::string, DevBuf> dev;
    std::map<std::string, HostBuf> host;
    int epoch = 0;
    // per-stage tracing (deeds_set_profiling)
    bool prof = false;
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    std::vector<cudaEvent_t> ev_mst;  // MST-input events of deeds_register_dev
    struct Mark { int stage; cudaEvent_t a, b; };
    std::vector<Mark> marks;
    double stage_ms[DEEDS_NUM_STAGES] = {0};
    long long stage_launches[DEEDS_NUM_STAGES] = {0};
    // cost-volume tile sizes chosen by the autotuner, per (g, hw, q); shared with batch lanes
    struct TuneTable {
        std::mutex mu;
        std::map<std::vector<int>, int> tile;
    };
    std::shared_ptr<TuneTable> tune = std::make_shared<TuneTable>();
    // lanes of deeds_register_batch (child contexts on the same device)
    std::vector<deeds_ctx*> lanes;
    // the last registration's control-grid field (for deeds_warp_segmentation)
    bool have_field = false;
    int fm = 0, fn = 0, fo = 0;      // its volume
    int fm1 = 0, fn1 = 0, fo1 = 0;   // its control grid (field in the "keep_grid" buffer)
    float fX[16];
    // soft-min levels whose forward state stays resident for their backward
    // (deeds_soft_forward_keep_dev); index = slot
    std::vector<std::shared_ptr<SoftKept>> kept;
};

namespace deeds {
std::atomic<long long> g_kernel_launches{0};
}

namespace {

thread_local std::string g_create_err;

cudaEvent_t pool_event(deeds_ctx* c) {
    if (c->ev_used == c->ev_pool.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        c->ev_pool.push_back(e);
    }
    return c->ev_pool[c->ev_used++];
}

// Brackets one stage of the pipeline with CUDA events on `s` (and counts its
// kernel launches) when profiling is on; a no-op otherwise.
struct StageScope {
    deeds_ctx* c;
    int stage;
    cudaStream_t s;
    cudaEvent_t a = nullptr;
    long long launches0;
    StageScope(deeds_ctx* c_, int stage_, cudaStream_t s_) : c(c_), stage(stage_), s(s_) {
        launches0 = deeds::g_kernel_launches.load();
        if (c->prof && (a = pool_event(c))) cudaEventRecord(a, s);
    }
    ~StageScope() {
        if (!c->prof) return;
        c->stage_launches[stage] += deeds::g_kernel_launches.load() - launches0;
        cudaEvent_t b = a ? pool_event(c) : nullptr;
        if (b) {
            cudaEventRecord(b, s);
            c->marks.push_back({stage, a, b});
        }
    }
};

// Host timeline of one registration (DEEDS_TRACE=1 in the environment): the
// moments the host-side inputs of the trees become ready, each tree is built and
// the level loop stops waiting for it, printed to stderr at the end.
struct Timeline {
    bool on = false;
    std::chrono::steady_clock::time_point t0;
    std::mutex mu;
    std::vector<std::pair<std::string, double>> ev;
    void start() {
        const char* e = std::getenv("DEEDS_TRACE");
        on = e && e[0] == '1';
        t0 = std::chrono::steady_clock::now();
    }
    void mark(const std::string& what) {
        if (!on) return;
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        std::lock_guard<std::mutex> lock(mu);
        ev.emplace_back(what, ms);
    }
    // device-side marks: an event recorded on `s`, reported against the first one
    std::vector<std::pair<std::string, cudaEvent_t>> dev;
    void dmark(const std::string& what, cudaStream_t s) {
        if (!on) return;
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return;
        cudaEventRecord(e, s);
        dev.emplace_back(what, e);
    }
    void dump() {
        if (!on) return;
        std::lock_guard<std::mutex> lock(mu);
        for (auto& e : ev) std::fprintf(stderr, "deeds trace %8.2f ms  %s\n", e.second, e.first.c_str());
        for (auto& d : dev) {
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, dev.front().second, d.second);
            std::fprintf(stderr, "deeds trace device +%8.2f ms  %s\n", ms, d.first.c_str());
        }
        for (auto& d : dev) cudaEventDestroy(d.second);
        dev.clear();
    }
};

void collect_marks(deeds_ctx* c) {
    for (auto& mk : c->marks) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, mk.a, mk.b) == cudaSuccess) c->stage_ms[mk.stage] += ms;
    }
    c->marks.clear();
    c->ev_used = 0;
    cudaGetLastError();
}

deeds_status fail(deeds_ctx* c, deeds_status st, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    else g_create_err = buf;
    return st;
}

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) return fail(ctx, DEEDS_ERR_CUDA, "%s: %s (%s:%d)", #call,           \
                                           cudaGetErrorString(e_), __FILE__, __LINE__);           \
    } while (0)

template <class T>
T* dbuf(deeds_ctx* ctx, const std::string& name, size_t count, deeds_status* st, bool zero = false) {
    DevBuf& b = ctx->dev[name];
    const size_t bytes = std::max<size_t>(count * sizeof(T), 16);
    if (b.cap < bytes) {
        if (b.p) cudaFree(b.p);
        b.p = nullptr;
        b.cap = 0;
        if (cudaMalloc(&b.p, bytes) != cudaSuccess) {
            cudaGetLastError();
            *st = fail(ctx, DEEDS_ERR_NOMEM, "cudaMalloc of %zu bytes for %s failed", bytes, name.c_str());
            return nullptr;
        }
        b.cap = bytes;
        if (zero && cudaMemset(b.p, 0, bytes) != cudaSuccess) {
            *st = fail(ctx, DEEDS_ERR_CUDA, "cudaMemset %s failed", name.c_str());
            return nullptr;
        }
    }
    return static_cast<T*>(b.p);
}

template <class T>
T* hbuf(deeds_ctx* ctx, const std::string& name, size_t count, deeds_status* st) {
    HostBuf& b = ctx->host[name];
    const size_t bytes = std::max<size_t>(count * sizeof(T), 16);
    if (b.cap < bytes) {
        if (b.p) cudaFreeHost(b.p);
        b.p = nullptr;
        b.cap = 0;
        if (cudaHostAlloc(&b.p, bytes, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            *st = fail(ctx, DEEDS_ERR_NOMEM, "cudaHostAlloc of %zu bytes for %s failed", bytes, name.c_str());
            return nullptr;
        }
        b.cap = bytes;
    }
    return static_cast<T*>(b.p);
}

void mind_thresholds(float thr[5]) {
    for (int c = 0; c < 5; c++) thr[c] = -std::log(((float)c + 1.5f) / 6);  // logf, src/MINDSSCbox.h:177-180
}

int mind_step(int q) { return (int)std::floor(0.5f * (float)q + 1.0f); }  // src/deedsBCV0.cpp:183-186

// alpha1 = float(0.5*(g/(alpha*q))/maxsamp), sampling strides for RAND_SAMPLES=1
// (src/dataCostD.h:141-163).
void data_cost_params(int g, int q, float alpha, int* sy, int* sx, int* sz, float* alpha1) {
    *sy = 1; *sx = 1; *sz = 1;
    if (g > 4) { *sx = 2; *sz = 2; }
    const float maxsamp = std::ceil((float)g / (float)*sx) * std::ceil((float)g / (float)*sz) *
                          std::ceil((float)g / (float)*sy);
    const float alphai = (float)g / (alpha * (float)q);
    *alpha1 = (float)(0.5 * alphai / (float)maxsamp);
}

// Cost volume through the TMA-staged kernel when the shape allows it, with the
// node-tile height chosen once per shape by timing the candidates (tiles only
// change the schedule; every candidate writes the same bits).  Other shapes use
// the generic kernel.
cudaError_t data_cost_auto(deeds_ctx* ctx, const uint64_t* F, const uint64_t* M, uint64_t* Mpad, int m, int n, int o,
                           int g, int hw, int q, float alpha, float* cost, int* d_err, cudaStream_t s) {
    int sy, sx, sz;
    float alpha1;
    data_cost_params(g, q, alpha, &sy, &sx, &sz, &alpha1);
    // the best tile depends on the level parameters, not on the volume size
    const std::vector<int> key{g, hw, q};
    std::lock_guard<std::mutex> lock(ctx->tune->mu);
    auto it = ctx->tune->tile.find(key);
    int tile;
    if (it != ctx->tune->tile.end()) {
        tile = it->second;
    } else {
        // tiles of whole warps' worth of (node, sample row) threads: 32k/g nodes
        int cands[8];
        for (int k = 1; k <= 8; k++) cands[k - 1] = 32 * k / g;
        tile = 0;
        float best = 1e30f;
        cudaEvent_t a, b;
        if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) return cudaErrorUnknown;
        // once per shape and context: time the candidates with the device otherwise
        // idle (other streams of the registration would skew the comparison), best
        // of three launches each after a warm-up launch
        cudaDeviceSynchronize();
        for (int c : cands) {
            if (!data_cost_tma_supported(g, hw, q, c) || c > m / g) continue;
            cudaError_t e = launch_data_cost_tma(F, M, Mpad, m, n, o, g, hw, q, c, alpha1, cost, d_err, s);
            if (e != cudaSuccess) { cudaGetLastError(); continue; }
            float c_best = 1e30f;
            for (int r = 0; r < 3; r++) {
                cudaEventRecord(a, s);
                launch_data_cost_tma(F, M, Mpad, m, n, o, g, hw, q, c, alpha1, cost, d_err, s);
                cudaEventRecord(b, s);
                if (cudaEventSynchronize(b) != cudaSuccess) { cudaGetLastError(); break; }
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, a, b);
                c_best = std::min(c_best, ms);
            }
            if (c_best < best) { best = c_best; tile = c; }
        }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        ctx->tune->tile[key] = tile;
    }
    if (tile > m / g) tile = 0;  // tuned on a larger volume: this one has fewer grid rows
    if (tile > 0) return launch_data_cost_tma(F, M, Mpad, m, n, o, g, hw, q, tile, alpha1, cost, d_err, s);
    return launch_data_cost(F, M, m, n, o, g, hw, q, sy, sx, sz, alpha1, cost, s);
}

deeds_status check_params(deeds_ctx* ctx, const deeds_params* p, int m, int n, int o) {
    if (!p) return fail(ctx, DEEDS_ERR_INVALID, "params is NULL");
    if (p->levels < 1 || p->levels > DEEDS_MAX_LEVELS)
        return fail(ctx, DEEDS_ERR_INVALID, "levels=%d outside 1..%d", p->levels, DEEDS_MAX_LEVELS);
    if (m < 1 || n < 1 || o < 1) return fail(ctx, DEEDS_ERR_INVALID, "bad dims %dx%dx%d", m, n, o);
    for (int l = 0; l < p->levels; l++) {
        const int g = p->grid[l], hw = p->radius[l], q = p->quant[l];
        if (g < 1 || hw < 0 || q < 1)
            return fail(ctx, DEEDS_ERR_INVALID, "level %d: grid=%d radius=%d quant=%d", l, g, hw, q);
        if (hw > 10) return fail(ctx, DEEDS_ERR_INVALID, "level %d: search radius %d > 10 unsupported", l, hw);
        if (m / g < 1 || n / g < 1 || o / g < 1)
            return fail(ctx, DEEDS_ERR_INVALID, "level %d: grid %d larger than the volume", l, g);
        const int qs = mind_step(q);
        if (qs > 7) return fail(ctx, DEEDS_ERR_INVALID, "level %d: MIND radius %d > 7 unsupported", l, qs);
        if (m < 2 * qs + 1 || n < 2 * qs + 1 || o < 2 * qs + 1)
            return fail(ctx, DEEDS_ERR_INVALID, "volume %dx%dx%d too small for MIND radius %d", m, n, o, qs);
    }
    return DEEDS_OK;
}

// One tree's host arrays packed for a single H2D copy (4-byte words).
struct PackedTree {
    int sz = 0, n_leaves = 0, n_chains = 0;
    size_t o_ordered, o_parents, o_edgemst, o_cptr, o_children, o_leaves, o_chptr, o_chnodes,
        total;
};

PackedTree pack_layout(int sz) {
    PackedTree t;
    t.sz = sz;
    size_t o = 0;
    t.o_ordered = o; o += sz;
    t.o_parents = o; o += sz;
    t.o_edgemst = o; o += sz;
    t.o_cptr = o; o += sz + 1;
    t.o_children = o; o += sz;
    t.o_leaves = o; o += sz;
    t.o_chptr = o; o += sz + 1;
    t.o_chnodes = o; o += sz;
    t.total = o;
    return t;
}

void pack_schedule(const TreeSchedule& s, uint32_t* blk, PackedTree& t) {
    t.n_leaves = (int)s.leaves.size();
    std::memcpy(blk + t.o_cptr, s.child_ptr.data(), sizeof(int) * s.child_ptr.size());
    std::memcpy(blk + t.o_children, s.children.data(), sizeof(int) * s.children.size());
    std::memcpy(blk + t.o_leaves, s.leaves.data(), sizeof(int) * s.leaves.size());
    t.n_chains = (int)s.chain_ptr.size() - 1;
    std::memcpy(blk + t.o_chptr, s.chain_ptr.data(), sizeof(int) * s.chain_ptr.size());
    std::memcpy(blk + t.o_chnodes, s.chain_nodes.data(), sizeof(int) * s.chain_nodes.size());
}

// Build one tree on the host into the packed pinned block `blk`.
void build_tree(const float* sad, float stddev, int m1, int n1, int o1, int g, uint32_t* blk, PackedTree& t) {
    const int sz = m1 * n1 * o1;
    int* ordered = reinterpret_cast<int*>(blk + t.o_ordered);
    int* parents = reinterpret_cast<int*>(blk + t.o_parents);
    float* edgemst = reinterpret_cast<float*>(blk + t.o_edgemst);
    prims_from_sad(sad, stddev, m1, n1, o1, g, ordered, parents, edgemst);
    TreeSchedule s;
    build_schedule(ordered, parents, sz, s, true);  // prims_from_sad: levels in node order
    pack_schedule(s, blk, t);
}

BpTree device_tree(const PackedTree& t, const uint32_t* dblk, const uint32_t* hblk, int len, float q, const float* u0,
                   const float* v0, const float* w0) {
    BpTree b;
    b.len = len;
    b.q = q;
    b.sz = t.sz;
    b.root = reinterpret_cast<const int*>(hblk + t.o_ordered)[0];
    b.n_leaves = t.n_leaves;
    b.leaves = reinterpret_cast<const int*>(dblk + t.o_leaves);
    b.child_ptr = reinterpret_cast<const int*>(dblk + t.o_cptr);
    b.children = reinterpret_cast<const int*>(dblk + t.o_children);
    b.parents = reinterpret_cast<const int*>(dblk + t.o_parents);
    b.edgemst = reinterpret_cast<const float*>(dblk + t.o_edgemst);
    b.u0 = u0; b.v0 = v0; b.w0 = w0;
    b.n_chains = t.n_chains;
    b.chain_ptr = reinterpret_cast<const int*>(dblk + t.o_chptr);
    b.chain_nodes = reinterpret_cast<const int*>(dblk + t.o_chnodes);
    return b;
}

// Run BP on one tree: upload its schedule, upward pass, downward pass.
deeds_status run_tree_bp(deeds_ctx* ctx, const std::string& tag, const PackedTree& pt, const uint32_t* h_blk,
                         float* d_cost, short* d_allinds, int len, int q, const float* u0, const float* v0,
                         const float* w0, float* u1, float* v1, float* w1, int* d_err, cudaStream_t s,
                         Timeline* tl = nullptr, const std::string& what = "", int concurrent = 1) {
    deeds_status st = DEEDS_OK;
    uint32_t* d_blk = dbuf<uint32_t>(ctx, "tree_" + tag, pt.total, &st);
    float* d_mins = dbuf<float>(ctx, "mins_" + tag, 4 * (size_t)pt.sz, &st);  // mins | edge offsets x, y, z
    int* d_arrived = dbuf<int>(ctx, "arrived_" + tag, pt.sz, &st);
    int* d_work = dbuf<int>(ctx, "work_" + tag, 3, &st);
    int* d_done = dbuf<int>(ctx, "done_" + tag, pt.sz, &st);
    int* d_lbl = dbuf<int>(ctx, "labels_" + tag, (size_t)pt.sz + 2, &st);
    float* d_pre = dbuf<float>(ctx, "pre_" + tag, (size_t)pt.sz * len * len * len, &st);
    if (st) return st;
    CK(cudaMemcpyAsync(d_blk, h_blk, pt.total * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    const BpTree bt = device_tree(pt, d_blk, h_blk, len, (float)q, u0, v0, w0);
    {
        StageScope sc(ctx, DEEDS_STAGE_BP_UP, s);
        CK(launch_bp_up(bt, d_cost, d_allinds, d_pre, d_mins, d_arrived, d_work, d_done, d_err, ctx->sm_count,
                        concurrent, s));
    }
    if (tl) tl->dmark(what + " sweep done", s);
    if (d_allinds) {
        // the argmin tables on the direction's low-priority stream, joined back before
        // the downward pass (without tables the downward pass evaluates the one entry
        // per node it needs from the stored scaled rows)
        const int dl = tag == "b" ? 1 : 0;
        CK(cudaEventRecord(ctx->ev_up[dl], s));
        CK(cudaStreamWaitEvent(ctx->low[dl], ctx->ev_up[dl], 0));
        {
            StageScope sc(ctx, DEEDS_STAGE_BP_ARGMIN, ctx->low[dl]);
            CK(launch_bp_argmin(bt, d_allinds, d_pre, d_mins, d_work, d_done, d_err, ctx->sm_count, ctx->low[dl]));
        }
        CK(cudaEventRecord(ctx->ev_arg[dl], ctx->low[dl]));
        CK(cudaStreamWaitEvent(s, ctx->ev_arg[dl], 0));
        if (tl) tl->dmark(what + " argmins joined", s);
    }
    {
        StageScope sc(ctx, DEEDS_STAGE_BP_DOWN, s);
        CK(launch_bp_down(bt, d_cost, d_allinds, d_pre, d_mins, u1, v1, w1, d_lbl, d_err, ctx->sm_count, s));
    }
    return DEEDS_OK;
}

// Every buffer one registration of an m x n x o pair needs, sized up front so
// that nothing is reallocated (cudaFree) while kernels of the pair are in flight.
struct PairBuffers {
    size_t max_sz1 = 0, max_cost = 0, max_pad = 0;
    std::vector<int> m1s, n1s, o1s;
    float *fix, *mov, *warp0;
    // MIND codes of the fixed and of the affine-warped moving image, one pair per
    // distinct MIND step of the level schedule (field-independent)
    std::vector<int> steps;
    std::vector<uint64_t*> c_fix, c_mov;
    float* mind_bg;  // MIND scratch of the stream that computes steps 1.. (deeds_ctx::bg)
    int* d_err;
    float* warped[2];
    uint64_t* c_warp[2];
    float* mind_scr[2];
    float* cost[2];
    uint64_t* mpad[2];
    float *grid, *kgrid, *cons_scr;  // kgrid: the last result's control-grid field (u | v | w)
    void* stats_scr;  // image statistics (deeds::launch_image_stats)
    float *d_stats, *h_stats;  // mean, std of the fixed and of the affine-warped moving image
    std::vector<float*> h_sad, d_sad;
    std::vector<PackedTree> pts;
    std::vector<uint32_t*> h_tree;
};

deeds_status acquire_buffers(deeds_ctx* ctx, int m, int n, int o, const deeds_params* P, PairBuffers& B) {
    deeds_status st = DEEDS_OK;
    const int L = P->levels;
    const size_t sz = (size_t)m * n * o;
    B.m1s.assign(L, 0); B.n1s.assign(L, 0); B.o1s.assign(L, 0);
    for (int l = 0; l < L; l++) {
        const int g = P->grid[l], len = 2 * P->radius[l] + 1;
        B.m1s[l] = m / g; B.n1s[l] = n / g; B.o1s[l] = o / g;
        const size_t sz1 = (size_t)B.m1s[l] * B.n1s[l] * B.o1s[l];
        B.max_sz1 = std::max(B.max_sz1, sz1);
        B.max_cost = std::max(B.max_cost, sz1 * len * len * len);
        B.max_pad = std::max(B.max_pad, padded_codes_count(m, n, o, P->quant[l] * P->radius[l]));
    }
    B.fix = dbuf<float>(ctx, "fix", sz, &st);
    B.mov = dbuf<float>(ctx, "mov", sz, &st);
    B.warp0 = dbuf<float>(ctx, "warp0", sz, &st);
    B.steps.clear();
    for (int l = 0; l < L; l++) {
        const int qs = mind_step(P->quant[l]);
        if (std::find(B.steps.begin(), B.steps.end(), qs) == B.steps.end()) B.steps.push_back(qs);
    }
    B.c_fix.assign(B.steps.size(), nullptr);
    B.c_mov.assign(B.steps.size(), nullptr);
    B.mind_bg = B.steps.size() > 1 ? dbuf<float>(ctx, "mind_bg", 6 * sz, &st) : nullptr;
    for (size_t k = 0; k < B.steps.size(); k++) {
        B.c_fix[k] = dbuf<uint64_t>(ctx, "c_fix_" + std::to_string(k), sz, &st);
        B.c_mov[k] = dbuf<uint64_t>(ctx, "c_mov_" + std::to_string(k), sz, &st);
    }
    B.d_err = dbuf<int>(ctx, "err", 2, &st);
    const char* tags[2] = {"f", "b"};
    for (int d = 0; d < 2; d++) {
        const std::string tg = tags[d];
        B.warped[d] = dbuf<float>(ctx, "warped_" + tg, sz, &st);
        B.c_warp[d] = dbuf<uint64_t>(ctx, "c_warp_" + tg, sz, &st);
        B.mind_scr[d] = dbuf<float>(ctx, "mind_" + tg, 6 * sz, &st);
        B.cost[d] = dbuf<float>(ctx, "cost_" + tg, B.max_cost, &st);
        B.mpad[d] = dbuf<uint64_t>(ctx, "mpad_" + tg, B.max_pad, &st);
        dbuf<uint32_t>(ctx, "tree_" + tg, pack_layout((int)B.max_sz1).total, &st);
        dbuf<float>(ctx, "mins_" + tg, 4 * B.max_sz1, &st);
        dbuf<int>(ctx, "arrived_" + tg, B.max_sz1, &st);
        dbuf<int>(ctx, "work_" + tg, 3, &st);
        dbuf<int>(ctx, "done_" + tg, B.max_sz1, &st);
        dbuf<int>(ctx, "labels_" + tg, B.max_sz1 + 2, &st);
        dbuf<float>(ctx, "pre_" + tg, B.max_cost, &st);  // scaled rows of the upward sweep (argmin input)
    }
    B.grid = dbuf<float>(ctx, "grid", 18 * B.max_sz1, &st);
    B.kgrid = dbuf<float>(ctx, "keep_grid", 3 * B.max_sz1, &st);
    B.cons_scr = dbuf<float>(ctx, "consistent", 12 * B.max_sz1, &st);
    B.stats_scr = dbuf<char>(ctx, "stats_scr", image_stats_scratch_bytes(sz, 2), &st);
    B.d_stats = dbuf<float>(ctx, "stats", 4, &st);
    B.h_stats = hbuf<float>(ctx, "h_stats", 4, &st);
    B.h_sad.assign(2 * L, nullptr); B.d_sad.assign(2 * L, nullptr);
    B.pts.assign(2 * L, PackedTree()); B.h_tree.assign(2 * L, nullptr);
    for (int l = 0; l < L; l++) {
        const size_t sz1 = (size_t)B.m1s[l] * B.n1s[l] * B.o1s[l];
        for (int d = 0; d < 2; d++) {
            const int t = 2 * l + d;
            B.h_sad[t] = hbuf<float>(ctx, "h_sad" + std::to_string(t), 6 * sz1, &st);
            B.pts[t] = pack_layout((int)sz1);
            B.h_tree[t] = hbuf<uint32_t>(ctx, "h_tree" + std::to_string(t), B.pts[t].total, &st);
            B.d_sad[t] = dbuf<float>(ctx, "sad" + std::to_string(t), 6 * sz1, &st);
        }
    }
    return st;
}

// The buffers of deeds_register (host inputs/outputs included) for one pair size.
deeds_status reserve_buffers(deeds_ctx* ctx, int m, int n, int o, const deeds_params* P, bool warped) {
    PairBuffers B;
    deeds_status st = acquire_buffers(ctx, m, n, o, P, B);
    if (st) return st;
    const size_t sz = (size_t)m * n * o;
    const int gl = P->grid[P->levels - 1];
    const size_t sz1 = (size_t)(m / gl) * (n / gl) * (o / gl);
    dbuf<float>(ctx, "in_fixed", sz, &st);
    dbuf<float>(ctx, "in_moving", sz, &st);
    dbuf<float>(ctx, "out_flow", 3 * sz1, &st);
    if (warped) dbuf<float>(ctx, "out_warped", sz, &st);
    return st;
}

}  // namespace

extern "C" {

const char* deeds_version(void) { return "deeds-gb300 0.1 (sm_103a)"; }

void deeds_default_params(deeds_params* p) {
    std::memset(p, 0, sizeof(*p));
    p->levels = 5;
    const int G[5] = {8, 7, 6, 5, 4}, L[5] = {8, 7, 6, 5, 4}, Q[5] = {5, 4, 3, 2, 1};
    for (int i = 0; i < 5; i++) { p->grid[i] = G[i]; p->radius[i] = L[i]; p->quant[i] = Q[i]; }
    p->alpha = 1.6f;
    p->intensity_shift = 1024.0f;
    p->verbose = 0;
}

deeds_status deeds_create(deeds_ctx** out, int device) {
    if (!out) return fail(nullptr, DEEDS_ERR_INVALID, "ctx pointer is NULL");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(nullptr, DEEDS_ERR_CUDA, "no CUDA device available (%s)", cudaGetErrorString(e));
    if (device < 0 || device >= ndev) return fail(nullptr, DEEDS_ERR_INVALID, "device %d of %d", device, ndev);
    std::unique_ptr<deeds_ctx> c(new deeds_ctx());
    c->device = device;
    deeds_ctx* ctx = c.get();
    CK(cudaSetDevice(device));
    CK(cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device));
    {
        // Priorities (numerically lower = sooner): the MST inputs (image statistics,
        // block SADs) start the host trees that the level loop waits for, so their
        // small kernels go first; the two direction streams, which carry the
        // latency-bound tree sweeps, come before the background stream's MIND codes
        // of later levels, which only fill SMs the sweeps leave idle.
        int least = 0, greatest = 0;
        CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        const int mid = greatest + 1 <= least ? greatest + 1 : least;
        CK(cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, greatest));
        CK(cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, mid));
        CK(cudaStreamCreateWithPriority(&c->stream_b, cudaStreamNonBlocking, mid));
        CK(cudaStreamCreateWithPriority(&c->bg, cudaStreamNonBlocking, least));
        for (int d = 0; d < 2; d++) {
            CK(cudaStreamCreateWithPriority(&c->low[d], cudaStreamNonBlocking, least));
            CK(cudaEventCreateWithFlags(&c->ev_up[d], cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&c->ev_arg[d], cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&c->ev_cost[d], cudaEventDisableTiming));
        }
    }
    CK(cudaEventCreateWithFlags(&c->ev_a, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->ev_b, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->ev_c, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->ev_d, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->ev_e, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->ev_f, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->ev_g, cudaEventDisableTiming));
    *out = c.release();
    return DEEDS_OK;
}

void deeds_destroy(deeds_ctx* ctx) {
    if (!ctx) return;
    for (deeds_ctx* lane : ctx->lanes) deeds_destroy(lane);
    ctx->lanes.clear();
    cudaSetDevice(ctx->device);
    for (cudaStream_t st : {ctx->stream, ctx->stream_b, ctx->side, ctx->bg, ctx->low[0], ctx->low[1]})
        if (st) cudaStreamSynchronize(st);
    for (auto& kv : ctx->dev) if (kv.second.p) cudaFree(kv.second.p);
    for (auto& kv : ctx->host) if (kv.second.p) cudaFreeHost(kv.second.p);
    for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->ev_mst) cudaEventDestroy(e);
    for (cudaEvent_t e : {ctx->ev_a, ctx->ev_b, ctx->ev_c, ctx->ev_d, ctx->ev_e, ctx->ev_f, ctx->ev_g, ctx->ev_up[0],
                          ctx->ev_up[1], ctx->ev_arg[0], ctx->ev_arg[1], ctx->ev_cost[0], ctx->ev_cost[1]})
        if (e) cudaEventDestroy(e);
    for (cudaStream_t st : {ctx->stream, ctx->stream_b, ctx->side, ctx->bg, ctx->low[0], ctx->low[1]})
        if (st) cudaStreamDestroy(st);
    delete ctx;
}

const char* deeds_last_error(const deeds_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_err.c_str(); }

deeds_status deeds_image_stats(const float* im, size_t count, float* mean, float* stddev) {
    if (!im || !mean || !stddev || count == 0) return fail(nullptr, DEEDS_ERR_INVALID, "deeds_image_stats: bad args");
    image_stats(im, count, mean, stddev);
    return DEEDS_OK;
}

deeds_status deeds_prims_from_sad(const float* sad, float stddev, int m1, int n1, int o1, int g, int* ordered,
                                  int* parents, float* edgemst) {
    if (!sad || !ordered || !parents || !edgemst || m1 < 1 || n1 < 1 || o1 < 1 || g < 1)
        return fail(nullptr, DEEDS_ERR_INVALID, "deeds_prims_from_sad: bad args");
    prims_from_sad(sad, stddev, m1, n1, o1, g, ordered, parents, edgemst);
    return DEEDS_OK;
}

deeds_status deeds_mind_ssc_dev(deeds_ctx* ctx, const float* d_im, int m, int n, int o, int qs, uint64_t* d_codes,
                                void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_im || !d_codes) return fail(ctx, DEEDS_ERR_INVALID, "null pointer");
    if (qs < 1 || qs > 7) return fail(ctx, DEEDS_ERR_INVALID, "MIND radius %d outside 1..7", qs);
    if (m < 2 * qs + 1 || n < 2 * qs + 1 || o < 2 * qs + 1)
        return fail(ctx, DEEDS_ERR_INVALID, "volume %dx%dx%d too small for radius %d", m, n, o, qs);
    CK(cudaSetDevice(ctx->device));
    deeds_status st = DEEDS_OK;
    float* scratch = dbuf<float>(ctx, "mind", (size_t)6 * m * n * o, &st);
    if (st) return st;
    float thr[5];
    mind_thresholds(thr);
    CK(launch_mind_ssc(d_im, m, n, o, qs, thr, scratch, d_codes, (cudaStream_t)stream));
    return DEEDS_OK;
}

deeds_status deeds_data_cost_dev(deeds_ctx* ctx, const uint64_t* d_F, const uint64_t* d_M, int m, int n, int o, int g,
                                 int hw, int q, float alpha, float* d_cost, void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_F || !d_M || !d_cost) return fail(ctx, DEEDS_ERR_INVALID, "null pointer");
    if (g < 1 || hw < 0 || q < 1 || m / g < 1 || n / g < 1 || o / g < 1)
        return fail(ctx, DEEDS_ERR_INVALID, "bad grid %d / radius %d / quant %d", g, hw, q);
    CK(cudaSetDevice(ctx->device));
    deeds_status st = DEEDS_OK;
    uint64_t* mpad = dbuf<uint64_t>(ctx, "mpad_stage", padded_codes_count(m, n, o, q * hw), &st);
    int* d_err = dbuf<int>(ctx, "err_dc_stage", 1, &st);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    CK(cudaMemsetAsync(d_err, 0, sizeof(int), s));
    CK(data_cost_auto(ctx, d_F, d_M, mpad, m, n, o, g, hw, q, alpha, d_cost, d_err, s));
    int herr = 0;
    CK(cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (herr) return fail(ctx, DEEDS_ERR_TIMEOUT, "cost volume: a bounded wait for a TMA copy expired");
    return DEEDS_OK;
}

deeds_status deeds_mst_edges_dev(deeds_ctx* ctx, const float* d_im, int m, int n, int o, int g, float* d_sad,
                                 void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_im || !d_sad || g < 1 || m / g < 1 || n / g < 1 || o / g < 1)
        return fail(ctx, DEEDS_ERR_INVALID, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    CK(launch_edge_sad(d_im, m, n, o, g, d_sad, (cudaStream_t)stream));
    return DEEDS_OK;
}

void deeds_mst_path_counts(long long out[4]) {
    if (out) mst_path_counts(out);
}

deeds_status deeds_image_stats_dev(deeds_ctx* ctx, const float* d_im, size_t count, float* d_out, void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_im || !d_out || count == 0) return fail(ctx, DEEDS_ERR_INVALID, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    deeds_status st = DEEDS_OK;
    void* scr = dbuf<char>(ctx, "stats_scr_api", image_stats_scratch_bytes(count, 1), &st);
    if (st) return st;
    CK(launch_image_stats(d_im, nullptr, 1, count, scr, d_out, (cudaStream_t)stream));
    return DEEDS_OK;
}

deeds_status deeds_tree_bp_dev(deeds_ctx* ctx, float* d_cost, const float* d_u0, const float* d_v0, const float* d_w0,
                               int m1, int n1, int o1, int hw, int q, const int* ordered, const int* parents,
                               const float* edgemst, float* d_u1, float* d_v1, float* d_w1, int16_t* d_allinds,
                               void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_cost || !d_u0 || !d_v0 || !d_w0 || !ordered || !parents || !edgemst || !d_u1 || !d_v1 || !d_w1)
        return fail(ctx, DEEDS_ERR_INVALID, "null pointer");
    if (hw < 0 || hw > 10 || q < 1) return fail(ctx, DEEDS_ERR_INVALID, "radius %d / quant %d", hw, q);
    if (reinterpret_cast<uintptr_t>(d_allinds) & 15)
        return fail(ctx, DEEDS_ERR_INVALID, "d_allinds must be 16-byte aligned");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = (cudaStream_t)stream;
    const int sz = m1 * n1 * o1;
    const int len = 2 * hw + 1;
    deeds_status st = DEEDS_OK;
    PackedTree pt = pack_layout(sz);
    uint32_t* h = hbuf<uint32_t>(ctx, "tree_stage", pt.total, &st);
    short* allinds = reinterpret_cast<short*>(d_allinds);  // NULL: no tables (the downward pass evaluates its entries)
    int* d_err = dbuf<int>(ctx, "err_stage", 1, &st);
    if (st) return st;
    CK(cudaStreamSynchronize(s));  // the pinned staging block is reused across calls
    std::memcpy(h + pt.o_ordered, ordered, sizeof(int) * sz);
    std::memcpy(h + pt.o_parents, parents, sizeof(int) * sz);
    std::memcpy(h + pt.o_edgemst, edgemst, sizeof(float) * sz);
    TreeSchedule sch;
    build_schedule(ordered, parents, sz, sch);
    pack_schedule(sch, h, pt);
    CK(cudaMemsetAsync(d_err, 0, sizeof(int), s));
    st = run_tree_bp(ctx, "stage", pt, h, d_cost, allinds, len, q, d_u0, d_v0, d_w0, d_u1, d_v1, d_w1, d_err, s);
    if (st) return st;
    int herr = 0;
    CK(cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (ctx->prof) collect_marks(ctx);
    if (herr == 4) return fail(ctx, DEEDS_ERR_TIMEOUT, "belief propagation: a bounded wait for a parent's label expired");
    if (herr) return fail(ctx, DEEDS_ERR_INTERNAL, "belief propagation produced an out-of-range argmin index");
    return DEEDS_OK;
}

deeds_status deeds_upsample_dev(const float* d_u0, const float* d_v0, const float* d_w0, int m2, int n2, int o2,
                                float* d_u, float* d_v, float* d_w, int m, int n, int o, void* stream) {
    deeds_ctx* ctx = nullptr;
    if (!d_u0 || !d_v0 || !d_w0 || !d_u || !d_v || !d_w || m2 < 1 || n2 < 1 || o2 < 1 || m < 1 || n < 1 || o < 1)
        return fail(nullptr, DEEDS_ERR_INVALID, "deeds_upsample_dev: bad arguments");
    CK(launch_upsample(d_u0, d_v0, d_w0, m2, n2, o2, d_u, d_v, d_w, m, n, o, (cudaStream_t)stream));
    return DEEDS_OK;
}

deeds_status deeds_warp_affine_dev(const float* d_in, const float X[16], const float* d_u, const float* d_v,
                                   const float* d_w, int m, int n, int o, float* d_out, void* stream) {
    deeds_ctx* ctx = nullptr;
    if (!d_in || !X || !d_out || m < 1 || n < 1 || o < 1)
        return fail(nullptr, DEEDS_ERR_INVALID, "deeds_warp_affine_dev: bad arguments");
    FieldRef f{(d_u && d_v && d_w) ? 1 : 0, d_u, d_v, d_w, 0, 0, 0};
    CK(launch_warp_affine(d_in, X, f, m, n, o, d_out, nullptr, nullptr, nullptr, (cudaStream_t)stream));
    return DEEDS_OK;
}

deeds_status deeds_warp_image_dev(const float* d_in, const float* d_u, const float* d_v, const float* d_w, int m, int n,
                                  int o, float* d_out, void* stream) {
    deeds_ctx* ctx = nullptr;
    if (!d_in || !d_u || !d_v || !d_w || !d_out || m < 1 || n < 1 || o < 1)
        return fail(nullptr, DEEDS_ERR_INVALID, "deeds_warp_image_dev: bad arguments");
    FieldRef f{1, d_u, d_v, d_w, 0, 0, 0};
    CK(launch_warp_image(d_in, f, m, n, o, d_out, (cudaStream_t)stream));
    return DEEDS_OK;
}

deeds_status deeds_warp_seg_dev(const int16_t* d_in, const float X[16], const float* d_u, const float* d_v,
                                const float* d_w, int m, int n, int o, int16_t* d_out, void* stream) {
    deeds_ctx* ctx = nullptr;
    if (!d_in || !X || !d_out || m < 1 || n < 1 || o < 1)
        return fail(nullptr, DEEDS_ERR_INVALID, "deeds_warp_seg_dev: bad arguments");
    FieldRef f{(d_u && d_v && d_w) ? 1 : 0, d_u, d_v, d_w, 0, 0, 0};
    CK(launch_warp_seg(reinterpret_cast<const short*>(d_in), X, f, m, n, o, reinterpret_cast<short*>(d_out),
                       (cudaStream_t)stream));
    return DEEDS_OK;
}

deeds_status deeds_consistent_dev(deeds_ctx* ctx, float* d_u, float* d_v, float* d_w, float* d_u2, float* d_v2,
                                  float* d_w2, int m, int n, int o, int g, void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_u || !d_v || !d_w || !d_u2 || !d_v2 || !d_w2 || m < 1 || n < 1 || o < 1 || g < 1)
        return fail(ctx, DEEDS_ERR_INVALID, "bad arguments");
    if (n > 65535 || o > 65535)  // grid y / z of the iteration kernel; checked before any launch
        return fail(ctx, DEEDS_ERR_INVALID, "deeds_consistent_dev: n and o must be at most 65535");
    CK(cudaSetDevice(ctx->device));
    deeds_status st = DEEDS_OK;
    float* scratch = dbuf<float>(ctx, "consistent", (size_t)12 * m * n * o, &st);
    if (st) return st;
    CK(launch_consistent(d_u, d_v, d_w, d_u2, d_v2, d_w2, m, n, o, g, scratch, (cudaStream_t)stream));
    return DEEDS_OK;
}

deeds_status deeds_jacobian_dev(deeds_ctx* ctx, const float* d_u, const float* d_v, const float* d_w, int m, int n,
                                int o, int g, float* jstd, float* neg_frac, void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_u || !d_v || !d_w || m < 1 || n < 1 || o < 1 || g < 1) return fail(ctx, DEEDS_ERR_INVALID, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    deeds_status st = DEEDS_OK;
    double* acc = dbuf<double>(ctx, "jac", 3, &st);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    CK(launch_jacobian(d_u, d_v, d_w, m, n, o, g, acc, s));
    double h[3];
    CK(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const double cnt = (double)m * n * o;
    const double mean = h[0] / cnt;
    const double var = cnt > 1 ? (h[1] - cnt * mean * mean) / (cnt - 1) : 0.0;
    if (jstd) *jstd = (float)std::sqrt(var > 0 ? var : 0.0);
    if (neg_frac) *neg_frac = (float)(h[2] / cnt);
    return DEEDS_OK;
}

deeds_status deeds_register_dev(deeds_ctx* ctx, const float* d_fixed, const float* d_moving, int m, int n, int o,
                                const float X[16], const deeds_params* P, float* d_flow_out, float* d_warped_out,
                                void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_fixed || !d_moving || !X || !d_flow_out) return fail(ctx, DEEDS_ERR_INVALID, "null pointer");
    deeds_status st = check_params(ctx, P, m, n, o);
    if (st) return st;
    CK(cudaSetDevice(ctx->device));
    // forward chain on the context's stream (after the caller's stream has reached
    // this call: the inputs), backward chain on the context's second stream; the
    // call returns when all of it is done
    cudaStream_t s = ctx->stream;
    if ((cudaStream_t)stream != s) {
        CK(cudaEventRecord(ctx->ev_d, (cudaStream_t)stream));
        CK(cudaStreamWaitEvent(s, ctx->ev_d, 0));
    }
    cudaStream_t sd[2] = {s, ctx->stream_b};
    const int L = P->levels;
    const size_t sz = (size_t)m * n * o;
    float thr[5];
    mind_thresholds(thr);

    Timeline tl;
    tl.start();
    PairBuffers B;
    st = acquire_buffers(ctx, m, n, o, P, B);
    if (st) return st;
    const size_t max_sz1 = B.max_sz1;
    const std::vector<int>& m1s = B.m1s;
    const std::vector<int>& n1s = B.n1s;
    const std::vector<int>& o1s = B.o1s;
    float* fix = B.fix;
    float* mov = B.mov;
    float* warp0 = B.warp0;
    int* d_err = B.d_err;
    float** warped = B.warped;
    uint64_t** c_warp = B.c_warp;
    float** mind_scr = B.mind_scr;
    float** cost = B.cost;
    uint64_t** mpad = B.mpad;
    const char* tags[2] = {"f", "b"};
    float* grid = B.grid;
    float* cons_scr = B.cons_scr;
    float* h_stats = B.h_stats;
    std::vector<float*>& h_sad = B.h_sad;
    std::vector<float*>& d_sad = B.d_sad;
    std::vector<PackedTree>& pts = B.pts;
    std::vector<uint32_t*>& h_tree = B.h_tree;
    float* prev[6];  // u1 v1 w1 u1i v1i w1i on the previous grid
    float* cur0[6];  // u0 v0 w0 on the current grid, per direction
    float* nxt[6];   // new fields on the current grid
    for (int i = 0; i < 6; i++) {
        prev[i] = grid + i * max_sz1;
        cur0[i] = grid + (6 + i) * max_sz1;
        nxt[i] = grid + (12 + i) * max_sz1;
    }

    // ---- inputs, affine-only warp of the moving image
    // MST-input events: [0] affine-warped moving image ready, [1] image statistics on
    // the host, [2 + t] block SADs of tree t on the host (t = 2 level + direction)
    while (ctx->ev_mst.size() < 2 + 2 * (size_t)L) {
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->ev_mst.push_back(e);
    }
    cudaEvent_t* ev = ctx->ev_mst.data();
    tl.dmark("start", s);
    CK(cudaMemsetAsync(d_err, 0, 2 * sizeof(int), s));
    CK(launch_shift(d_fixed, fix, (int64_t)sz, P->intensity_shift, s));
    CK(launch_shift(d_moving, mov, (int64_t)sz, P->intensity_shift, s));
    {
        StageScope sc(ctx, DEEDS_STAGE_TRANSFORM, s);
        FieldRef zero{0, nullptr, nullptr, nullptr, 0, 0, 0};
        CK(launch_warp_affine(mov, X, zero, m, n, o, warp0, nullptr, nullptr, nullptr, s));
    }
    CK(cudaEventRecord(ev[0], s));

    // ---- MST inputs on the side stream, to the host trees on worker threads: the
    // image statistics of both images (exact, on the device), then the block SADs
    // in the order the trees are needed: the finest forward tree takes longest on
    // the host, the first level's trees start the device's level loop, the finest
    // backward tree is next longest, then the other levels.  Each tree starts as
    // soon as its own inputs are on the host.
    CK(cudaStreamWaitEvent(ctx->side, ev[0], 0));
    {
        StageScope sc(ctx, DEEDS_STAGE_MST, ctx->side);
        CK(launch_image_stats(fix, warp0, 2, sz, B.stats_scr, B.d_stats, ctx->side));
    }
    CK(cudaMemcpyAsync(h_stats, B.d_stats, 4 * sizeof(float), cudaMemcpyDeviceToHost, ctx->side));
    CK(cudaEventRecord(ev[1], ctx->side));
    {
        std::vector<int> order = {2 * (L - 1)};
        if (L > 1) order.insert(order.end(), {0, 1});
        order.push_back(2 * (L - 1) + 1);
        for (int l = L - 2; l >= 1; l--) order.insert(order.end(), {2 * l, 2 * l + 1});
        for (int t : order) {
            const int l = t / 2, d = t % 2;
            const size_t sz1 = (size_t)m1s[l] * n1s[l] * o1s[l];
            {
                StageScope sc(ctx, DEEDS_STAGE_MST, ctx->side);
                CK(launch_edge_sad(d == 0 ? fix : warp0, m, n, o, P->grid[l], d_sad[t], ctx->side));
            }
            CK(cudaMemcpyAsync(h_sad[t], d_sad[t], 6 * sz1 * sizeof(float), cudaMemcpyDeviceToHost, ctx->side));
            CK(cudaEventRecord(ev[2 + t], ctx->side));
        }
    }
    std::vector<std::promise<void>> ready(2 * L);
    std::vector<std::shared_future<void>> ready_f(2 * L);
    for (int t = 0; t < 2 * L; t++) ready_f[t] = ready[t].get_future().share();
    const int dev = ctx->device;
    std::thread builder([&, ev, dev]() {
        cudaSetDevice(dev);
        // finest trees are the slowest: start the workers in reverse level order
        std::vector<std::thread> workers;
        for (int t = 2 * L - 1; t >= 0; t--) {
            workers.emplace_back([&, t]() {
                const int l = t / 2, d = t % 2;
                try {
                    cudaSetDevice(dev);
                    if (cudaEventSynchronize(ev[1]) != cudaSuccess || cudaEventSynchronize(ev[2 + t]) != cudaSuccess)
                        throw std::runtime_error("MST inputs: CUDA error");
                    tl.mark("tree level " + std::to_string(l) + (d ? " backward" : " forward") + " inputs on host");
                    build_tree(h_sad[t], h_stats[2 * d + 1], m1s[l], n1s[l], o1s[l], P->grid[l], h_tree[t], pts[t]);
                    tl.mark("tree level " + std::to_string(l) + (d ? " backward" : " forward") + " built");
                    ready[t].set_value();
                } catch (...) {
                    ready[t].set_exception(std::current_exception());
                }
            });
        }
        for (auto& w : workers) w.join();
    });
    struct Joiner {
        std::thread& t;
        ~Joiner() { if (t.joinable()) t.join(); }
    } joiner{builder};

    // ---- level loop (src/deedsBCV0.cpp:222-330)
    int m2 = m1s[0], n2 = n1s[0], o2 = o1s[0];
    CK(cudaMemsetAsync(grid, 0, 6 * max_sz1 * sizeof(float), s));
    bool bg_joined = false;
    for (int l = 0; l < L; l++) {
        const int g = P->grid[l], hw = P->radius[l], q = P->quant[l];
        const int qs = mind_step(q);
        const int m1 = m1s[l], n1 = n1s[l], o1 = o1s[l];
        const int len = 2 * hw + 1;
        if (P->verbose)
            printf("Level %d grid=%d with sizes: %dx%dx%d hw=%d quant=%d\n", l, g, m1, n1, o1, hw, q);
        const size_t ks = std::find(B.steps.begin(), B.steps.end(), qs) - B.steps.begin();
        uint64_t* c_fix = B.c_fix[ks];
        uint64_t* c_mov = B.c_mov[ks];
        if (ks > 0 && !bg_joined) {  // codes of the background stream (both directions follow s)
            CK(cudaStreamWaitEvent(s, ctx->ev_g, 0));
            bg_joined = true;
        }
        if (l == 0) {
            StageScope sc(ctx, DEEDS_STAGE_MIND, s);
            CK(launch_mind_ssc(warp0, m, n, o, qs, thr, mind_scr[0], c_mov, s));
            CK(launch_mind_ssc(fix, m, n, o, qs, thr, mind_scr[0], c_fix, s));
        }
        int sy, sx, szs;
        float alpha1;
        data_cost_params(g, q, P->alpha, &sy, &sx, &szs, &alpha1);
        // the backward chain starts once the level's shared inputs are ready
        CK(cudaEventRecord(ctx->ev_d, s));
        CK(cudaStreamWaitEvent(sd[1], ctx->ev_d, 0));
        for (int d = 0; d < 2; d++) {
            cudaStream_t sdd = sd[d];
            float** pv = prev + 3 * d;
            float** c0 = cur0 + 3 * d;
            // At the first level the forward field is zero, and warpAffine with the
            // upsampled zero field adds +0 to the same coordinates as the affine-only
            // warp: the warped moving image is warp0 bit for bit, and its codes are
            // the level's field-independent ones (c_mov), so they are not recomputed.
            const bool reuse = l == 0 && d == 0;
            {
                StageScope sc(ctx, DEEDS_STAGE_TRANSFORM, sdd);
                CK(launch_upsample(pv[0], pv[1], pv[2], m2, n2, o2, c0[0], c0[1], c0[2], m1, n1, o1, sdd));
                FieldRef f{2, c0[0], c0[1], c0[2], m1, n1, o1};
                if (d == 0 && !reuse)
                    CK(launch_warp_affine(mov, X, f, m, n, o, warped[d], nullptr, nullptr, nullptr, sdd));
                else if (d == 1)
                    CK(launch_warp_image(fix, f, m, n, o, warped[d], sdd));
            }
            if (!reuse) {
                StageScope sc(ctx, DEEDS_STAGE_MIND, sdd);
                CK(launch_mind_ssc(warped[d], m, n, o, qs, thr, mind_scr[d], c_warp[d], sdd));
            }
            // The first level's cost volumes (long-running CTAs that fill the SMs) do
            // not wait for the image statistics: beside them the latency-bound
            // statistics kernels take longer and the host trees start ~1 ms later,
            // but the finest trees are still built by the time the level loop needs
            // them, and the loop itself starts ~1.6 ms earlier (61.6 -> 60.2 ms per
            // 192x160x256 pair, measured both ways).
            {
                StageScope sc(ctx, DEEDS_STAGE_DATACOST, sdd);
                CK(data_cost_auto(ctx, d == 0 ? c_fix : c_mov, reuse ? c_mov : c_warp[d], mpad[d], m, n, o, g, hw, q,
                                  P->alpha, cost[d], d_err + d, sdd));
            }
            CK(cudaEventRecord(ctx->ev_cost[d], sdd));
        }
        if (l == 0 && B.steps.size() > 1) {
            // the other levels' field-independent codes on their own stream, after both
            // directions' level-0 cost volumes: they run while the coarsest tree sweeps
            // leave most of the GPU idle; the first level that needs them waits (ev_g)
            CK(cudaEventRecord(ctx->ev_e, sd[0]));
            CK(cudaEventRecord(ctx->ev_f, sd[1]));
            CK(cudaStreamWaitEvent(ctx->bg, ctx->ev_e, 0));
            CK(cudaStreamWaitEvent(ctx->bg, ctx->ev_f, 0));
            {
                StageScope sc(ctx, DEEDS_STAGE_MIND, ctx->bg);
                for (size_t k = 1; k < B.steps.size(); k++) {
                    CK(launch_mind_ssc(warp0, m, n, o, B.steps[k], thr, B.mind_bg, B.c_mov[k], ctx->bg));
                    CK(launch_mind_ssc(fix, m, n, o, B.steps[k], thr, B.mind_bg, B.c_fix[k], ctx->bg));
                }
            }
            CK(cudaEventRecord(ctx->ev_g, ctx->bg));
        }
        // each direction's sweeps are queued as soon as its own tree is built (the two
        // directions' trees finish at different times; their streams are independent)
        bool queued[2] = {false, false};
        for (int k = 0; k < 2; k++) {
            int d = -1;
            {
                const auto w0 = std::chrono::steady_clock::now();
                tl.mark("level " + std::to_string(l) + " waits for a tree");
                while (d < 0) {
                    for (int c = 0; c < 2 && d < 0; c++)
                        if (!queued[c] && ready_f[2 * l + c].wait_for(std::chrono::seconds(0)) == std::future_status::ready)
                            d = c;
                    if (d < 0) ready_f[2 * l + (queued[0] ? 1 : 0)].wait_for(std::chrono::microseconds(50));
                }
                queued[d] = true;
                try {
                    ready_f[2 * l + d].get();
                } catch (const std::exception& ex) {
                    return fail(ctx, DEEDS_ERR_INTERNAL, "MST construction failed: %s", ex.what());
                }
                if (ctx->prof)
                    ctx->stage_ms[DEEDS_STAGE_TREE_WAIT] +=
                        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
            }
            const int t = 2 * l + d;
            // a sweep is latency bound and runs at about half speed beside a cost-volume
            // kernel on the same SMs (2.8 ms alone, 7.9 ms beside one at grid 8), so it
            // starts once the other direction's cost volume is done too
            CK(cudaStreamWaitEvent(sd[d], ctx->ev_cost[1 - d], 0));
            tl.dmark("level " + std::to_string(l) + (d ? " backward" : " forward") + " BP starts", sd[d]);
            st = run_tree_bp(ctx, tags[d], pts[t], h_tree[t], cost[d], nullptr, len, q, cur0[3 * d],
                             cur0[3 * d + 1], cur0[3 * d + 2], nxt[3 * d], nxt[3 * d + 1], nxt[3 * d + 2], d_err + d,
                             sd[d],
                             &tl, "level " + std::to_string(l) + (d ? " backward" : " forward"), 2);
            if (st) return st;
            tl.dmark("level " + std::to_string(l) + (d ? " backward" : " forward") + " BP done", sd[d]);
        }
        CK(cudaEventRecord(ctx->ev_d, sd[1]));
        CK(cudaStreamWaitEvent(s, ctx->ev_d, 0));
        {
            StageScope sc(ctx, DEEDS_STAGE_CONSISTENT, s);
            CK(launch_consistent(nxt[0], nxt[1], nxt[2], nxt[3], nxt[4], nxt[5], m1, n1, o1, g, cons_scr, s));
        }
        if (P->verbose) {
            float js = 0, neg = 0;
            deeds_status js_st = deeds_jacobian_dev(ctx, nxt[0], nxt[1], nxt[2], m1, n1, o1, g, &js, &neg, s);
            if (js_st == DEEDS_OK)
                printf("std(J)=%.2f (J<0)=%.2fe-7\n", std::round(js * 100) / 100.0, std::round(neg * 1e7) / 100.0);
        }
        for (int i = 0; i < 6; i++) std::swap(prev[i], nxt[i]);
        m2 = m1; n2 = n1; o2 = o1;
    }

    // ---- outputs (src/deedsBCV0.cpp:339-356): the control-grid flow, kept on the
    // context as well (deeds_warp_segmentation upsamples it on the fly, with the
    // arithmetic of upsample-then-warp); the warped moving image only on request
    const size_t sz1 = (size_t)m2 * n2 * o2;
    if (prev[1] == prev[0] + sz1 && prev[2] == prev[1] + sz1) {  // u, v, w adjacent (finest grid)
        CK(cudaMemcpyAsync(d_flow_out, prev[0], 3 * sz1 * sizeof(float), cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(B.kgrid, prev[0], 3 * sz1 * sizeof(float), cudaMemcpyDeviceToDevice, s));
    } else {
        for (int c = 0; c < 3; c++) {
            CK(cudaMemcpyAsync(d_flow_out + c * sz1, prev[c], sz1 * sizeof(float), cudaMemcpyDeviceToDevice, s));
            CK(cudaMemcpyAsync(B.kgrid + c * sz1, prev[c], sz1 * sizeof(float), cudaMemcpyDeviceToDevice, s));
        }
    }
    if (d_warped_out) {
        StageScope sc(ctx, DEEDS_STAGE_TRANSFORM, s);
        FieldRef f{2, prev[0], prev[1], prev[2], m2, n2, o2};
        CK(launch_warp_affine(mov, X, f, m, n, o, warped[0], nullptr, nullptr, nullptr, s));
        CK(launch_shift(warped[0], d_warped_out, (int64_t)sz, -P->intensity_shift, s));
    }
    tl.dmark("output done", s);
    int herr[2] = {0, 0};
    CK(cudaMemcpyAsync(herr, d_err, sizeof(herr), cudaMemcpyDeviceToHost, s));
    tl.mark("all work queued");
    CK(cudaStreamSynchronize(s));
    tl.mark("device done");
    if (builder.joinable()) builder.join();
    tl.dump();
    if (ctx->prof) collect_marks(ctx);
    if (herr[0] == 3 || herr[1] == 3) return fail(ctx, DEEDS_ERR_TIMEOUT, "cost volume: a bounded wait for a TMA copy expired");
    if (herr[0] == 4 || herr[1] == 4)
        return fail(ctx, DEEDS_ERR_TIMEOUT, "belief propagation: a bounded wait for a parent's label expired");
    if (herr[0] || herr[1])
        return fail(ctx, DEEDS_ERR_INTERNAL, "belief propagation produced an out-of-range argmin index");
    ctx->have_field = true;
    ctx->fm = m; ctx->fn = n; ctx->fo = o;
    ctx->fm1 = m2; ctx->fn1 = n2; ctx->fo1 = o2;
    std::memcpy(ctx->fX, X, sizeof(ctx->fX));
    return DEEDS_OK;
}

deeds_status deeds_register(deeds_ctx* ctx, const float* fixed, const float* moving, int m, int n, int o,
                            const float X[16], const deeds_params* params, float* flow_out, float* warped_out) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!fixed || !moving || !X || !flow_out) return fail(ctx, DEEDS_ERR_INVALID, "null pointer");
    deeds_status st = check_params(ctx, params, m, n, o);
    if (st) return st;
    CK(cudaSetDevice(ctx->device));
    const size_t sz = (size_t)m * n * o;
    const int gl = params->grid[params->levels - 1];
    const size_t sz1 = (size_t)(m / gl) * (n / gl) * (o / gl);
    float* d_f = dbuf<float>(ctx, "in_fixed", sz, &st);
    float* d_m = dbuf<float>(ctx, "in_moving", sz, &st);
    float* d_flow = dbuf<float>(ctx, "out_flow", 3 * sz1, &st);
    float* d_w = warped_out ? dbuf<float>(ctx, "out_warped", sz, &st) : nullptr;
    if (st) return st;
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(d_f, fixed, sz * sizeof(float), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_m, moving, sz * sizeof(float), cudaMemcpyHostToDevice, s));
    st = deeds_register_dev(ctx, d_f, d_m, m, n, o, X, params, d_flow, d_w, s);
    if (st) return st;
    CK(cudaMemcpyAsync(flow_out, d_flow, 3 * sz1 * sizeof(float), cudaMemcpyDeviceToHost, s));
    if (warped_out) CK(cudaMemcpyAsync(warped_out, d_w, sz * sizeof(float), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return DEEDS_OK;
}

deeds_status deeds_register_batch(deeds_ctx* ctx, const deeds_pair* pairs, int n_pairs, const deeds_params* params,
                                  int lanes) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (n_pairs < 0 || (n_pairs > 0 && !pairs)) return fail(ctx, DEEDS_ERR_INVALID, "bad pair list");
    if (n_pairs == 0) return DEEDS_OK;
    for (int i = 0; i < n_pairs; i++) {
        const deeds_pair& p = pairs[i];
        if (!p.fixed || !p.moving || !p.flow_out) return fail(ctx, DEEDS_ERR_INVALID, "pair %d: null pointer", i);
        deeds_status st = check_params(ctx, params, p.m, p.n, p.o);
        if (st) return fail(ctx, st, "pair %d: %s", i, ctx->err.c_str());
    }
    if (lanes <= 0) lanes = 3;
    if (lanes > n_pairs) lanes = n_pairs;
    while ((int)ctx->lanes.size() < lanes) {
        deeds_ctx* lane = nullptr;
        deeds_status st = deeds_create(&lane, ctx->device);
        if (st) return fail(ctx, st, "batch lane: %s", deeds_last_error(nullptr));
        lane->tune = ctx->tune;
        ctx->lanes.push_back(lane);
    }
    // size every lane's buffers for the largest pair up front: growing a buffer
    // mid-batch would cudaFree, which synchronises the whole device
    for (deeds_ctx* lane : ctx->lanes) {
        for (int i = 0; i < n_pairs; i++) {
            deeds_status st = reserve_buffers(lane, pairs[i].m, pairs[i].n, pairs[i].o, params, pairs[i].warped_out != nullptr);
            if (st) return fail(ctx, st, "batch lane: %s", lane->err.c_str());
        }
    }
    std::atomic<int> next{0};
    std::atomic<int> failed{-1};
    std::vector<deeds_status> lane_st(lanes, DEEDS_OK);
    std::vector<std::string> lane_err(lanes);
    std::vector<std::thread> threads;
    for (int li = 0; li < lanes; li++) {
        threads.emplace_back([&, li]() {
            deeds_ctx* lane = ctx->lanes[li];
            float ident[16];
            for (int i = 0; i < 16; i++) ident[i] = (i % 5 == 0) ? 1.0f : 0.0f;
            for (;;) {
                if (failed.load() >= 0) return;
                const int i = next.fetch_add(1);
                if (i >= n_pairs) return;
                const deeds_pair& p = pairs[i];
                const deeds_status st = deeds_register(lane, p.fixed, p.moving, p.m, p.n, p.o, p.X ? p.X : ident,
                                                       params, p.flow_out, p.warped_out);
                if (st) {
                    lane_st[li] = st;
                    lane_err[li] = "pair " + std::to_string(i) + ": " + lane->err;
                    int expect = -1;
                    failed.compare_exchange_strong(expect, li);
                    return;
                }
            }
        });
    }
    for (auto& t : threads) t.join();
    if (failed.load() >= 0) {
        const int li = failed.load();
        return fail(ctx, lane_st[li], "%s", lane_err[li].c_str());
    }
    return DEEDS_OK;
}

deeds_status deeds_warp_segmentation(deeds_ctx* ctx, const int16_t* seg, int16_t* seg_out) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!seg || !seg_out) return fail(ctx, DEEDS_ERR_INVALID, "null pointer");
    if (!ctx->have_field) return fail(ctx, DEEDS_ERR_INVALID, "no registration has been run on this context");
    CK(cudaSetDevice(ctx->device));
    const size_t sz = (size_t)ctx->fm * ctx->fn * ctx->fo;
    deeds_status st = DEEDS_OK;
    short* d_in = dbuf<short>(ctx, "seg_in", sz, &st);
    short* d_out = dbuf<short>(ctx, "seg_out", sz, &st);
    if (st) return st;
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(d_in, seg, sz * sizeof(short), cudaMemcpyHostToDevice, s));
    float* kg = static_cast<float*>(ctx->dev["keep_grid"].p);
    const size_t sz1 = (size_t)ctx->fm1 * ctx->fn1 * ctx->fo1;
    FieldRef f{2, kg, kg + sz1, kg + 2 * sz1, ctx->fm1, ctx->fn1, ctx->fo1};
    CK(launch_warp_seg(d_in, ctx->fX, f, ctx->fm, ctx->fn, ctx->fo, d_out, s));
    CK(cudaMemcpyAsync(seg_out, d_out, sz * sizeof(short), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return DEEDS_OK;
}

deeds_status deeds_apply_flow(deeds_ctx* ctx, const float* flow, size_t flow_len, int g, const float X[16],
                              const void* in, int dtype, int m, int n, int o, void* out) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!flow || !X || !in || !out || m < 1 || n < 1 || o < 1 || (dtype != 0 && dtype != 1))
        return fail(ctx, DEEDS_ERR_INVALID, "bad arguments");
    if (flow_len < 3 || flow_len % 3) return fail(ctx, DEEDS_ERR_INVALID, "flow length %zu is not 3*sz1", flow_len);
    const size_t sz = (size_t)m * n * o;
    const size_t sz3 = flow_len / 3;
    if (g <= 0) {  // grid step from the file size (src/applyBCV.cpp:163-164)
        const float ratio = (float)sz / (float)sz3;
        g = (int)std::round(std::pow((double)ratio, 0.3333333));
    }
    if (g < 1) return fail(ctx, DEEDS_ERR_INVALID, "inferred grid step %d", g);
    const int m1 = m / g, n1 = n / g, o1 = o / g;
    if ((size_t)m1 * n1 * o1 != sz3 || m1 < 1 || n1 < 1 || o1 < 1)
        return fail(ctx, DEEDS_ERR_INVALID, "flow of %zu nodes does not match grid step %d on %dx%dx%d", sz3, g, m, n, o);
    CK(cudaSetDevice(ctx->device));
    deeds_status st = DEEDS_OK;
    float* d_flow = dbuf<float>(ctx, "apply_flow", flow_len, &st);
    const size_t esz = dtype == 0 ? sizeof(short) : sizeof(float);
    void* d_in = dbuf<char>(ctx, "apply_in", sz * esz, &st);
    void* d_out = dbuf<char>(ctx, "apply_out", sz * esz, &st);
    if (st) return st;
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(d_flow, flow, flow_len * sizeof(float), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_in, in, sz * esz, cudaMemcpyHostToDevice, s));
    FieldRef f{2, d_flow, d_flow + sz3, d_flow + 2 * sz3, m1, n1, o1};
    if (dtype == 0)
        CK(launch_warp_seg(static_cast<short*>(d_in), X, f, m, n, o, static_cast<short*>(d_out), s));
    else
        CK(launch_warp_affine(static_cast<float*>(d_in), X, f, m, n, o, static_cast<float*>(d_out), nullptr, nullptr,
                              nullptr, s));
    CK(cudaMemcpyAsync(out, d_out, sz * esz, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return DEEDS_OK;
}

deeds_status deeds_fuse_labels_dev(deeds_ctx* ctx, const float* d_target, const float* const* d_images,
                                   const int16_t* const* d_labels, int n_atlas, int m, int n, int o, int radius,
                                   float eps, int power, int16_t* d_out, void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_target || !d_images || !d_labels || !d_out || m < 1 || n < 1 || o < 1)
        return fail(ctx, DEEDS_ERR_INVALID, "bad arguments");
    if (n_atlas < 1 || n_atlas > DEEDS_FUSE_MAX_ATLASES)
        return fail(ctx, DEEDS_ERR_INVALID, "%d atlases (1..%d)", n_atlas, DEEDS_FUSE_MAX_ATLASES);
    if (radius < 0 || power < 0 || !(eps > 0.0f)) return fail(ctx, DEEDS_ERR_INVALID, "radius/power/eps");
    FusionAtlases at{};
    for (int a = 0; a < n_atlas; a++) {
        if (!d_images[a] || !d_labels[a]) return fail(ctx, DEEDS_ERR_INVALID, "atlas %d: null pointer", a);
        at.image[a] = d_images[a];
        at.labels[a] = d_labels[a];
    }
    CK(cudaSetDevice(ctx->device));
    deeds_status st = DEEDS_OK;
    float* scr = dbuf<float>(ctx, "fuse_scratch", fuse_scratch_floats(n_atlas, m, n, o), &st);
    if (st) return st;
    CK(launch_fuse_labels(d_target, at, n_atlas, m, n, o, radius, eps, power, scr, d_out, (cudaStream_t)stream));
    return DEEDS_OK;
}

deeds_status deeds_multi_atlas(deeds_ctx* ctx, const float* target, const float* const* atlas_images,
                               const int16_t* const* atlas_labels, int n_atlas, int m, int n, int o,
                               const deeds_params* params, int lanes, int radius, float eps, int power,
                               int16_t* labels_out, int16_t* warped_labels_out, float* warped_images_out) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!target || !atlas_images || !atlas_labels || !labels_out || m < 1 || n < 1 || o < 1)
        return fail(ctx, DEEDS_ERR_INVALID, "bad arguments");
    if (n_atlas < 1 || n_atlas > DEEDS_FUSE_MAX_ATLASES)
        return fail(ctx, DEEDS_ERR_INVALID, "%d atlases (1..%d)", n_atlas, DEEDS_FUSE_MAX_ATLASES);
    deeds_params P;
    if (params) P = *params;
    else deeds_default_params(&P);
    if (P.levels < 1 || P.levels > 10) return fail(ctx, DEEDS_ERR_INVALID, "levels %d", P.levels);
    const size_t sz = (size_t)m * n * o;
    const int g = P.grid[P.levels - 1];
    if (g < 1 || m / g < 1 || n / g < 1 || o / g < 1) return fail(ctx, DEEDS_ERR_INVALID, "grid step %d", g);
    const size_t sz1 = (size_t)(m / g) * (n / g) * (o / g);
    // 1. every atlas registered to the target
    std::vector<float> flows(n_atlas * 3 * sz1), own_images;
    float* warped = warped_images_out;
    if (!warped) {
        own_images.resize((size_t)n_atlas * sz);
        warped = own_images.data();
    }
    std::vector<deeds_pair> pairs(n_atlas);
    for (int a = 0; a < n_atlas; a++) {
        if (!atlas_images[a] || !atlas_labels[a]) return fail(ctx, DEEDS_ERR_INVALID, "atlas %d: null pointer", a);
        pairs[a] = deeds_pair{target, atlas_images[a], m, n, o, nullptr, flows.data() + a * 3 * sz1, warped + a * sz};
    }
    deeds_status st = deeds_register_batch(ctx, pairs.data(), n_atlas, &P, lanes);
    if (st) return st;
    // 2. each atlas' labels warped with its flow
    std::vector<int16_t> own;
    int16_t* wl = warped_labels_out;
    if (!wl) {
        own.resize((size_t)n_atlas * sz);
        wl = own.data();
    }
    float ident[16] = {0};
    ident[0] = ident[5] = ident[10] = ident[15] = 1.0f;
    for (int a = 0; a < n_atlas; a++) {
        st = deeds_apply_flow(ctx, flows.data() + a * 3 * sz1, 3 * sz1, g, ident, atlas_labels[a], 0, m, n, o,
                              wl + a * sz);
        if (st) return st;
    }
    // 3. the vote on the device
    CK(cudaSetDevice(ctx->device));
    float* d_t = dbuf<float>(ctx, "fuse_target", sz, &st);
    float* d_im = dbuf<float>(ctx, "fuse_images", (size_t)n_atlas * sz, &st);
    int16_t* d_lab = dbuf<int16_t>(ctx, "fuse_labels", (size_t)n_atlas * sz, &st);
    int16_t* d_out = dbuf<int16_t>(ctx, "fuse_out", sz, &st);
    if (st) return st;
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(d_t, target, sz * sizeof(float), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_im, warped, (size_t)n_atlas * sz * sizeof(float), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_lab, wl, (size_t)n_atlas * sz * sizeof(int16_t), cudaMemcpyHostToDevice, s));
    std::vector<const float*> ims(n_atlas);
    std::vector<const int16_t*> labs(n_atlas);
    for (int a = 0; a < n_atlas; a++) {
        ims[a] = d_im + a * sz;
        labs[a] = d_lab + a * sz;
    }
    st = deeds_fuse_labels_dev(ctx, d_t, ims.data(), labs.data(), n_atlas, m, n, o, radius, eps, power, d_out, s);
    if (st) return st;
    CK(cudaMemcpyAsync(labels_out, d_out, sz * sizeof(int16_t), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return DEEDS_OK;
}

deeds_status deeds_set_profiling(deeds_ctx* ctx, int on) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    ctx->prof = on != 0;
    return DEEDS_OK;
}

deeds_status deeds_stage_times(deeds_ctx* ctx, float* ms, long long* launches) {
    if (!ctx || !ms) return fail(ctx, DEEDS_ERR_INVALID, "bad arguments");
    for (int i = 0; i < DEEDS_NUM_STAGES; i++) {
        ms[i] = (float)ctx->stage_ms[i];
        if (launches) launches[i] = ctx->stage_launches[i];
    }
    return DEEDS_OK;
}

deeds_status deeds_reset_stage_times(deeds_ctx* ctx) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    for (int i = 0; i < DEEDS_NUM_STAGES; i++) { ctx->stage_ms[i] = 0; ctx->stage_launches[i] = 0; }
    return DEEDS_OK;
}

long long deeds_kernel_launches(void) { return deeds::g_kernel_launches.load(); }

deeds_status deeds_measure_popc_rate(deeds_ctx* ctx, double* rate) {
    if (!ctx || !rate) return fail(ctx, DEEDS_ERR_INVALID, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    deeds_status st = DEEDS_OK;
    unsigned long long* sink = dbuf<unsigned long long>(ctx, "popc_sink", 1, &st);
    if (st) return st;
    const int threads = 256, blocks = ctx->sm_count * 8, iters = 1 << 14;
    cudaStream_t s = ctx->stream;
    CK(launch_popc_probe(blocks, threads, 256, sink, s));  // warm-up
    cudaEvent_t a = pool_event(ctx), b = pool_event(ctx);
    CK(cudaEventRecord(a, s));
    CK(launch_popc_probe(blocks, threads, iters, sink, s));
    CK(cudaEventRecord(b, s));
    CK(cudaEventSynchronize(b));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, a, b));
    ctx->ev_used = 0;
    *rate = (double)blocks * threads * iters * 9.0 / (ms * 1e-3);  // 64-bit samples per second
    return DEEDS_OK;
}

// ---------------------------------------------------------------------------
// Soft-min form (soft.cu)

void deeds_soft_default_params(deeds_soft_params* p) {
    if (!p) return;
    p->grid = 4;
    p->radius = 3;
    p->quant = 1;
    p->mind_radius = 0;
    p->alpha = 1.6f;
    p->tau = 0.5f;
    p->eps = 0.01f;
}

}  // extern "C"

namespace {

deeds_status soft_check(deeds_ctx* ctx, int m, int n, int o, const deeds_soft_params* p, int* qs) {
    if (!p) return fail(ctx, DEEDS_ERR_INVALID, "params is NULL");
    if (p->grid < 1 || p->radius < 0 || p->radius > 5 || p->quant < 1)
        return fail(ctx, DEEDS_ERR_INVALID, "soft level: grid %d radius %d (0..5) quant %d", p->grid, p->radius,
                    p->quant);
    if (!(p->tau > 0.0f) || !(p->eps > 0.0f) || !(p->alpha > 0.0f))
        return fail(ctx, DEEDS_ERR_INVALID, "soft level: tau, eps and alpha must be > 0");
    *qs = p->mind_radius > 0 ? p->mind_radius : mind_step(p->quant);
    if (*qs > 7) return fail(ctx, DEEDS_ERR_INVALID, "MIND radius %d > 7 unsupported", *qs);
    if (m < 2 * *qs + 1 || n < 2 * *qs + 1 || o < 2 * *qs + 1)
        return fail(ctx, DEEDS_ERR_INVALID, "volume %dx%dx%d too small for MIND radius %d", m, n, o, *qs);
    if (m < p->grid || n < p->grid || o < p->grid)
        return fail(ctx, DEEDS_ERR_INVALID, "volume %dx%dx%d smaller than grid %d", m, n, o, p->grid);
    if (n > 65535 || 6LL * o > 65535)  // launch grid limits of the descriptor kernels
        return fail(ctx, DEEDS_ERR_INVALID, "volume %dx%dx%d too large for the soft descriptor", m, n, o);
    return DEEDS_OK;
}

float soft_alpha1(const deeds_soft_params* p) {
    int sy, sx, sz;
    float alpha1;
    data_cost_params(p->grid, p->quant, p->alpha, &sy, &sx, &sz, &alpha1);
    return alpha1;
}

}  // namespace

extern "C" {

deeds_status deeds_soft_descriptor_dev(deeds_ctx* ctx, const float* d_im, int m, int n, int o, int qs, float* d_desc,
                                       void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_im || !d_desc || qs < 1 || qs > 7 || m < 2 * qs + 1 || n < 2 * qs + 1 || o < 2 * qs + 1 || n > 65535 ||
        6LL * o > 65535)
        return fail(ctx, DEEDS_ERR_INVALID, "deeds_soft_descriptor_dev: bad arguments");
    CK(cudaSetDevice(ctx->device));
    deeds_status st = DEEDS_OK;
    float* w6 = dbuf<float>(ctx, "soft_w6", (size_t)6 * m * n * o, &st);
    float* w6b = dbuf<float>(ctx, "soft_w6b", (size_t)6 * m * n * o, &st);
    if (st) return st;
    CK(launch_soft_descriptor(d_im, w6, w6b, d_desc, m, n, o, qs, (cudaStream_t)stream));
    return DEEDS_OK;
}

deeds_status deeds_soft_cost_dev(deeds_ctx* ctx, const float* d_F, const float* d_M, int m, int n, int o,
                                 const deeds_soft_params* p, float* d_cost, void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_F || !d_M || !d_cost) return fail(ctx, DEEDS_ERR_INVALID, "null pointer");
    int qs = 0;
    if (deeds_status e = soft_check(ctx, m, n, o, p, &qs)) return e;
    CK(cudaSetDevice(ctx->device));
    CK(launch_soft_cost(d_F, d_M, d_cost, m, n, o, p->grid, p->radius, p->quant, soft_alpha1(p), p->eps,
                        (cudaStream_t)stream));
    return DEEDS_OK;
}

}  // extern "C"

namespace {

// Everything one soft level needs on the device, from the caller's host tree.
struct SoftLevel {
    int qs = 0, m1 = 0, n1 = 0, o1 = 0, sz1 = 0, len = 0;
    size_t len3 = 0, sz = 0;
    TreeSchedule sch;
    SoftTreeDev tree{};
    float *w6 = nullptr, *w6b = nullptr, *sF = nullptr, *sM = nullptr, *cost = nullptr, *B = nullptr, *M = nullptr, *Mmin = nullptr,
          *logp = nullptr, *disp = nullptr;
    int* sweep = nullptr;  // persistent sweeps: ticket, per-node flags, error word
};

}  // namespace

// One resident forward state: the level as set up, with the arguments it was set
// up with, so that a backward can check it is given the same problem.
struct SoftKept {
    bool used = false, valid = false, prior = false;
    int m = 0, n = 0, o = 0;
    deeds_soft_params p{};
    SoftLevel L;
};

namespace {

// `tag` prefixes the names of the buffers that hold the level's state (tree,
// descriptors, cost volume, messages, marginals, sweep flags); the MIND scratch
// is shared by every level.
deeds_status soft_setup(deeds_ctx* ctx, int m, int n, int o, const deeds_soft_params* p, const int* ordered,
                        const int* parents, const float* edgemst, const float* d_prior, cudaStream_t s,
                        SoftLevel& L, const std::string& tag = "soft_") {
    if (deeds_status e = soft_check(ctx, m, n, o, p, &L.qs)) return e;
    if (!ordered || !parents || !edgemst) return fail(ctx, DEEDS_ERR_INVALID, "null tree array");
    L.m1 = m / p->grid; L.n1 = n / p->grid; L.o1 = o / p->grid;
    L.sz1 = L.m1 * L.n1 * L.o1;
    L.len = 2 * p->radius + 1;
    L.len3 = (size_t)L.len * L.len * L.len;
    L.sz = (size_t)m * n * o;
    for (int t = 0; t < L.sz1; t++)  // the root's parent entry is unused
        if (ordered[t] < 0 || ordered[t] >= L.sz1 ||
            (t > 0 && (parents[ordered[t]] < 0 || parents[ordered[t]] >= L.sz1)))
            return fail(ctx, DEEDS_ERR_INVALID, "tree arrays out of range at %d", t);
    {
        // every parent must precede its children in `ordered` (the sweeps' ticket order)
        std::vector<int> pos(L.sz1, -1);
        for (int t = 0; t < L.sz1; t++) {
            if (pos[ordered[t]] >= 0) return fail(ctx, DEEDS_ERR_INVALID, "ordered repeats node %d", ordered[t]);
            pos[ordered[t]] = t;
        }
        for (int t = 1; t < L.sz1; t++)
            if (pos[parents[ordered[t]]] >= t)
                return fail(ctx, DEEDS_ERR_INVALID, "parent of node %d does not precede it in ordered", ordered[t]);
    }
    build_schedule(ordered, parents, L.sz1, L.sch);
    CK(cudaSetDevice(ctx->device));
    deeds_status st = DEEDS_OK;
    // packed tree: ordered | parents | edgemst | child_ptr | children
    const size_t words = (size_t)L.sz1 * 5 + 2;
    uint32_t* h = hbuf<uint32_t>(ctx, "soft_tree_h", words, &st);
    uint32_t* d = dbuf<uint32_t>(ctx, tag + "tree_d", words, &st);
    L.w6 = dbuf<float>(ctx, "soft_w6", 6 * L.sz, &st);
    L.w6b = dbuf<float>(ctx, "soft_w6b", 6 * L.sz, &st);
    L.sF = dbuf<float>(ctx, tag + "sF", 12 * L.sz, &st);
    L.sM = dbuf<float>(ctx, tag + "sM", 12 * L.sz, &st);
    L.cost = dbuf<float>(ctx, tag + "cost", L.sz1 * L.len3, &st);
    L.B = dbuf<float>(ctx, tag + "B", L.sz1 * L.len3, &st);
    L.M = dbuf<float>(ctx, tag + "M", L.sz1 * L.len3, &st);
    L.Mmin = dbuf<float>(ctx, tag + "Mmin", L.sz1, &st);
    L.logp = dbuf<float>(ctx, tag + "logp", L.sz1 * L.len3, &st);
    L.disp = dbuf<float>(ctx, tag + "disp", 3 * (size_t)L.sz1, &st);
    L.sweep = dbuf<int>(ctx, tag + "sweep", (size_t)L.sz1 + 2, &st);
    if (st) return st;
    CK(cudaMemsetAsync(L.sweep + L.sz1 + 1, 0, sizeof(int), s));
    CK(cudaStreamSynchronize(s));  // the pinned staging block is reused across calls
    const size_t o_par = L.sz1, o_edge = 2 * (size_t)L.sz1, o_cptr = 3 * (size_t)L.sz1,
                 o_ch = 4 * (size_t)L.sz1 + 1;
    std::memcpy(h, ordered, sizeof(int) * L.sz1);
    std::memcpy(h + o_par, parents, sizeof(int) * L.sz1);
    std::memcpy(h + o_edge, edgemst, sizeof(float) * L.sz1);
    std::memcpy(h + o_cptr, L.sch.child_ptr.data(), sizeof(int) * (L.sz1 + 1));
    if (!L.sch.children.empty()) std::memcpy(h + o_ch, L.sch.children.data(), sizeof(int) * L.sch.children.size());
    CK(cudaMemcpyAsync(d, h, words * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    L.tree.len = L.len;
    L.tree.sz = L.sz1;
    L.tree.root = ordered[0];
    L.tree.q = p->quant;
    L.tree.tau = p->tau;
    L.tree.ordered = reinterpret_cast<const int*>(d);
    L.tree.parents = reinterpret_cast<const int*>(d + o_par);
    L.tree.edgemst = reinterpret_cast<const float*>(d + o_edge);
    L.tree.child_ptr = reinterpret_cast<const int*>(d + o_cptr);
    L.tree.children = reinterpret_cast<const int*>(d + o_ch);
    L.tree.off = nullptr;
    L.tree.offbar = nullptr;
    if (d_prior) {
        float* off = dbuf<float>(ctx, tag + "off", 3 * (size_t)L.sz1, &st);
        if (st) return st;
        CK(launch_soft_offsets(d_prior, L.tree.parents, L.tree.root, L.sz1, (float)p->quant, off, s));
        L.tree.off = off;
    }
    return DEEDS_OK;
}

deeds_status soft_run_forward(deeds_ctx* ctx, const float* d_fixed, const float* d_moving, int m, int n, int o,
                              const deeds_soft_params* p, SoftLevel& L, float* d_disp, cudaStream_t s) {
    CK(launch_soft_descriptor(d_fixed, L.w6, L.w6b, L.sF, m, n, o, L.qs, s));
    CK(launch_soft_descriptor(d_moving, L.w6, L.w6b, L.sM, m, n, o, L.qs, s));
    CK(launch_soft_cost(L.sF, L.sM, L.cost, m, n, o, p->grid, p->radius, p->quant, soft_alpha1(p), p->eps, s));
    CK(launch_soft_tree_forward(L.tree, L.sweep, L.cost, L.B, L.M, L.Mmin, L.logp, d_disp, s));
    return DEEDS_OK;
}

// Pinned words a level reads back when its stream is done: the sweeps' error
// word and the alpha dot product.  Pinned, so that the copies stay asynchronous
// and several lanes can be in flight.
struct SoftReadback {
    int* err = nullptr;
    double* dot = nullptr;
};

deeds_status soft_readback(deeds_ctx* ctx, SoftReadback& rb) {
    deeds_status st = DEEDS_OK;
    rb.err = hbuf<int>(ctx, "soft_rb_err", 1, &st);
    rb.dot = hbuf<double>(ctx, "soft_rb_dot", 1, &st);
    return st;
}

deeds_status soft_enqueue_status(deeds_ctx* ctx, const SoftLevel& L, const SoftReadback& rb, cudaStream_t s) {
    CK(cudaMemcpyAsync(rb.err, L.sweep + L.sz1 + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    return DEEDS_OK;
}

// Waits for the stream and reads the sweeps' status.
deeds_status soft_wait(deeds_ctx* ctx, const SoftReadback& rb, cudaStream_t s) {
    CK(cudaStreamSynchronize(s));
    if (*rb.err) return fail(ctx, DEEDS_ERR_TIMEOUT, "a tree sweep gave up waiting for a node's dependencies");
    return DEEDS_OK;
}

// Enqueues the adjoint of one level whose forward state (descriptors, cost
// volume, messages, marginals) is in L, and the read-back of its status and (with
// want_alpha) of the alpha dot product.
deeds_status soft_issue_backward(deeds_ctx* ctx, const float* d_fixed, const float* d_moving, int m, int n, int o,
                                 const deeds_soft_params* p, SoftLevel& L, const float* d_gdisp, float* d_gfixed,
                                 float* d_gmoving, float* d_gprior, bool want_alpha, const SoftReadback& rb,
                                 cudaStream_t s) {
    deeds_status st = DEEDS_OK;
    // the MIND scratch is shared and may have been reallocated since L was set up
    L.w6 = dbuf<float>(ctx, "soft_w6", 6 * L.sz, &st);
    L.w6b = dbuf<float>(ctx, "soft_w6b", 6 * L.sz, &st);
    if (st) return st;
    L.tree.offbar = nullptr;
    if (d_gprior) {
        float* offbar = dbuf<float>(ctx, "soft_offbar", 3 * (size_t)L.sz1, &st);
        if (st) return st;
        CK(cudaMemsetAsync(offbar, 0, sizeof(float) * 3 * L.sz1, s));
        L.tree.offbar = offbar;
    }
    float* R = dbuf<float>(ctx, "soft_R", L.sz1 * L.len3, &st);
    float* Bbar = dbuf<float>(ctx, "soft_Bbar", L.sz1 * L.len3, &st);
    float* sFbar = dbuf<float>(ctx, "soft_sFbar", 12 * L.sz, &st);
    float* sMbar = dbuf<float>(ctx, "soft_sMbar", 12 * L.sz, &st);
    float* dbar6 = dbuf<float>(ctx, "soft_dbar6", 6 * L.sz, &st);
    double* dot = dbuf<double>(ctx, "soft_dot", 1, &st);
    if (st) return st;
    CK(launch_soft_tree_backward(L.tree, L.sweep, L.B, L.M, L.logp, d_gdisp, R, Bbar, s));
    if (d_gprior) {
        CK(cudaMemsetAsync(d_gprior, 0, sizeof(float) * 3 * L.sz1, s));
        CK(launch_soft_offbar_to_prior(L.tree.offbar, L.tree.parents, L.tree.root, L.sz1, (float)p->quant, d_gprior,
                                       s));
    }
    // Bbar is now dL/dcost
    CK(launch_soft_cost_adj(L.sF, L.sM, Bbar, L.cost, sFbar, sMbar, dot, m, n, o, p->grid, p->radius, p->quant,
                            soft_alpha1(p), p->eps, s));
    if (d_gfixed) {
        CK(cudaMemsetAsync(d_gfixed, 0, sizeof(float) * L.sz, s));
        CK(launch_soft_descriptor_adj(d_fixed, L.w6, L.w6b, sFbar, dbar6, d_gfixed, m, n, o, L.qs, s));
    }
    if (d_gmoving) {
        CK(cudaMemsetAsync(d_gmoving, 0, sizeof(float) * L.sz, s));
        CK(launch_soft_descriptor_adj(d_moving, L.w6, L.w6b, sMbar, dbar6, d_gmoving, m, n, o, L.qs, s));
    }
    if (want_alpha) CK(cudaMemcpyAsync(rb.dot, dot, sizeof(double), cudaMemcpyDeviceToHost, s));
    return soft_enqueue_status(ctx, L, rb, s);
}

float soft_grad_alpha(const SoftReadback& rb, const deeds_soft_params* p) {
    return (float)(-*rb.dot / (double)p->alpha);
}

// The first free kept slot of ctx (appended when none is free), marked in use.
SoftKept& soft_acquire_slot(deeds_ctx* ctx, int* slot) {
    int k = 0;
    while (k < (int)ctx->kept.size() && ctx->kept[k]->used) k++;
    if (k == (int)ctx->kept.size()) ctx->kept.push_back(std::make_shared<SoftKept>());
    SoftKept& K = *ctx->kept[k];
    K.used = true;
    K.valid = false;
    *slot = k;
    return K;
}

std::string soft_slot_tag(int k) { return "softk" + std::to_string(k) + "_"; }

void soft_fill_slot(SoftKept& K, int m, int n, int o, const deeds_soft_params* p, bool prior) {
    K.m = m; K.n = n; K.o = o;
    K.p = *p;
    K.prior = prior;
    K.valid = true;
}

// The kept state of `slot` if it was filled for exactly this problem, else NULL
// with the context's error set.
SoftKept* soft_kept_for(deeds_ctx* ctx, int slot, int m, int n, int o, const deeds_soft_params* p, bool prior) {
    if (slot < 0 || slot >= (int)ctx->kept.size() || !ctx->kept[slot]->used || !ctx->kept[slot]->valid) {
        fail(ctx, DEEDS_ERR_INVALID, "slot %d holds no forward state", slot);
        return nullptr;
    }
    SoftKept& K = *ctx->kept[slot];
    const bool same = K.m == m && K.n == n && K.o == o && K.p.grid == p->grid && K.p.radius == p->radius &&
                      K.p.quant == p->quant && K.p.mind_radius == p->mind_radius && K.p.alpha == p->alpha &&
                      K.p.tau == p->tau && K.p.eps == p->eps && K.prior == prior;
    if (!same) {
        fail(ctx, DEEDS_ERR_INVALID, "slot %d was filled for another level or parameters", slot);
        return nullptr;
    }
    return &K;
}

// Pairs of a batch run in waves of at most this many lanes (child contexts with
// their own streams and buffers); pair i of a wave runs on lane i.
constexpr int kSoftMaxLanes = 8;

deeds_status soft_lanes(deeds_ctx* ctx, int want) {
    while ((int)ctx->lanes.size() < want) {
        deeds_ctx* lane = nullptr;
        deeds_status st = deeds_create(&lane, ctx->device);
        if (st) return fail(ctx, st, "batch lane: %s", deeds_last_error(nullptr));
        lane->tune = ctx->tune;
        ctx->lanes.push_back(lane);
    }
    return DEEDS_OK;
}

deeds_status lane_fail(deeds_ctx* ctx, deeds_ctx* lane, deeds_status st, int pair) {
    return fail(ctx, st, "pair %d: %s", pair, lane->err.c_str());
}

}  // namespace

extern "C" {

deeds_status deeds_soft_forward_dev(deeds_ctx* ctx, const float* d_fixed, const float* d_moving, int m, int n, int o,
                                    const deeds_soft_params* p, const int* ordered, const int* parents,
                                    const float* edgemst, const float* d_prior, float* d_disp, void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_fixed || !d_moving || !d_disp) return fail(ctx, DEEDS_ERR_INVALID, "null pointer");
    cudaStream_t s = (cudaStream_t)stream;
    SoftLevel L;
    SoftReadback rb;
    if (deeds_status e = soft_readback(ctx, rb)) return e;
    if (deeds_status e = soft_setup(ctx, m, n, o, p, ordered, parents, edgemst, d_prior, s, L)) return e;
    if (deeds_status e = soft_run_forward(ctx, d_fixed, d_moving, m, n, o, p, L, d_disp, s)) return e;
    if (deeds_status e = soft_enqueue_status(ctx, L, rb, s)) return e;
    return soft_wait(ctx, rb, s);
}

deeds_status deeds_soft_backward_dev(deeds_ctx* ctx, const float* d_fixed, const float* d_moving, int m, int n, int o,
                                     const deeds_soft_params* p, const int* ordered, const int* parents,
                                     const float* edgemst, const float* d_prior, const float* d_gdisp,
                                     float* d_gfixed, float* d_gmoving, float* d_gprior, float* grad_alpha,
                                     void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_fixed || !d_moving || !d_gdisp) return fail(ctx, DEEDS_ERR_INVALID, "null pointer");
    if (d_gprior && !d_prior) return fail(ctx, DEEDS_ERR_INVALID, "grad_prior needs a prior field");
    cudaStream_t s = (cudaStream_t)stream;
    SoftLevel L;
    SoftReadback rb;
    if (deeds_status e = soft_readback(ctx, rb)) return e;
    if (deeds_status e = soft_setup(ctx, m, n, o, p, ordered, parents, edgemst, d_prior, s, L)) return e;
    // recompute the forward state (descriptors, cost, messages, marginals)
    if (deeds_status e = soft_run_forward(ctx, d_fixed, d_moving, m, n, o, p, L, L.disp, s)) return e;
    if (deeds_status e = soft_issue_backward(ctx, d_fixed, d_moving, m, n, o, p, L, d_gdisp, d_gfixed, d_gmoving,
                                             d_gprior, grad_alpha != nullptr, rb, s))
        return e;
    if (deeds_status e = soft_wait(ctx, rb, s)) return e;
    if (grad_alpha) *grad_alpha = soft_grad_alpha(rb, p);
    return DEEDS_OK;
}

deeds_status deeds_soft_forward_keep_dev(deeds_ctx* ctx, const float* d_fixed, const float* d_moving, int m, int n,
                                         int o, const deeds_soft_params* p, const int* ordered, const int* parents,
                                         const float* edgemst, const float* d_prior, float* d_disp, int* slot,
                                         void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_fixed || !d_moving || !d_disp || !slot || !p) return fail(ctx, DEEDS_ERR_INVALID, "null pointer");
    cudaStream_t s = (cudaStream_t)stream;
    SoftReadback rb;
    if (deeds_status e = soft_readback(ctx, rb)) return e;
    int k = -1;
    SoftKept& K = soft_acquire_slot(ctx, &k);
    deeds_status e = soft_setup(ctx, m, n, o, p, ordered, parents, edgemst, d_prior, s, K.L, soft_slot_tag(k));
    if (!e) e = soft_run_forward(ctx, d_fixed, d_moving, m, n, o, p, K.L, d_disp, s);
    if (!e) e = soft_enqueue_status(ctx, K.L, rb, s);
    if (!e) e = soft_wait(ctx, rb, s);
    if (e) {
        K.used = false;  // nothing is kept
        return e;
    }
    soft_fill_slot(K, m, n, o, p, d_prior != nullptr);
    *slot = k;
    return DEEDS_OK;
}

deeds_status deeds_soft_backward_kept_dev(deeds_ctx* ctx, int slot, const float* d_fixed, const float* d_moving,
                                          int m, int n, int o, const deeds_soft_params* p, const float* d_prior,
                                          const float* d_gdisp, float* d_gfixed, float* d_gmoving, float* d_gprior,
                                          float* grad_alpha, void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_fixed || !d_moving || !d_gdisp || !p) return fail(ctx, DEEDS_ERR_INVALID, "null pointer");
    if (d_gprior && !d_prior) return fail(ctx, DEEDS_ERR_INVALID, "grad_prior needs a prior field");
    SoftKept* K = soft_kept_for(ctx, slot, m, n, o, p, d_prior != nullptr);
    if (!K) return DEEDS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    SoftReadback rb;
    if (deeds_status e = soft_readback(ctx, rb)) return e;
    if (deeds_status e = soft_issue_backward(ctx, d_fixed, d_moving, m, n, o, p, K->L, d_gdisp, d_gfixed, d_gmoving,
                                             d_gprior, grad_alpha != nullptr, rb, s))
        return e;
    if (deeds_status e = soft_wait(ctx, rb, s)) return e;
    if (grad_alpha) *grad_alpha = soft_grad_alpha(rb, p);
    return DEEDS_OK;
}

deeds_status deeds_soft_release(deeds_ctx* ctx, int slot) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (slot < 0 || slot >= (int)ctx->kept.size() || !ctx->kept[slot]->used)
        return fail(ctx, DEEDS_ERR_INVALID, "slot %d is not in use", slot);
    ctx->kept[slot]->used = false;
    ctx->kept[slot]->valid = false;
    return DEEDS_OK;
}

static deeds_status soft_trim_one(deeds_ctx* ctx) {
    CK(cudaSetDevice(ctx->device));
    for (size_t k = 0; k < ctx->kept.size(); k++) {
        if (ctx->kept[k]->used) continue;
        const std::string tag = soft_slot_tag((int)k);
        for (auto it = ctx->dev.lower_bound(tag); it != ctx->dev.end() && it->first.compare(0, tag.size(), tag) == 0;) {
            if (it->second.p) CK(cudaFree(it->second.p));
            it = ctx->dev.erase(it);
        }
    }
    return DEEDS_OK;
}

deeds_status deeds_soft_trim(deeds_ctx* ctx) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (deeds_status e = soft_trim_one(ctx)) return e;
    for (deeds_ctx* lane : ctx->lanes)
        if (deeds_status e = soft_trim_one(lane)) return fail(ctx, e, "lane: %s", lane->err.c_str());
    return DEEDS_OK;
}

deeds_status deeds_soft_forward_batch_dev(deeds_ctx* ctx, int npairs, const float* const* d_fixed,
                                          const float* const* d_moving, int m, int n, int o,
                                          const deeds_soft_params* p, const int* const* ordered,
                                          const int* const* parents, const float* const* edgemst,
                                          const float* const* d_prior, float* const* d_disp, int* slots,
                                          void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (npairs < 0) return fail(ctx, DEEDS_ERR_INVALID, "npairs < 0");
    if (npairs == 0) return DEEDS_OK;
    if (!d_fixed || !d_moving || !p || !ordered || !parents || !edgemst || !d_disp)
        return fail(ctx, DEEDS_ERR_INVALID, "null array");
    for (int i = 0; i < npairs; i++) {
        if (!d_fixed[i] || !d_moving[i] || !d_disp[i]) return fail(ctx, DEEDS_ERR_INVALID, "pair %d: null pointer", i);
        if (d_prior && !d_prior[i]) return fail(ctx, DEEDS_ERR_INVALID, "pair %d: null prior", i);
    }
    int qs = 0;
    if (deeds_status e = soft_check(ctx, m, n, o, p, &qs)) return e;
    const int nl = std::min(npairs, kSoftMaxLanes);
    if (deeds_status e = soft_lanes(ctx, nl)) return e;
    cudaStream_t s = (cudaStream_t)stream;
    CK(cudaSetDevice(ctx->device));
    CK(cudaEventRecord(ctx->ev_a, s));  // inputs written on the caller's stream
    if (slots)
        for (int i = 0; i < npairs; i++) slots[i] = -1;
    for (int w0 = 0; w0 < npairs; w0 += nl) {
        const int w1 = std::min(npairs, w0 + nl);
        std::vector<SoftLevel> local(w1 - w0);
        std::vector<SoftLevel*> lv(w1 - w0);
        std::vector<SoftReadback> rb(w1 - w0);
        deeds_status err = DEEDS_OK;
        int bad = -1;
        for (int i = w0; i < w1 && !err; i++) {
            deeds_ctx* lane = ctx->lanes[i - w0];
            cudaStream_t ls = lane->stream;
            std::string tag = "soft_";
            if (slots) {
                SoftKept& K = soft_acquire_slot(lane, &slots[i]);
                lv[i - w0] = &K.L;
                tag = soft_slot_tag(slots[i]);
            } else {
                lv[i - w0] = &local[i - w0];
            }
            SoftLevel& L = *lv[i - w0];
            bad = i;
            if (cudaStreamWaitEvent(ls, ctx->ev_a, 0) != cudaSuccess) err = fail(lane, DEEDS_ERR_CUDA, "event wait");
            if (!err) err = soft_readback(lane, rb[i - w0]);
            if (!err)
                err = soft_setup(lane, m, n, o, p, ordered[i], parents[i], edgemst[i], d_prior ? d_prior[i] : nullptr,
                                 ls, L, tag);
            if (!err) err = soft_run_forward(lane, d_fixed[i], d_moving[i], m, n, o, p, L, d_disp[i], ls);
            if (!err) err = soft_enqueue_status(lane, L, rb[i - w0], ls);
        }
        for (int i = w0; i < w1; i++) {  // every issued lane finishes before returning
            deeds_ctx* lane = ctx->lanes[i - w0];
            if (!rb[i - w0].err) continue;
            deeds_status e = soft_wait(lane, rb[i - w0], lane->stream);
            if (e && !err) { err = e; bad = i; }
        }
        if (err) {
            if (slots)
                for (int i = 0; i < w1; i++)
                    if (slots[i] >= 0) {
                        ctx->lanes[i % nl]->kept[slots[i]]->used = false;
                        slots[i] = -1;
                    }
            return lane_fail(ctx, ctx->lanes[bad - w0], err, bad);
        }
        if (slots)
            for (int i = w0; i < w1; i++)
                soft_fill_slot(*ctx->lanes[i - w0]->kept[slots[i]], m, n, o, p, d_prior != nullptr);
    }
    return DEEDS_OK;
}

deeds_status deeds_soft_backward_batch_dev(deeds_ctx* ctx, int npairs, const int* slots,
                                           const float* const* d_fixed, const float* const* d_moving, int m, int n,
                                           int o, const deeds_soft_params* p, const int* const* ordered,
                                           const int* const* parents, const float* const* edgemst,
                                           const float* const* d_prior, const float* const* d_gdisp,
                                           float* const* d_gfixed, float* const* d_gmoving, float* const* d_gprior,
                                           float* grad_alpha, void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (npairs < 0) return fail(ctx, DEEDS_ERR_INVALID, "npairs < 0");
    if (npairs == 0) return DEEDS_OK;
    if (!d_fixed || !d_moving || !p || !d_gdisp) return fail(ctx, DEEDS_ERR_INVALID, "null array");
    if (!slots && (!ordered || !parents || !edgemst))
        return fail(ctx, DEEDS_ERR_INVALID, "the recomputing backward needs the trees");
    if (d_gprior && !d_prior) return fail(ctx, DEEDS_ERR_INVALID, "grad_prior needs a prior field");
    for (int i = 0; i < npairs; i++) {
        if (!d_fixed[i] || !d_moving[i] || !d_gdisp[i]) return fail(ctx, DEEDS_ERR_INVALID, "pair %d: null pointer", i);
        if (d_prior && !d_prior[i]) return fail(ctx, DEEDS_ERR_INVALID, "pair %d: null prior", i);
    }
    int qs = 0;
    if (deeds_status e = soft_check(ctx, m, n, o, p, &qs)) return e;
    const int nl = std::min(npairs, kSoftMaxLanes);
    if (deeds_status e = soft_lanes(ctx, nl)) return e;
    std::vector<SoftKept*> kept(npairs, nullptr);
    if (slots)
        for (int i = 0; i < npairs; i++) {
            deeds_ctx* lane = ctx->lanes[i % nl];
            kept[i] = soft_kept_for(lane, slots[i], m, n, o, p, d_prior != nullptr);
            if (!kept[i]) return lane_fail(ctx, lane, DEEDS_ERR_INVALID, i);
        }
    cudaStream_t s = (cudaStream_t)stream;
    CK(cudaSetDevice(ctx->device));
    CK(cudaEventRecord(ctx->ev_a, s));
    for (int w0 = 0; w0 < npairs; w0 += nl) {
        const int w1 = std::min(npairs, w0 + nl);
        std::vector<SoftLevel> local(w1 - w0);
        std::vector<SoftReadback> rb(w1 - w0);
        deeds_status err = DEEDS_OK;
        int bad = -1;
        for (int i = w0; i < w1 && !err; i++) {
            deeds_ctx* lane = ctx->lanes[i - w0];
            cudaStream_t ls = lane->stream;
            const float* prior = d_prior ? d_prior[i] : nullptr;
            SoftLevel& L = slots ? kept[i]->L : local[i - w0];
            bad = i;
            if (cudaStreamWaitEvent(ls, ctx->ev_a, 0) != cudaSuccess) err = fail(lane, DEEDS_ERR_CUDA, "event wait");
            if (!err) err = soft_readback(lane, rb[i - w0]);
            if (!err && !slots) {
                err = soft_setup(lane, m, n, o, p, ordered[i], parents[i], edgemst[i], prior, ls, L);
                if (!err) err = soft_run_forward(lane, d_fixed[i], d_moving[i], m, n, o, p, L, L.disp, ls);
            }
            if (!err)
                err = soft_issue_backward(lane, d_fixed[i], d_moving[i], m, n, o, p, L, d_gdisp[i],
                                          d_gfixed ? d_gfixed[i] : nullptr, d_gmoving ? d_gmoving[i] : nullptr,
                                          d_gprior ? d_gprior[i] : nullptr, grad_alpha != nullptr, rb[i - w0], ls);
        }
        for (int i = w0; i < w1; i++) {
            deeds_ctx* lane = ctx->lanes[i - w0];
            if (!rb[i - w0].err) continue;
            deeds_status e = soft_wait(lane, rb[i - w0], lane->stream);
            if (e && !err) { err = e; bad = i; }
            if (!e && !err && grad_alpha) grad_alpha[i] = soft_grad_alpha(rb[i - w0], p);
        }
        if (err) return lane_fail(ctx, ctx->lanes[bad - w0], err, bad);
    }
    return DEEDS_OK;
}

deeds_status deeds_soft_release_batch(deeds_ctx* ctx, int npairs, const int* slots) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (npairs < 0 || (npairs > 0 && !slots)) return fail(ctx, DEEDS_ERR_INVALID, "bad slot list");
    const int nl = std::min(npairs, kSoftMaxLanes);
    for (int i = 0; i < npairs; i++) {
        if (i % nl >= (int)ctx->lanes.size()) return fail(ctx, DEEDS_ERR_INVALID, "pair %d: no lane", i);
        if (deeds_status e = deeds_soft_release(ctx->lanes[i % nl], slots[i])) return lane_fail(ctx, ctx->lanes[i % nl], e, i);
    }
    return DEEDS_OK;
}

deeds_status deeds_soft_upsample_dev(deeds_ctx* ctx, const float* d_in, int mA, int nA, int oA, float* d_out, int m,
                                     int n, int o, void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_in || !d_out || mA < 1 || nA < 1 || oA < 1 || m < 1 || n < 1 || o < 1 || n > 65535 || o > 65535)
        return fail(ctx, DEEDS_ERR_INVALID, "deeds_soft_upsample_dev: bad arguments");
    CK(cudaSetDevice(ctx->device));
    CK(launch_soft_upsample(d_in, mA, nA, oA, d_out, m, n, o, (cudaStream_t)stream));
    return DEEDS_OK;
}

deeds_status deeds_soft_upsample_backward_dev(deeds_ctx* ctx, const float* d_gout, int m, int n, int o, float* d_gin,
                                              int mA, int nA, int oA, void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_gout || !d_gin || mA < 1 || nA < 1 || oA < 1 || m < 1 || n < 1 || o < 1)
        return fail(ctx, DEEDS_ERR_INVALID, "deeds_soft_upsample_backward_dev: bad arguments");
    CK(cudaSetDevice(ctx->device));
    CK(launch_soft_upsample_adj(d_gout, m, n, o, d_gin, mA, nA, oA, (cudaStream_t)stream));
    return DEEDS_OK;
}

deeds_status deeds_soft_warp_dev(deeds_ctx* ctx, const float* d_moving, int m, int n, int o, const float* d_grid,
                                 int mA, int nA, int oA, float* d_out, void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_moving || !d_grid || !d_out || mA < 1 || nA < 1 || oA < 1 || m < 1 || n < 1 || o < 1 || n > 65535 ||
        o > 65535)
        return fail(ctx, DEEDS_ERR_INVALID, "deeds_soft_warp_dev: bad arguments");
    CK(cudaSetDevice(ctx->device));
    CK(launch_soft_warp(d_moving, d_grid, mA, nA, oA, d_out, m, n, o, (cudaStream_t)stream));
    return DEEDS_OK;
}

deeds_status deeds_soft_warp_backward_dev(deeds_ctx* ctx, const float* d_moving, int m, int n, int o,
                                          const float* d_grid, int mA, int nA, int oA, const float* d_gout,
                                          float* d_gmoving, float* d_ggrid, void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_moving || !d_grid || !d_gout || mA < 1 || nA < 1 || oA < 1 || m < 1 || n < 1 || o < 1 || n > 65535 ||
        o > 65535)
        return fail(ctx, DEEDS_ERR_INVALID, "deeds_soft_warp_backward_dev: bad arguments");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = (cudaStream_t)stream;
    const size_t sz = (size_t)m * n * o;
    deeds_status st = DEEDS_OK;
    float* gfull = d_ggrid ? dbuf<float>(ctx, "soft_gfull", 3 * sz, &st) : nullptr;
    if (st) return st;
    if (d_gmoving) CK(cudaMemsetAsync(d_gmoving, 0, sizeof(float) * sz, s));
    CK(launch_soft_warp_adj(d_moving, d_grid, mA, nA, oA, d_gout, d_gmoving, gfull, m, n, o, s));
    if (d_ggrid) CK(launch_soft_upsample_adj(gfull, m, n, o, d_ggrid, mA, nA, oA, s));
    return DEEDS_OK;
}

// ---------------------------------------------------------------------------
// linearBCV (src/linearBCV.cpp:163-262)

void deeds_linear_default_params(deeds_linear_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    const int G[4] = {7, 6, 5, 4}, L[4] = {5, 4, 3, 2}, Q[4] = {4, 3, 2, 1};  // src/linearBCV.cpp:86-89
    p->levels = 4;
    for (int l = 0; l < 4; l++) { p->grid[l] = G[l]; p->radius[l] = L[l]; p->quant[l] = Q[l]; }
    p->rigid = 0;
    p->intensity_shift = 1024.0f;
    p->verbose = 0;
}

}  // extern "C"

namespace {

deeds_status check_linear_params(deeds_ctx* ctx, const deeds_linear_params* p, int m, int n, int o) {
    if (!p) return fail(ctx, DEEDS_ERR_INVALID, "params is NULL");
    deeds_params d;
    deeds_default_params(&d);
    d.levels = p->levels;
    if (p->levels < 1 || p->levels > DEEDS_MAX_LEVELS)
        return fail(ctx, DEEDS_ERR_INVALID, "levels=%d outside 1..%d", p->levels, DEEDS_MAX_LEVELS);
    for (int l = 0; l < p->levels; l++) {
        d.grid[l] = p->grid[l]; d.radius[l] = p->radius[l]; d.quant[l] = p->quant[l];
        // estimateAffine2 needs interior nodes (two from each border) to fit anything
        const int g = p->grid[l];
        if (g >= 1 && (m / g < 5 || n / g < 5 || o / g < 5))
            return fail(ctx, DEEDS_ERR_INVALID, "level %d: grid %d leaves fewer than 5 control points on an axis", l, g);
    }
    return check_params(ctx, &d, m, n, o);
}

// One linearBCV level after the cost volumes: smoothing, node statistics (GPU),
// then the fit on the host.  Returns the number of points used.
deeds_status linear_estimate(deeds_ctx* ctx, const float* fix, const float* mov, float* cost0, float* cost1, int m,
                             int n, int o, int g, int hw, int q, bool rigid, const float Xprev[16], float X[16],
                             int* used, int* allcount, float* quantile, cudaStream_t s, cudaStream_t s2) {
    const int m1 = m / g, n1 = n / g, o1 = o / g, sz1 = m1 * n1 * o1;
    const int len = 2 * hw + 1, len3 = len * len * len;
    deeds_status st = DEEDS_OK;
    float* d_minval = dbuf<float>(ctx, "lin_minval", 2 * (size_t)sz1, &st);
    int* d_minind = dbuf<int>(ctx, "lin_minind", 2 * (size_t)sz1, &st);
    float* h_minval = hbuf<float>(ctx, "lin_h_minval", 2 * (size_t)sz1, &st);
    int* h_minind = hbuf<int>(ctx, "lin_h_minind", 2 * (size_t)sz1, &st);
    if (st) return st;
    if (s2 && s2 != s) {
        // each volume smoothed on the stream that built it, then joined
        CK(launch_lin_smooth(cost1, nullptr, m1, n1, o1, len3, s2));
        CK(cudaEventRecord(ctx->ev_d, s2));
        CK(launch_lin_smooth(cost0, nullptr, m1, n1, o1, len3, s));
        CK(cudaStreamWaitEvent(s, ctx->ev_d, 0));
    } else {
        CK(launch_lin_smooth(cost0, cost1, m1, n1, o1, len3, s));
    }
    CK(launch_lin_node_stats(cost0, cost1, fix, mov, m, n, o, g, len3, d_minval, d_minind, s));
    CK(cudaMemcpyAsync(h_minval, d_minval, 2 * (size_t)sz1 * sizeof(float), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(h_minind, d_minind, 2 * (size_t)sz1 * sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    int ac = 0;
    float qf = 0.0f;
    const int u = lin_estimate_from_stats(X, Xprev, h_minval, h_minind, m1, n1, o1, g, (float)q, hw, rigid, &ac, &qf);
    if (u < kMinFitPoints)
        return fail(ctx, DEEDS_ERR_INVALID,
                    "grid %d: %d of %d control-point votes fall below the selection quantile (at least %d needed)", g,
                    u, ac, kMinFitPoints);
    if (used) *used = u;
    if (allcount) *allcount = ac;
    if (quantile) *quantile = qf;
    return DEEDS_OK;
}

}  // namespace

extern "C" {

deeds_status deeds_lin_warp_dev(const float* d_in, const float X[16], int m, int n, int o, float* d_out, void* stream) {
    deeds_ctx* ctx = nullptr;
    if (!d_in || !X || !d_out || m < 1 || n < 1 || o < 1 || n > 65535 || o > 65535)
        return fail(nullptr, DEEDS_ERR_INVALID, "deeds_lin_warp_dev: bad arguments");
    CK(launch_lin_warp(d_in, X, m, n, o, d_out, (cudaStream_t)stream));
    return DEEDS_OK;
}

deeds_status deeds_lin_smooth_dev(float* d_cost, int m1, int n1, int o1, int len3, void* stream) {
    deeds_ctx* ctx = nullptr;
    if (!d_cost || m1 < 1 || n1 < 1 || o1 < 1 || len3 < 1)
        return fail(nullptr, DEEDS_ERR_INVALID, "deeds_lin_smooth_dev: bad arguments");
    CK(launch_lin_smooth(d_cost, nullptr, m1, n1, o1, len3, (cudaStream_t)stream));
    return DEEDS_OK;
}

deeds_status deeds_estimate_affine_dev(deeds_ctx* ctx, const float* d_fixed, const float* d_moving, float* d_cost,
                                       float* d_cost2, int m, int n, int o, int g, int hw, int q, int rigid,
                                       const float Xprev[16], float X[16], int* points_used, void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_fixed || !d_moving || !d_cost || !d_cost2 || !Xprev || !X) return fail(ctx, DEEDS_ERR_INVALID, "null pointer");
    if (m < 1 || n < 1 || o < 1 || g < 1 || hw < 0 || q < 1 || m / g < 1 || n / g < 1 || o / g < 1)
        return fail(ctx, DEEDS_ERR_INVALID, "bad dims or level parameters");
    CK(cudaSetDevice(ctx->device));
    return linear_estimate(ctx, d_fixed, d_moving, d_cost, d_cost2, m, n, o, g, hw, q, rigid != 0, Xprev, X,
                           points_used, nullptr, nullptr, (cudaStream_t)stream, nullptr);
}

deeds_status deeds_affine_robust(const float* pts1, const float* pts2, int len, int rigid, float RT[16]) {
    deeds_ctx* ctx = nullptr;
    if (!pts1 || !pts2 || !RT || len < kMinFitPoints)
        return fail(ctx, DEEDS_ERR_INVALID, "deeds_affine_robust: bad arguments (len %d, at least %d)", len, kMinFitPoints);
    lin_affine_robust(RT, pts1, pts2, len, rigid != 0);
    return DEEDS_OK;
}

deeds_status deeds_linear_register_dev(deeds_ctx* ctx, const float* d_fixed, const float* d_moving, int m, int n,
                                       int o, const deeds_linear_params* P, float X_out[16], void* stream) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!d_fixed || !d_moving || !X_out) return fail(ctx, DEEDS_ERR_INVALID, "null pointer");
    deeds_status st = check_linear_params(ctx, P, m, n, o);
    if (st) return st;
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = (cudaStream_t)stream, sb = ctx->stream_b;
    const size_t sz = (size_t)m * n * o;
    size_t max_cost = 0, max_pad = 0;
    for (int l = 0; l < P->levels; l++) {
        const int g = P->grid[l], len = 2 * P->radius[l] + 1;
        max_cost = std::max(max_cost, (size_t)(m / g) * (n / g) * (o / g) * len * len * len);
        max_pad = std::max(max_pad, padded_codes_count(m, n, o, P->quant[l] * P->radius[l]));
    }
    float* fix = dbuf<float>(ctx, "lin_fix", sz, &st);
    float* mov = dbuf<float>(ctx, "lin_mov", sz, &st);
    float* warped[2] = {dbuf<float>(ctx, "lin_w1", sz, &st), dbuf<float>(ctx, "lin_w2", sz, &st)};
    uint64_t* c_fix = dbuf<uint64_t>(ctx, "lin_c_fix", sz, &st);
    uint64_t* c_mov = dbuf<uint64_t>(ctx, "lin_c_mov", sz, &st);
    uint64_t* c_warp[2] = {dbuf<uint64_t>(ctx, "lin_c_w1", sz, &st), dbuf<uint64_t>(ctx, "lin_c_w2", sz, &st)};
    float* scr[2] = {dbuf<float>(ctx, "lin_mind1", 6 * sz, &st), dbuf<float>(ctx, "lin_mind2", 6 * sz, &st)};
    float* cost[2] = {dbuf<float>(ctx, "lin_cost1", max_cost, &st), dbuf<float>(ctx, "lin_cost2", max_cost, &st)};
    uint64_t* mpad[2] = {dbuf<uint64_t>(ctx, "lin_mpad1", max_pad, &st), dbuf<uint64_t>(ctx, "lin_mpad2", max_pad, &st)};
    int* d_err = dbuf<int>(ctx, "lin_err", 2, &st);
    if (st) return st;
    float thr[5];
    mind_thresholds(thr);
    CK(cudaMemsetAsync(d_err, 0, 2 * sizeof(int), s));
    CK(launch_shift(d_fixed, fix, (int64_t)sz, P->intensity_shift, s));
    CK(launch_shift(d_moving, mov, (int64_t)sz, P->intensity_shift, s));
    float Xprev[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    const float ident[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    float X[16];
    std::memcpy(X, Xprev, sizeof(X));
    int prev_step = -1;
    for (int l = 0; l < P->levels; l++) {
        const int g = P->grid[l], hw = P->radius[l], q = P->quant[l];
        const int qs = mind_step(q);
        float Xinv[16];
        lin_qrsolve(Xinv, Xprev, ident, 4, 4);  // src/linearBCV.cpp:186-187
        if (l == 0 || qs != prev_step) {
            StageScope sc(ctx, DEEDS_STAGE_MIND, s);
            CK(launch_mind_ssc(mov, m, n, o, qs, thr, scr[0], c_mov, s));
            CK(launch_mind_ssc(fix, m, n, o, qs, thr, scr[0], c_fix, s));
        }
        prev_step = qs;
        CK(cudaEventRecord(ctx->ev_d, s));
        CK(cudaStreamWaitEvent(sb, ctx->ev_d, 0));
        // direction 1: fixed codes against the moving image warped by X; direction 2:
        // moving codes against the fixed image warped by the inverse
        for (int d = 0; d < 2; d++) {
            cudaStream_t sd = d == 0 ? s : sb;
            {
                StageScope sc(ctx, DEEDS_STAGE_TRANSFORM, sd);
                CK(launch_lin_warp(d == 0 ? mov : fix, d == 0 ? Xprev : Xinv, m, n, o, warped[d], sd));
            }
            {
                StageScope sc(ctx, DEEDS_STAGE_MIND, sd);
                CK(launch_mind_ssc(warped[d], m, n, o, qs, thr, scr[d], c_warp[d], sd));
            }
            {
                StageScope sc(ctx, DEEDS_STAGE_DATACOST, sd);
                CK(data_cost_auto(ctx, d == 0 ? c_fix : c_mov, c_warp[d], mpad[d], m, n, o, g, hw, q, 1.0f, cost[d],
                                  d_err + d, sd));
            }
        }
        int used = 0, allcount = 0;
        float quant = 0.0f;
        st = linear_estimate(ctx, fix, mov, cost[0], cost[1], m, n, o, g, hw, q, P->rigid != 0, Xprev, X, &used,
                             &allcount, &quant, s, sb);
        if (st) return st;
        if (P->verbose) printf("# points used: %d/%d, quantile: %f\n", used, allcount, quant);
        std::memcpy(Xprev, X, sizeof(X));
    }
    int herr[2] = {0, 0};
    CK(cudaMemcpyAsync(herr, d_err, sizeof(herr), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (ctx->prof) collect_marks(ctx);
    if (herr[0] == 3 || herr[1] == 3) return fail(ctx, DEEDS_ERR_TIMEOUT, "cost volume: a bounded wait for a TMA copy expired");
    if (herr[0] || herr[1]) return fail(ctx, DEEDS_ERR_INTERNAL, "cost volume kernel reported error %d", herr[0] | herr[1]);
    std::memcpy(X_out, X, sizeof(X));
    return DEEDS_OK;
}

deeds_status deeds_affine_warp_segmentation(deeds_ctx* ctx, const int16_t* seg, int m, int n, int o, const float X[16],
                                           int16_t* seg_out) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!seg || !seg_out || !X || m < 1 || n < 1 || o < 1 || n > 65535 || o > 65535)
        return fail(ctx, DEEDS_ERR_INVALID, "deeds_affine_warp_segmentation: bad arguments");
    CK(cudaSetDevice(ctx->device));
    const size_t sz = (size_t)m * n * o;
    deeds_status st = DEEDS_OK;
    short* d_in = dbuf<short>(ctx, "seg_in", sz, &st);
    short* d_out = dbuf<short>(ctx, "seg_out", sz, &st);
    if (st) return st;
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(d_in, seg, sz * sizeof(short), cudaMemcpyHostToDevice, s));
    FieldRef zero{0, nullptr, nullptr, nullptr, 0, 0, 0};
    CK(launch_warp_seg(d_in, X, zero, m, n, o, d_out, s));
    CK(cudaMemcpyAsync(seg_out, d_out, sz * sizeof(short), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return DEEDS_OK;
}

deeds_status deeds_linear_register(deeds_ctx* ctx, const float* fixed, const float* moving, int m, int n, int o,
                                   const deeds_linear_params* params, float X_out[16]) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    if (!fixed || !moving || !X_out) return fail(ctx, DEEDS_ERR_INVALID, "null pointer");
    deeds_status st = check_linear_params(ctx, params, m, n, o);
    if (st) return st;
    CK(cudaSetDevice(ctx->device));
    const size_t sz = (size_t)m * n * o;
    float* d_f = dbuf<float>(ctx, "in_fixed", sz, &st);
    float* d_m = dbuf<float>(ctx, "in_moving", sz, &st);
    if (st) return st;
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(d_f, fixed, sz * sizeof(float), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_m, moving, sz * sizeof(float), cudaMemcpyHostToDevice, s));
    return deeds_linear_register_dev(ctx, d_f, d_m, m, n, o, params, X_out, s);
}

deeds_status deeds_selftest_bounded_waits(deeds_ctx* ctx, int* sweep_gave_up, int* tma_gave_up, double* seconds) {
    if (!ctx) return fail(nullptr, DEEDS_ERR_INVALID, "ctx is NULL");
    CK(cudaSetDevice(ctx->device));
    deeds_status st = DEEDS_OK;
    int* d = dbuf<int>(ctx, "selftest", 4, &st);
    if (st) return st;
    cudaStream_t s = ctx->stream;
    CK(cudaMemsetAsync(d, 0, 4 * sizeof(int), s));  // flag (never set), error word, two statuses
    const auto t0 = std::chrono::steady_clock::now();
    CK(launch_selftest_flag_wait(d, d + 1, d + 2, s));
    CK(launch_selftest_mbar_wait(d + 3, s));
    int h[4] = {0, 0, 0, 0};
    CK(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (sweep_gave_up) *sweep_gave_up = h[2] == 1 && h[1] == 1;
    if (tma_gave_up) *tma_gave_up = h[3] == 1;
    return DEEDS_OK;
}

}  // extern "C"
