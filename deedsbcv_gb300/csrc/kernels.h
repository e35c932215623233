// Kernel launchers of libdeeds_gpu (host-callable, C++ linkage, internal).
#pragma once
#include <atomic>
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace deeds {

// Process-wide count of kernels launched by this library (for accounting).
extern std::atomic<long long> g_kernel_launches;
inline void count_launches(int n) { g_kernel_launches.fetch_add(n, std::memory_order_relaxed); }

// Device-side description of one MST for the belief-propagation kernels.
struct BpTree {
    int len;                 // 2*hw+1
    float q;                 // label quantisation
    int sz;                  // nodes
    int root;                // ordered[0]
    int n_leaves;            // nodes without children (root excluded)
    const int* leaves;       // [n_leaves] deepest first
    const int* child_ptr;    // [sz+1] CSR of children per node
    const int* children;     // children of each node, in MST ordering order
    const int* parents;      // [sz]
    const float* edgemst;    // [sz] weight of the edge to the parent
    const float* u0;         // [sz] current displacement (label offsets are relative)
    const float* v0;
    const float* w0;
    int n_chains;            // heavy-path chains (downward pass)
    const int* chain_ptr;    // [n_chains+1] ranges into chain_nodes
    const int* chain_nodes;  // [sz] each chain's nodes from its start down to a leaf
};

// A displacement field given at full resolution (mode 1), on a control grid
// to be upsampled on the fly (mode 2), or zero (mode 0).
struct FieldRef {
    int mode;
    const float* u;
    const float* v;
    const float* w;
    int m1, n1, o1;
};

cudaError_t launch_mind_ssc(const float* d_im, int m, int n, int o, int qs, const float thr[5], float* d_scratch,
                            uint64_t* d_codes, cudaStream_t s);
cudaError_t launch_data_cost(const uint64_t* d_F, const uint64_t* d_M, int m, int n, int o, int g, int hw, int q,
                             int sy, int sx, int sz, float alpha1, float* d_cost, cudaStream_t s);
bool data_cost_tma_supported(int g, int hw, int q, int ny_tile);
size_t padded_codes_count(int m, int n, int o, int pad);
cudaError_t launch_data_cost_tma(const uint64_t* d_F, const uint64_t* d_M, uint64_t* d_Mpad, int m, int n, int o,
                                 int g, int hw, int q, int ny_tile, float alpha1, float* d_cost, int* d_err,
                                 cudaStream_t s);
cudaError_t launch_edge_sad(const float* d_im, int m, int n, int o, int g, float* d_sad, cudaStream_t s);
// Mean and standard deviation of one or two images in the reference's sequential
// float semantics (stats.cu): out[2*img + 0 / 1]; im1 unused when nimg is 1.
size_t image_stats_scratch_bytes(size_t sz, int nimg);
cudaError_t launch_image_stats(const float* im0, const float* im1, int nimg, size_t sz, void* scratch, float* out,
                               cudaStream_t s);
// d_mins: 4 * t.sz floats (per-node message minima, then the x | y | z edge offsets);
// d_pre: t.sz * len^3 floats (each node's scaled row, the transform's input)
// d_work: 3 ints; d_done: t.sz ints (list of finished nodes); d_err: error word (4: a bounded wait expired).
// The sweep's idle CTAs compute the argmin tables of finished nodes.
// concurrent: sweeps expected to run at once on the GPU (each takes its share of the CTA slots);
// d_allinds non-NULL: the argmin tables are wanted (the sweep lists its nodes for launch_bp_argmin)
cudaError_t launch_bp_up(const BpTree& t, float* d_cost, short* d_allinds, float* d_pre, float* d_mins, int* d_arrived,
                         int* d_work, int* d_done, int* d_err, int sm_count, int concurrent, cudaStream_t s);
// the argmin tables (allinds) of the nodes the sweep left, from its stored rows (after launch_bp_up)
cudaError_t launch_bp_argmin(const BpTree& t, short* d_allinds, const float* d_pre, const float* d_mins, int* d_work,
                             int* d_done, int* d_err, int sm_count, cudaStream_t s);
// d_lbl: t.sz + 2 ints of scratch (the nodes' labels as the walk resolves them, a
// ticket counter, an abort flag).  With d_allinds (16-byte aligned) the labels are
// gathered from the argmin tables; with d_allinds NULL each node's one needed
// entry is evaluated from its stored scaled row (d_pre, 16-byte aligned) and edge
// offsets (d_mins + t.sz: x | y | z), and no table is read or written.
cudaError_t launch_bp_down(const BpTree& t, const float* d_cost, short* d_allinds, const float* d_pre,
                           const float* d_mins, float* d_u1, float* d_v1, float* d_w1, int* d_lbl, int* d_err,
                           int sm_count, cudaStream_t s);
cudaError_t launch_shift(const float* d_in, float* d_out, int64_t n, float shift, cudaStream_t s);
cudaError_t launch_upsample(const float* u0, const float* v0, const float* w0, int m2, int n2, int o2, float* u,
                            float* v, float* w, int m, int n, int o, cudaStream_t s);
cudaError_t launch_warp_affine(const float* d_in, const float* X, const FieldRef& f, int m, int n, int o, float* d_out,
                               float* keep_u, float* keep_v, float* keep_w, cudaStream_t s);
cudaError_t launch_warp_image(const float* d_in, const FieldRef& f, int m, int n, int o, float* d_out, cudaStream_t s);
cudaError_t launch_warp_seg(const short* d_in, const float* X, const FieldRef& f, int m, int n, int o, short* d_out,
                            cudaStream_t s);
cudaError_t launch_consistent(float* u, float* v, float* w, float* u2, float* v2, float* w2, int m, int n, int o, int g,
                              float* scratch, cudaStream_t s);
// Soft-min level (soft.cu).  Tree arrays on the device; `ordered` is breadth-level
// order and the host keeps the level ranges.
struct SoftTreeDev {
    int len, sz, root, q;
    float tau;
    const int* ordered;
    const int* parents;
    const float* edgemst;
    const int* child_ptr;
    const int* children;
    const float* off;  // nullable: (3, sz) x|y|z label-unit offsets of each node's edge
    float* offbar;     // nullable (backward): dL/doff, (3, sz), zeroed by the caller
};
cudaError_t launch_soft_offsets(const float* prior, const int* parents, int root, int sz, float q, float* off,
                                cudaStream_t st);
cudaError_t launch_soft_offbar_to_prior(const float* offbar, const int* parents, int root, int sz, float q,
                                        float* gprior, cudaStream_t st);
cudaError_t launch_soft_upsample(const float* in, int mA, int nA, int oA, float* out, int m, int n, int o,
                                 cudaStream_t s);
cudaError_t launch_soft_upsample_adj(const float* gout, int m, int n, int o, float* gin, int mA, int nA, int oA,
                                     cudaStream_t s);
cudaError_t launch_soft_warp(const float* mov, const float* grid, int mA, int nA, int oA, float* out, int m, int n,
                             int o, cudaStream_t s);
cudaError_t launch_soft_warp_adj(const float* mov, const float* grid, int mA, int nA, int oA, const float* gout,
                                 float* gmov, float* gfull, int m, int n, int o, cudaStream_t s);
cudaError_t launch_soft_descriptor(const float* d_im, float* w6a, float* w6b, float* s12, int m, int n, int o, int qs,
                                   cudaStream_t st);
cudaError_t launch_soft_descriptor_adj(const float* d_im, float* w6a, float* w6b, const float* sbar12, float* dbar6,
                                       float* imbar, int m, int n, int o, int qs, cudaStream_t st);
cudaError_t launch_soft_cost(const float* sF, const float* sM, float* cost, int m, int n, int o, int g, int hw, int q,
                             float alpha1, float eps, cudaStream_t st);
cudaError_t launch_soft_cost_adj(const float* sF, const float* sM, const float* cbar, const float* cost, float* sFbar,
                                 float* sMbar, double* dot, int m, int n, int o, int g, int hw, int q, float alpha1,
                                 float eps, cudaStream_t st);
size_t soft_tree_smem(int len);
// Tree sweeps are persistent kernels; sweep_mem holds sz + 2 ints (ticket, per-node
// flags, error word).  The error word must be zeroed before the first sweep and is
// non-zero afterwards if a bounded wait gave up.
cudaError_t launch_soft_tree_forward(const SoftTreeDev& d, int* sweep_mem, const float* cost, float* B, float* M,
                                     float* Mmin, float* logp, float* disp, cudaStream_t st);
cudaError_t launch_soft_tree_backward(const SoftTreeDev& d, int* sweep_mem, const float* B, const float* M,
                                      const float* logp, const float* gdisp, float* R, float* Bbar, cudaStream_t st);
// linearBCV (linear.cu)
cudaError_t launch_lin_warp(const float* d_in, const float* X, int m, int n, int o, float* d_out, cudaStream_t s);
cudaError_t launch_lin_smooth(float* d_c0, float* d_c1, int m1, int n1, int o1, int len3, cudaStream_t s);
cudaError_t launch_lin_node_stats(const float* d_c0, const float* d_c1, const float* d_fixed, const float* d_moving,
                                  int m, int n, int o, int g, int len3, float* d_minval, int* d_minind,
                                  cudaStream_t s);
// Multi-atlas label fusion (fusion.cu): atlases warped onto the target vote per voxel.
constexpr int kFuseMaxAtlases = 64;
struct FusionAtlases {
    const float* image[kFuseMaxAtlases];     // warped atlas images (m*n*o)
    const int16_t* labels[kFuseMaxAtlases];  // warped atlas labels (m*n*o)
};
size_t fuse_scratch_floats(int n_atlas, int m, int n, int o);
cudaError_t launch_fuse_labels(const float* d_target, const FusionAtlases& at, int n_atlas, int m, int n, int o,
                               int radius, float eps, int power, float* d_scratch, int16_t* d_out, cudaStream_t s);
// Self-tests of the bounded device-side waits (a flag / an mbarrier nothing releases).
cudaError_t launch_selftest_flag_wait(const int* flag, int* err, int* status, cudaStream_t s);
cudaError_t launch_selftest_mbar_wait(int* status, cudaStream_t s);
cudaError_t launch_popc_probe(int blocks, int threads, int iters, unsigned long long* d_sink, cudaStream_t s);
cudaError_t launch_jacobian(const float* u, const float* v, const float* w, int m, int n, int o, int g, double* d_acc,
                            cudaStream_t s);

}  // namespace deeds
