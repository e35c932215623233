/*
 * deeds_gpu.h — C ABI of the GB300 (sm_103a) implementation of the deeds dense
 * discrete registration hot path (libdeeds_gpu.so).
 *
 * The reference (mattiaspaul/deedsBCV) has no library API: its stages are
 * header-inlined functions that take raw pointers and read process globals
 * (image_m/n/o, RAND_SAMPLES, SSD0/1; src/deedsBCV0.cpp:24-28).  Each entry point
 * below replaces one of those functions (cited per declaration) with explicit
 * dimensions, no globals, caller-owned buffers and an int status.
 *
 * Conventions
 *  - Volumes are m x n x o with i (size m, "y") fastest: index i + j*m + k*m*n
 *    (src/MINDSSCbox.h:84).  Displacements: u = x (dim 2), v = y (dim 1),
 *    w = z (dim 3), in voxels (src/deedsBCV0.cpp:193-194).
 *  - A control grid of spacing g has m1 = m/g, n1 = n/g, o1 = o/g nodes.
 *  - The affine matrix X is 16 floats, rows y, x, z at X[0..3], X[4..7],
 *    X[8..11] (src/dataCostD.h:281-283), as read from a linearBCV matrix file
 *    (src/deedsBCV0.cpp:159-165).
 *  - Functions named *_dev take device pointers and run on `stream` (a
 *    cudaStream_t passed as void*; NULL = the legacy default stream).  They are
 *    asynchronous unless stated otherwise.  All other pointers are host memory.
 *  - Every function returns DEEDS_OK (0) or an error code; deeds_last_error()
 *    gives the message.  No function calls exit().
 *  - A context holds the device scratch memory and is not thread-safe: use one
 *    context per host thread.
 */
#ifndef DEEDS_GPU_H
#define DEEDS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int deeds_status;
#define DEEDS_OK 0
#define DEEDS_ERR_INVALID 1   /* bad argument (dims, level parameters, null pointer) */
#define DEEDS_ERR_CUDA 2      /* a CUDA runtime call failed */
#define DEEDS_ERR_NOMEM 3     /* device or host allocation failed */
#define DEEDS_ERR_TIMEOUT 4   /* reserved: a bounded device-side wait gave up */
#define DEEDS_ERR_INTERNAL 5

#define DEEDS_MAX_LEVELS 10

typedef struct deeds_ctx deeds_ctx;

/* Registration parameters: the -a/-l/-G/-L/-Q flags of deedsBCV
 * (src/parseArguments.h:12-174, defaults src/deedsBCV0.cpp:76-79). */
typedef struct deeds_params {
    int levels;                      /* number of levels (<= DEEDS_MAX_LEVELS) */
    int grid[DEEDS_MAX_LEVELS];      /* -G grid spacing per level */
    int radius[DEEDS_MAX_LEVELS];    /* -L search radius (label half-width) per level */
    int quant[DEEDS_MAX_LEVELS];     /* -Q label quantisation per level */
    float alpha;                     /* -a regularisation weight (default 1.6) */
    float intensity_shift;           /* added to both images before registering (1024 for CT, src/deedsBCV0.cpp:139-144) */
    int verbose;                     /* print per-level progress like the reference */
} deeds_params;

/* Fill the reference defaults: 5 levels, G 8x7x6x5x4, L 8x7x6x5x4, Q 5x4x3x2x1, alpha 1.6, shift 1024. */
void deeds_default_params(deeds_params* p);

/* Create / destroy a context on CUDA device `device`. */
deeds_status deeds_create(deeds_ctx** ctx, int device);
void deeds_destroy(deeds_ctx* ctx);
/* Message of the last error on this context (or of the last failed deeds_create when ctx is NULL). */
const char* deeds_last_error(const deeds_ctx* ctx);
/* Library version string. */
const char* deeds_version(void);

/* ---------------------------------------------------------------------------
 * Whole registration (replaces main()'s level loop and output stage,
 * src/deedsBCV0.cpp:183-356).
 *
 * fixed, moving: host float volumes (m*n*o) as read from file (HU for CT);
 * params->intensity_shift is added to both.  flow_out: host, 3*sz1 floats
 * [u|v|w] on the last level's grid, exactly the *_displacements.dat payload
 * (src/deedsBCV0.cpp:341-349).  warped_out (nullable): the moving image warped by
 * the final field, with the shift removed again (src/deedsBCV0.cpp:350-356).
 * Synchronous.  The full-resolution field of the last call stays on the device
 * for deeds_warp_segmentation().
 */
deeds_status deeds_register(deeds_ctx* ctx, const float* fixed, const float* moving, int m, int n, int o,
                            const float X[16], const deeds_params* params, float* flow_out, float* warped_out);

/* Same with device-resident inputs/outputs; d_fixed/d_moving are not modified.
 * Host-side work (Prim's MST, schedules) still runs inside the call; returns
 * after the result is on the device. */
deeds_status deeds_register_dev(deeds_ctx* ctx, const float* d_fixed, const float* d_moving, int m, int n, int o,
                                const float X[16], const deeds_params* params, float* d_flow_out,
                                float* d_warped_out, void* stream);

/* One pair of a batch: host buffers, any size (pairs of one batch may differ). */
typedef struct deeds_pair {
    const float* fixed;   /* m*n*o, raw intensities (params->intensity_shift is added) */
    const float* moving;  /* m*n*o */
    int m, n, o;
    const float* X;       /* 16-float affine matrix, or NULL for identity */
    float* flow_out;      /* 3*sz1 of the last level, as deeds_register */
    float* warped_out;    /* m*n*o or NULL */
} deeds_pair;

/* Batched registration (no counterpart in the reference, which registers one
 * pair per process): registers n_pairs independent pairs with `lanes` pairs in
 * flight at a time.  Each lane is an internal context with its own streams and
 * scratch; while one lane's pair waits for its host-built MSTs, the others keep
 * the GPU busy.  Results are identical to calling deeds_register per pair.
 * lanes <= 0 picks a default (3).  Synchronous; returns the first failing
 * pair's status (its index in the message) after all lanes have stopped. */
deeds_status deeds_register_batch(deeds_ctx* ctx, const deeds_pair* pairs, int n_pairs, const deeds_params* params,
                                  int lanes);

/* Warp a label volume with the last deeds_register() result: nearest-neighbour,
 * clamp-to-edge (the -S output, src/deedsBCV0.cpp:361-379 via warpAffineS,
 * src/dataCostD.h:241-266).  Host buffers; synchronous. */
deeds_status deeds_warp_segmentation(deeds_ctx* ctx, const int16_t* seg, int16_t* seg_out);

/* applyBCV / applyBCVfloat: upsample a grid flow (3*sz1, grid step g inferred from
 * its length as src/applyBCV.cpp:161-164 does, or given if g > 0) to full
 * resolution and warp `in`.  dtype 0: int16 labels, nearest (src/applyBCV.cpp:186-198);
 * dtype 1: float image, trilinear (src/applyBCVfloat.cpp:190-198).  Host buffers. */
deeds_status deeds_apply_flow(deeds_ctx* ctx, const float* flow, size_t flow_len, int g, const float X[16],
                              const void* in, int dtype, int m, int n, int o, void* out);

/* ---------------------------------------------------------------------------
 * Stage entry points (device pointers, asynchronous on `stream`).
 */

/* descriptor(): MIND-SSC with patch radius qs, quantised to one 64-bit code per
 * voxel (src/MINDSSCbox.h:127-232).  Bit-exact with the reference. */
deeds_status deeds_mind_ssc_dev(deeds_ctx* ctx, const float* d_im, int m, int n, int o, int qs,
                                uint64_t* d_codes, void* stream);

/* dataCostCL(): Hamming cost volume cost[node*len3 + label], len3=(2hw+1)^3,
 * label = ly + lx*len + lz*len^2 (src/dataCostD.h:108-210).  Bit-exact. */
deeds_status deeds_data_cost_dev(deeds_ctx* ctx, const uint64_t* d_fixed_codes, const uint64_t* d_moving_codes,
                                 int m, int n, int o, int g, int hw, int q, float alpha, float* d_cost,
                                 void* stream);

/* The edge-cost half of primsGraph(): per-node block SADs to the 6 neighbours,
 * d_sad[nb*sz1 + node], nb order -x,+x,-y,+y,-z,+z (src/primsMST.h:75-100). */
deeds_status deeds_mst_edges_dev(deeds_ctx* ctx, const float* d_im, int m, int n, int o, int g, float* d_sad,
                                 void* stream);

/* The tree half of primsGraph() (host): image statistics (src/primsMST.h:101-110)
 * and Prim's algorithm over the SAD edge weights, giving the breadth-level
 * ordering, parents and per-child edge weights (src/primsMST.h:112-211). */
deeds_status deeds_image_stats(const float* im, size_t count, float* mean, float* stddev);
deeds_status deeds_prims_from_sad(const float* sad, float stddev, int m1, int n1, int o1, int g, int* ordered,
                                  int* parents, float* edgemst);

/* The image statistics of primsGraph() (src/primsMST.h:101-110) on the device:
 * the reference's sequential float mean and standard deviation of d_im
 * (count floats), to the bit, written to d_out[0] (mean) and d_out[1] (std).
 * The registration computes these on the device for its host trees. */
deeds_status deeds_image_stats_dev(deeds_ctx* ctx, const float* d_im, size_t count, float* d_out, void* stream);

/* Diagnostic counters of the host MST construction (process-wide, since load):
 * out[0] trees whose minimum spanning tree is unique (built without a Prim
 * walk), out[1] trees with ambiguous equal-weight edges (Prim's heap walk decides
 * them, stopped once it has), out[2] Prim steps walked for those trees (the
 * walk starts while the tie analysis runs; a unique tree's steps are discarded),
 * out[3] steps that full walks of the same trees would take.  Every tree equals
 * primsGraph()'s. */
void deeds_mst_path_counts(long long out[4]);

/* regularisationCL(): exact min-sum belief propagation on the MST with 3-D
 * quadratic distance-transform messages (src/regularisation.h:6-303).
 * d_cost (sz1*len3) is overwritten with the upward-pass state (each non-root
 * row = that node's message, root row = its total), as the reference leaves it.
 * ordered/parents/edgemst are host arrays (from deeds_prims_from_sad).
 * d_allinds (nullable, sz1*len3 int16, 16-byte aligned as any cudaMalloc block
 * is) receives the argmin tables. Synchronous. */
deeds_status deeds_tree_bp_dev(deeds_ctx* ctx, float* d_cost, const float* d_u0, const float* d_v0,
                               const float* d_w0, int m1, int n1, int o1, int hw, int q, const int* ordered,
                               const int* parents, const float* edgemst, float* d_u1, float* d_v1, float* d_w1,
                               int16_t* d_allinds, void* stream);

/* upsampleDeformationsCL(): trilinear resample of a (m2,n2,o2) field to (m,n,o)
 * (src/transformations.h:245-279). */
deeds_status deeds_upsample_dev(const float* d_u0, const float* d_v0, const float* d_w0, int m2, int n2, int o2,
                                float* d_u, float* d_v, float* d_w, int m, int n, int o, void* stream);

/* warpAffine(): affine + dense field, trilinear, clamp-to-edge
 * (src/dataCostD.h:267-298). d_u/d_v/d_w may be NULL for a zero field. */
deeds_status deeds_warp_affine_dev(const float* d_in, const float X[16], const float* d_u, const float* d_v,
                                   const float* d_w, int m, int n, int o, float* d_out, void* stream);

/* warpImageCL(): warp by a field relative to the voxel position (src/dataCostD.h:213-239). */
deeds_status deeds_warp_image_dev(const float* d_in, const float* d_u, const float* d_v, const float* d_w, int m,
                                  int n, int o, float* d_out, void* stream);

/* warpAffineS(): nearest-neighbour label warp (src/dataCostD.h:241-266). */
deeds_status deeds_warp_seg_dev(const int16_t* d_in, const float X[16], const float* d_u, const float* d_v,
                                const float* d_w, int m, int n, int o, int16_t* d_out, void* stream);

/* consistentMappingCL(): 10 inverse-consistency iterations on both grid fields,
 * in place (src/transformations.h:189-242). */
deeds_status deeds_consistent_dev(deeds_ctx* ctx, float* d_u, float* d_v, float* d_w, float* d_u2, float* d_v2,
                                  float* d_w2, int m, int n, int o, int g, void* stream);

/* consistentMappingCL() for callers that cannot allocate device memory while
 * they run (no counterpart in the reference): host frameworks whose memory pool
 * owns the device, real-time loops that size everything at start-up, and code
 * that must not block on the device synchronisation cudaMalloc/cudaFree can
 * imply.  Same kernels and results as deeds_consistent_dev, but the 12 grid
 * fields of scratch live in a fixed device array of DEEDS_NOALLOC_MAX_NODES
 * nodes (6 MiB); no context is needed and no call allocates.  With lazy module
 * loading (the CUDA default) that array is reserved when the first call on a
 * device loads the library's module into its context, and the device holds it
 * until the context ends (process exit or cudaDeviceReset): make the first
 * call per device at start-up, before a memory pool reserves the device and
 * before any stream capture; it resolves the array's device address with that
 * device current.  The address is kept per device and context, so a call in a
 * new context of the device (e.g. after cudaDeviceReset) resolves it again,
 * which again loads the module and reserves the array.  Grids with more than
 * DEEDS_NOALLOC_MAX_NODES nodes, or with n or o above 65535, are rejected with
 * DEEDS_ERR_INVALID before anything runs.  All calls share the array: calls
 * that overlap on the GPU race.  Errors are reported by status only (no message
 * is recorded, as that would allocate). */
#define DEEDS_NOALLOC_MAX_NODES 131072
deeds_status deeds_consistent_noalloc_dev(float* d_u, float* d_v, float* d_w, float* d_u2, float* d_v2, float* d_w2,
                                          int m, int n, int o, int g, void* stream);

/* jacobian(): std of the Jacobian determinant and fraction of J<0 of a grid
 * field (src/transformations.h:84-185; a diagnostic, parallel reduction, not
 * bit-exact).  Synchronous. */
deeds_status deeds_jacobian_dev(deeds_ctx* ctx, const float* d_u, const float* d_v, const float* d_w, int m, int n,
                                int o, int g, float* jstd, float* neg_frac, void* stream);

/* ---------------------------------------------------------------------------
 * Tracing and accounting (the reference times each stage with gettimeofday and
 * prints per-level seconds, src/deedsBCV0.cpp:228-308; here CUDA events).
 */
#define DEEDS_STAGE_MIND 0       /* MIND-SSC descriptors */
#define DEEDS_STAGE_DATACOST 1   /* Hamming cost volumes */
#define DEEDS_STAGE_MST 2        /* MST edge SADs (GPU side of primsGraph) */
#define DEEDS_STAGE_BP_UP 3      /* upward belief propagation */
#define DEEDS_STAGE_BP_DOWN 4    /* root argmin + downward pass */
#define DEEDS_STAGE_TRANSFORM 5  /* upsampling and warps */
#define DEEDS_STAGE_CONSISTENT 6 /* inverse-consistent mapping */
#define DEEDS_STAGE_TREE_WAIT 7  /* host time spent waiting for Prim trees */
#define DEEDS_STAGE_BP_ARGMIN 8  /* argmin tables of the upward pass (from its stored rows) */
#define DEEDS_NUM_STAGES 9

/* Enable/disable per-stage CUDA-event timing in deeds_register*(). */
deeds_status deeds_set_profiling(deeds_ctx* ctx, int on);
/* Milliseconds per stage accumulated since the last reset (DEEDS_NUM_STAGES
 * floats); `launches` (nullable) receives per-stage kernel launch counts. */
deeds_status deeds_stage_times(deeds_ctx* ctx, float* ms, long long* launches);
deeds_status deeds_reset_stage_times(deeds_ctx* ctx);
/* Number of kernels this library has launched in the process so far. */
long long deeds_kernel_launches(void);
/* Measure this GPU's rate of the cost-volume inner operation with a register-only
 * probe kernel: 64-bit samples XORed with a key and summed three at a time
 * through a carry-save adder (two 64-bit POPCs per three samples); returns
 * samples (popc64 equivalents) per second. Synchronous, ~0.2 s. */
deeds_status deeds_measure_popc_rate(deeds_ctx* ctx, double* popc64_per_s);

/* ---------------------------------------------------------------------------
 * Soft-min form (no counterpart in the reference).  One deeds level
 * (src/deedsBCV0.cpp:238-306) relaxed so that it is differentiable in both
 * images and in alpha:
 *   - descriptor: the continuous MIND-SSC level s = 6 exp(-mind1) per channel,
 *     i.e. the quantity src/MINDSSCbox.h:175-224 thresholds into codes;
 *   - cost: alpha1 * sum over the node's samples (src/dataCostD.h:141-200
 *     sampling and clamping) and the 12 channels of sqrt(d^2 + eps^2) - eps;
 *   - messages: src/regularisation.h:190-238 with min replaced by the soft-min
 *     -tau log sum exp(-x/tau), over the MST given by primsGraph();
 *   - output: the expected displacement sum_l p(l) d(l) per control point
 *     (u|v|w, 3 x m1*n1*o1 floats), from soft root-to-leaf marginals.
 * The prior field is zero (the level registers `moving` as given).
 * tau -> 0 recovers the hard argmin of the min-sum tree.
 */
typedef struct deeds_soft_params {
    int grid;        /* control-point spacing g */
    int radius;      /* label half-width hw, 0..5: label set (2hw+1)^3 */
    int quant;       /* label quantisation q */
    int mind_radius; /* MIND-SSC radius; 0 = floor(q/2 + 1) as src/deedsBCV0.cpp:183-186 */
    float alpha;     /* regularisation weight (-a) */
    float tau;       /* soft-min temperature, > 0 */
    float eps;       /* smoothing of |x| in the descriptor cost, > 0 */
} deeds_soft_params;

/* grid 4, radius 3, quant 1, mind_radius 0, alpha 1.6, tau 0.5, eps 0.01 */
void deeds_soft_default_params(deeds_soft_params* p);

/* Continuous MIND-SSC descriptor: 12 x m*n*o floats (channel-major). */
deeds_status deeds_soft_descriptor_dev(deeds_ctx* ctx, const float* d_im, int m, int n, int o, int mind_radius,
                                       float* d_desc, void* stream);

/* Soft cost volume m1*n1*o1 x (2hw+1)^3 from two soft descriptors. */
deeds_status deeds_soft_cost_dev(deeds_ctx* ctx, const float* d_desc_fixed, const float* d_desc_moving, int m, int n,
                                 int o, const deeds_soft_params* p, float* d_cost, void* stream);

/* Forward: expected displacement (u|v|w) of the soft level, relative to the
 * prior field when d_prior is given.  ordered/parents/edgemst are the host arrays
 * of primsGraph() on the fixed image at this grid (deeds_prims_from_sad); every
 * parent must precede its children in `ordered`.  d_prior (nullable): the current
 * grid field u|v|w (3 x m1*n1*o1), which enters the pairwise term as in
 * regularisationCL (src/regularisation.h:205-208): |lab(child) - lab(parent) - off|^2,
 * off = (prior[parent] - prior[child]) / q; `moving` is then expected to be
 * warped by the prior already (deeds_soft_warp_dev).  Synchronous (it reads back
 * the tree sweeps' status; DEEDS_ERR_TIMEOUT if a bounded device-side wait gave
 * up). */
deeds_status deeds_soft_forward_dev(deeds_ctx* ctx, const float* d_fixed, const float* d_moving, int m, int n, int o,
                                    const deeds_soft_params* p, const int* ordered, const int* parents,
                                    const float* edgemst, const float* d_prior, float* d_disp, void* stream);

/* Backward: given dL/d(displacement) (3 x m1*n1*o1), writes dL/dfixed and
 * dL/dmoving (m*n*o each, overwritten; either may be NULL), dL/dprior through the
 * pairwise offsets (3 x m1*n1*o1, overwritten; NULL unless d_prior is given) and
 * dL/dalpha (host float, may be NULL).  Recomputes the forward sweeps (no state is
 * kept from deeds_soft_forward_dev).  Synchronous, like the forward. */
deeds_status deeds_soft_backward_dev(deeds_ctx* ctx, const float* d_fixed, const float* d_moving, int m, int n, int o,
                                     const deeds_soft_params* p, const int* ordered, const int* parents,
                                     const float* edgemst, const float* d_prior, const float* d_grad_disp,
                                     float* d_grad_fixed, float* d_grad_moving, float* d_grad_prior,
                                     float* grad_alpha, void* stream);

/* Forward that keeps the level's state resident on the device (descriptors of
 * both images, cost volume, tree, messages and marginals: about
 * (96*m*n*o + 16*m1*n1*o1*(2hw+1)^3) bytes) under a slot of the context, written
 * to *slot, so that deeds_soft_backward_kept_dev runs only the adjoint.  Same
 * arguments and results as deeds_soft_forward_dev.  The slot stays in use until
 * deeds_soft_release; a released slot's buffers serve the next keep forward
 * (deeds_soft_trim frees those of unused slots). */
deeds_status deeds_soft_forward_keep_dev(deeds_ctx* ctx, const float* d_fixed, const float* d_moving, int m, int n,
                                         int o, const deeds_soft_params* p, const int* ordered, const int* parents,
                                         const float* edgemst, const float* d_prior, float* d_disp, int* slot,
                                         void* stream);

/* deeds_soft_backward_dev for the forward kept in `slot`: no recomputation.  The
 * images, dimensions, parameters and prior must be those of that forward, with
 * the images and prior unchanged since (dimensions, parameters and the presence
 * of a prior are checked: DEEDS_ERR_INVALID otherwise).  May run any number of
 * times while the slot is in use. */
deeds_status deeds_soft_backward_kept_dev(deeds_ctx* ctx, int slot, const float* d_fixed, const float* d_moving,
                                          int m, int n, int o, const deeds_soft_params* p, const float* d_prior,
                                          const float* d_grad_disp, float* d_grad_fixed, float* d_grad_moving,
                                          float* d_grad_prior, float* grad_alpha, void* stream);

/* Ends the use of a kept slot (its buffers are kept for reuse). */
deeds_status deeds_soft_release(deeds_ctx* ctx, int slot);

/* Frees the device buffers of every kept slot not in use (synchronises the device). */
deeds_status deeds_soft_trim(deeds_ctx* ctx);

/* Batched soft level: npairs pairs of one size and one parameter set, each with
 * its own images, tree (ordered[i], parents[i], edgemst[i]) and, when d_prior is
 * non-NULL, prior field, run concurrently on lane streams of the context (child
 * contexts with their own buffers; at most 8 lanes, pair i of each group of 8 on
 * lane i).  The tree sweeps are latency-bound, so pairs on different lanes fill
 * each other's idle SMs.  The lanes start after the work already enqueued on
 * `stream`; the call returns when every lane is done (synchronous, like the
 * single-pair forms).  With slots non-NULL each pair's forward state is kept:
 * slots[i] (written) names it in its lane, for deeds_soft_backward_batch_dev
 * and deeds_soft_release_batch with the same npairs.  Errors name the pair. */
deeds_status deeds_soft_forward_batch_dev(deeds_ctx* ctx, int npairs, const float* const* d_fixed,
                                          const float* const* d_moving, int m, int n, int o,
                                          const deeds_soft_params* p, const int* const* ordered,
                                          const int* const* parents, const float* const* edgemst,
                                          const float* const* d_prior, float* const* d_disp, int* slots,
                                          void* stream);

/* Backward of a batch: with slots (from deeds_soft_forward_batch_dev, same
 * npairs) over the kept states, else recomputing each pair's forward from its
 * tree.  d_grad_fixed / d_grad_moving / d_grad_prior: NULL or npairs pointers;
 * grad_alpha: NULL or npairs floats (dL/dalpha per pair). */
deeds_status deeds_soft_backward_batch_dev(deeds_ctx* ctx, int npairs, const int* slots,
                                           const float* const* d_fixed, const float* const* d_moving, int m, int n,
                                           int o, const deeds_soft_params* p, const int* const* ordered,
                                           const int* const* parents, const float* const* edgemst,
                                           const float* const* d_prior, const float* const* d_grad_disp,
                                           float* const* d_grad_fixed, float* const* d_grad_moving,
                                           float* const* d_grad_prior, float* grad_alpha, void* stream);

/* Ends the use of a batch's kept slots. */
deeds_status deeds_soft_release_batch(deeds_ctx* ctx, int npairs, const int* slots);

/* Differentiable trilinear upsampling of a field u|v|w from an mA x nA x oA grid to
 * m x n x o (the coordinates of upsampleDeformationsCL, src/transformations.h:245-279,
 * in float arithmetic), and its adjoint (gin overwritten). */
deeds_status deeds_soft_upsample_dev(deeds_ctx* ctx, const float* d_in, int mA, int nA, int oA, float* d_out, int m,
                                     int n, int o, void* stream);
deeds_status deeds_soft_upsample_backward_dev(deeds_ctx* ctx, const float* d_grad_out, int m, int n, int o,
                                              float* d_grad_in, int mA, int nA, int oA, void* stream);

/* Differentiable warp of an m x n x o image by a grid field u|v|w (mA x nA x oA,
 * upsampled on the fly): warpAffine with the identity (src/dataCostD.h:267-295) in
 * float arithmetic; its adjoint writes dL/dmoving and dL/dgrid (each nullable,
 * overwritten). */
deeds_status deeds_soft_warp_dev(deeds_ctx* ctx, const float* d_moving, int m, int n, int o, const float* d_grid,
                                 int mA, int nA, int oA, float* d_out, void* stream);
deeds_status deeds_soft_warp_backward_dev(deeds_ctx* ctx, const float* d_moving, int m, int n, int o,
                                          const float* d_grid, int mA, int nA, int oA, const float* d_grad_out,
                                          float* d_grad_moving, float* d_grad_grid, void* stream);

/* ---------------------------------------------------------------------------
 * linearBCV: affine / rigid pre-registration (src/linearBCV.cpp:163-262).  Per
 * level both images are warped by the current matrix (the moving image forwards,
 * the fixed image by its QR inverse), MIND-SSC codes and Hamming cost volumes are
 * built in both directions (alpha 1), the volumes are smoothed along y, x and z,
 * each control point votes with its best label, and a least-trimmed-squares fit
 * of the best half of the votes updates the matrix.  The matrix uses the deeds
 * layout (X[0..3] gives y, X[4..7] x, X[8..11] z) and maps fixed voxels to moving
 * voxels; the linearBCV CLI writes it as stem_matrix.txt for deedsBCV -A. */
typedef struct deeds_linear_params {
    int levels;                      /* -l (default 4) */
    int grid[DEEDS_MAX_LEVELS];      /* -G (default 7x6x5x4) */
    int radius[DEEDS_MAX_LEVELS];    /* -L (default 5x4x3x2) */
    int quant[DEEDS_MAX_LEVELS];     /* -Q (default 4x3x2x1) */
    int rigid;                       /* -R: 6-parameter rigid fit instead of affine */
    float intensity_shift;           /* added to both images (1024, src/linearBCV.cpp:146-153) */
    int verbose;                     /* print "# points used" per level like the reference */
} deeds_linear_params;

void deeds_linear_default_params(deeds_linear_params* p);

/* Whole linearBCV registration on host buffers (copied to the device inside);
 * X_out: 16 floats.  Replaces main of src/linearBCV.cpp:163-262. */
deeds_status deeds_linear_register(deeds_ctx* ctx, const float* fixed, const float* moving, int m, int n, int o,
                                   const deeds_linear_params* params, float X_out[16]);
/* The same on device buffers and the caller's stream (synchronises it once per level). */
deeds_status deeds_linear_register_dev(deeds_ctx* ctx, const float* d_fixed, const float* d_moving, int m, int n,
                                       int o, const deeds_linear_params* params, float X_out[16], void* stream);

/* The -S output of linearBCV (src/linearBCV.cpp:301-317): a label map warped by X
 * alone (nearest neighbour, warpAffineS with a zero field); host buffers. */
deeds_status deeds_affine_warp_segmentation(deeds_ctx* ctx, const int16_t* seg, int m, int n, int o, const float X[16],
                                           int16_t* seg_out);

/* warpAffine of src/affineLTS1.h:39-68: affine map only, 0 outside the volume. */
deeds_status deeds_lin_warp_dev(const float* d_in, const float X[16], int m, int n, int o, float* d_out, void* stream);
/* The three in-place smoothing passes of estimateAffine2 (src/affineLTS1.h:124-158)
 * on one cost volume (m1 x n1 x o1 nodes x len3 labels). */
deeds_status deeds_lin_smooth_dev(float* d_cost, int m1, int n1, int o1, int len3, void* stream);
/* estimateAffine2 (src/affineLTS1.h:91-236): smooths both cost volumes in place
 * and returns X = fit * Xprev; d_fixed/d_moving are the shifted (+1024) images.
 * *points_used (nullable) receives the number of points fitted. */
deeds_status deeds_estimate_affine_dev(deeds_ctx* ctx, const float* d_fixed, const float* d_moving, float* d_cost,
                                       float* d_cost2, int m, int n, int o, int g, int hw, int q, int rigid,
                                       const float Xprev[16], float X[16], int* points_used, void* stream);
/* affineRobust (src/QRsolve.h:258-296) on host point sets in column layout
 * (y | x | z | 1, len points each). */
deeds_status deeds_affine_robust(const float* pts1, const float* pts2, int len, int rigid, float RT[16]);

/* Self-test of the bounded device-side waits: the tree sweeps' wait on a flag and
 * the cost volume's wait on a TMA mbarrier are each run on a flag / barrier that
 * nothing releases; *sweep_gave_up / *tma_gave_up are set to 1 when the wait
 * expired and reported it (the error word for the sweep), *seconds to the time
 * both took.  The context stays usable afterwards. */
deeds_status deeds_selftest_bounded_waits(deeds_ctx* ctx, int* sweep_gave_up, int* tma_gave_up, double* seconds);

/* ---------------------------------------------------------------------------
 * Multi-atlas segmentation.  The reference names joint label fusion of several
 * registered atlases as future work (README.md:8, README.md:201) and has no
 * implementation; these entry points register atlases to a target with the
 * deeds path above and fuse their warped labels by locally weighted voting:
 *   D_i(x) = window sum over the (2*radius+1)^3 patch around x (clamp-to-edge;
 *            separable: i, then j, then k) of (target - image_i)^2;
 *   w_i(x) = (1 / (D_i(x) + eps))^power   (power 0: majority vote);
 *   label(x) = argmax over labels L of sum_i w_i [labels_i(x) == L] (sums in
 *              atlas order; ties to the smaller label).
 */
#define DEEDS_FUSE_MAX_ATLASES 64

/* Fusion of atlases already warped onto the target (device pointers: d_images
 * and d_labels are host arrays of n_atlas device pointers, each m*n*o).
 * Asynchronous on `stream`; scratch (2 * n_atlas * m*n*o floats) belongs to ctx. */
deeds_status deeds_fuse_labels_dev(deeds_ctx* ctx, const float* d_target, const float* const* d_images,
                                   const int16_t* const* d_labels, int n_atlas, int m, int n, int o, int radius,
                                   float eps, int power, int16_t* d_out, void* stream);

/* End to end (host buffers): registers every atlas image to the target
 * (deeds_register_batch with `lanes`; identity affine), warps each atlas' labels
 * with its flow (as deeds_apply_flow, nearest neighbour), fuses them with the
 * warped atlas images, and writes the fused labels (m*n*o).  warped_labels_out
 * and warped_images_out (nullable) receive the n_atlas warped label volumes and
 * warped images back to back.  Synchronous. */
deeds_status deeds_multi_atlas(deeds_ctx* ctx, const float* target, const float* const* atlas_images,
                               const int16_t* const* atlas_labels, int n_atlas, int m, int n, int o,
                               const deeds_params* params, int lanes, int radius, float eps, int power,
                               int16_t* labels_out, int16_t* warped_labels_out, float* warped_images_out);

/* ---------------------------------------------------------------------------
 * Parallel gzip IO for NIfTI volumes (host only; the reference uses single-
 * threaded zlib, src/imageIOgzType.h:14-26, 212-218).  deeds_gz_write deflates
 * head ++ data in 4 MiB chunks on `threads` threads (0 = all cores) into
 * concatenated gzip members that any gzip reader accepts; level as zlib
 * (-1 = default 6).  deeds_gz_read inflates such files in parallel and any
 * other gzip or plain file through zlib; *total receives the decompressed size
 * (out = NULL only asks for it; a too small cap returns DEEDS_ERR_INVALID with
 * *total set). */
deeds_status deeds_gz_write(const char* path, const void* head, size_t head_bytes, const void* data,
                            size_t data_bytes, int level, int threads);
deeds_status deeds_gz_read(const char* path, void* out, size_t cap, size_t* total, int threads);
const char* deeds_gz_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* DEEDS_GPU_H */
