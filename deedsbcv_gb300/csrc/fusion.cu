// Multi-atlas label fusion on sm_103a.  The reference names joint label fusion
// as future work for multi-atlas segmentation (README.md:8, README.md:201) and
// implements none; this is the voting step that follows registering several
// atlases to one target with deeds: every atlas' labels and image, warped onto
// the target, vote per voxel.
//
// Rule (locally weighted voting by inverse patch distance):
//   D_i(x) = sum over the (2r+1)^3 patch around x (clamp-to-edge) of
//            (T - A_i)^2, summed as three separable window passes (i, then j,
//            then k; each window sum in offset order -r..r from 0);
//   w_i(x) = (1 / (D_i(x) + eps))^p  (p integer >= 0; p = 0 is majority vote);
//   label(x) = the label L maximising sum_i w_i [L_i(x) == L], the sum taken in
//              atlas order; ties go to the smaller label.
// Every step is a float operation whose order is fixed above (built with
// --fmad=false), so the CPU restatement reproduces it bit for bit.
//
// Roofline: HBM.  Per voxel and atlas: target + image read and the squared
// differences written (12 B), two more window passes (2 x 8 B), and the vote's
// read of the distances and labels (6 B): ~34 B per voxel per atlas, plus the
// 2 B label written.
#include "common.cuh"
#include "kernels.h"

namespace deeds {

namespace {

// Window sum along one axis (stride, extent) with clamp-to-edge, for every atlas
// (gridDim.y); SQ: the input is (T - A_i)^2 formed on the fly.
template <bool SQ>
__global__ void __launch_bounds__(256) k_window(const float* __restrict__ target, FusionAtlases at,
                                                const float* __restrict__ in, float* __restrict__ out, int m, int n,
                                                int o, int axis, int r) {
    const int64_t sz = (int64_t)m * n * o;
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= sz) return;
    const int a = blockIdx.y;
    const int64_t base = (int64_t)a * sz;
    const int i = (int)(v % m), j = (int)((v / m) % n), k = (int)(v / ((int64_t)m * n));
    const int c = axis == 0 ? i : (axis == 1 ? j : k);
    const int ext = axis == 0 ? m : (axis == 1 ? n : o);
    const int64_t stride = axis == 0 ? 1 : (axis == 1 ? (int64_t)m : (int64_t)m * n);
    const int64_t row0 = v - (int64_t)c * stride;
    float s = 0.0f;
    for (int d = -r; d <= r; d++) {
        const int64_t p = row0 + (int64_t)clampi(c + d, 0, ext - 1) * stride;
        float x;
        if (SQ) {
            const float df = target[p] - at.image[a][p];
            x = df * df;
        } else {
            x = in[base + p];
        }
        s = s + x;
    }
    out[base + v] = s;
}

// The vote: weights from the window sums, labels of every atlas, the winner.
__global__ void __launch_bounds__(256) k_vote(FusionAtlases at, int n_atlas, const float* __restrict__ dist,
                                              int64_t sz, float eps, int power, int16_t* __restrict__ out) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= sz) return;
    float w[kFuseMaxAtlases];
    int16_t lab[kFuseMaxAtlases];
    for (int a = 0; a < n_atlas; a++) {
        const float inv = 1.0f / (dist[(int64_t)a * sz + v] + eps);
        float x = 1.0f;
        for (int q = 0; q < power; q++) x = x * inv;
        w[a] = x;
        lab[a] = at.labels[a][v];
    }
    int best = lab[0];
    float best_s = -1.0f;
    for (int a = 0; a < n_atlas; a++) {
        const int L = lab[a];
        float s = 0.0f;
        for (int b = 0; b < n_atlas; b++)
            if (lab[b] == L) s = s + w[b];
        if (s > best_s || (s == best_s && L < best)) {
            best_s = s;
            best = L;
        }
    }
    out[v] = (int16_t)best;
}

}  // namespace

size_t fuse_scratch_floats(int n_atlas, int m, int n, int o) { return 2 * (size_t)n_atlas * m * n * o; }

cudaError_t launch_fuse_labels(const float* d_target, const FusionAtlases& at, int n_atlas, int m, int n, int o,
                               int radius, float eps, int power, float* d_scratch, int16_t* d_out, cudaStream_t s) {
    if (n_atlas < 1 || n_atlas > kFuseMaxAtlases || radius < 0 || power < 0) return cudaErrorInvalidValue;
    const int64_t sz = (int64_t)m * n * o;
    float* a = d_scratch;
    float* b = d_scratch + (size_t)n_atlas * sz;
    const dim3 grid((unsigned)((sz + 255) / 256), n_atlas);
    k_window<true><<<grid, 256, 0, s>>>(d_target, at, nullptr, a, m, n, o, 0, radius);
    k_window<false><<<grid, 256, 0, s>>>(d_target, at, a, b, m, n, o, 1, radius);
    k_window<false><<<grid, 256, 0, s>>>(d_target, at, b, a, m, n, o, 2, radius);
    k_vote<<<(unsigned)((sz + 255) / 256), 256, 0, s>>>(at, n_atlas, a, sz, eps, power, d_out);
    count_launches(4);
    return cudaGetLastError();
}

}  // namespace deeds
