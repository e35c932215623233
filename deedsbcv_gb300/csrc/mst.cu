// MST edge costs on sm_103a: the image-sized half of primsGraph
// (src/primsMST.h:75-100).  Each undirected grid edge is computed once (the
// reference computes it from both ends; |a-b| = |b-a| and the block order is the
// same, so both values are bit-identical) with the reference's sequential float
// sum over the g^3 block in k, j, i order.
// Output sad[nb*sz1 + node], nb = -x,+x,-y,+y,-z,+z; 0 where the neighbour is
// outside the grid.  Roofline: L2-bound gather, ~2 x 4 B per voxel per edge
// direction (3 directions), negligible next to the cost volume.
#include "common.cuh"
#include "kernels.h"

namespace deeds {

namespace {

__global__ void k_edge_sad(const float* __restrict__ im, float* __restrict__ sad, int m, int n, int o, int g) {
    const int m1 = m / g, n1 = n / g, o1 = o / g;
    const int64_t sz1 = (int64_t)m1 * n1 * o1;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * sz1) return;
    const int dir = (int)(t / sz1);  // 0: x, 1: y, 2: z
    const int64_t node = t % sz1;
    const int k = (int)(node / ((int64_t)m1 * n1)), j = (int)((node / m1) % n1), i = (int)(node % m1);
    const int di = dir == 1, dj = dir == 0, dk = dir == 2;
    const int ii = i + di, jj = j + dj, kk = k + dk;
    const int64_t mn = (int64_t)m * n;
    // the "-dir" slot of this node is written here when it has no -dir neighbour
    const int has_neg = dir == 0 ? j > 0 : (dir == 1 ? i > 0 : k > 0);
    if (!has_neg) sad[(2 * dir) * sz1 + node] = 0.0f;
    if (ii >= m1 || jj >= n1 || kk >= o1) {
        sad[(2 * dir + 1) * sz1 + node] = 0.0f;
        return;
    }
    const float* a = im + (int64_t)i * g + (int64_t)j * g * m + (int64_t)k * g * mn;
    const float* b = im + (int64_t)ii * g + (int64_t)jj * g * m + (int64_t)kk * g * mn;
    float s = 0.0f;
    for (int c = 0; c < g; c++)
        for (int bb = 0; bb < g; bb++) {
            const int64_t off = (int64_t)bb * m + (int64_t)c * mn;
            for (int aa = 0; aa < g; aa++) s = s + fabsf(__ldg(a + off + aa) - __ldg(b + off + aa));
        }
    const int64_t nb_node = ii + (int64_t)jj * m1 + (int64_t)kk * m1 * n1;
    sad[(2 * dir + 1) * sz1 + node] = s;   // +dir edge of this node
    sad[(2 * dir) * sz1 + nb_node] = s;    // -dir edge of the neighbour
}

}  // namespace

cudaError_t launch_edge_sad(const float* d_im, int m, int n, int o, int g, float* d_sad, cudaStream_t s) {
    const int64_t sz1 = (int64_t)(m / g) * (n / g) * (o / g);
    const int64_t total = 3 * sz1;
    const int threads = 128;
    k_edge_sad<<<(unsigned)((total + threads - 1) / threads), threads, 0, s>>>(d_im, d_sad, m, n, o, g);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace deeds
