// Host half of the MST stage: image statistics, Prim's algorithm and the
// belief-propagation schedule (src/primsMST.h:52-223, src/regularisation.h:145-169).
//
// Prim's algorithm is a priority-queue walk whose tie handling decides the tree
// whenever two candidate edges have bit-equal weights, which is common on CT
// backgrounds (weights are exp() of block SADs quantised to float).  To give
// the reference's tree node for node, it runs on the host with the same binary
// heap discipline (std::push_heap / std::pop_heap over the same edge sequence and
// comparator).  The edge SADs come from the GPU (deeds_mst_edges_dev); the
// statistics are sequential float sums as in the reference.  Compiled with
// -ffp-contract=off.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "tree_host.h"

namespace deeds {

void image_stats(const float* im, size_t sz, float* mean_out, float* std_out) {
    float mean = 0.0f;
    for (size_t i = 0; i < sz; i++) mean += im[i];
    mean /= (float)sz;
    float var = 0.0f;
    for (size_t i = 0; i < sz; i++) {
        const double d = (double)(im[i] - mean);
        var = (float)((double)var + d * d);  // float += pow(float,2) in double
    }
    *mean_out = mean;
    *std_out = std::sqrt(var / (float)sz);
}

namespace {
// A candidate edge: weight and (from vertex, direction).  The reference stores
// the weight as double; comparing the float is the same order, and the heap
// algorithm only sees comparison results, so the pop order (ties included) is
// unchanged while the element shrinks to 8 bytes.
struct QueuedEdge {
    float weight;
    uint32_t from_dir;  // from * 8 + nb
    // std heaps are max-heaps: inverting '<' pops the lightest edge first
    bool operator<(const QueuedEdge& b) const { return weight > b.weight; }
};
}  // namespace

void prims_from_sad(const float* sad, float stddev, int m1, int n1, int o1, int g, int* ordered, int* parents,
                    float* edgemst) {
    const int sz = m1 * n1 * o1;
    // -exp(-(sad/g^3) / (2 std)) in float, as edgecost2weight() (src/primsMST.h:48-50, :112-117)
    std::vector<float> w((size_t)sz * 6);
    const float g3 = (float)std::pow((double)g, 3.0);
    const float twostd = 2.0f * stddev;
    for (size_t e = 0; e < (size_t)sz * 6; e++) w[e] = -std::exp(-(sad[e] / g3) / twostd);
    const int stride_n = m1, stride_o = m1 * n1;
    // neighbour of v in direction nb (-x,+x,-y,+y,-z,+z) or -1
    auto nbr = [&](int v, int nb) -> int {
        const int k = v / stride_o, j = (v / m1) % n1, i = v % m1;
        switch (nb) {
            case 0: return j > 0 ? v - stride_n : -1;
            case 1: return j + 1 < n1 ? v + stride_n : -1;
            case 2: return i > 0 ? v - 1 : -1;
            case 3: return i + 1 < m1 ? v + 1 : -1;
            case 4: return k > 0 ? v - stride_o : -1;
            default: return k + 1 < o1 ? v + stride_o : -1;
        }
    };
    std::vector<QueuedEdge> heap;
    heap.reserve((size_t)sz * 3);
    std::vector<uint8_t> in_tree(sz, 0);
    std::vector<int> depth(sz, 0);
    for (int v = 0; v < sz; v++) parents[v] = -1;
    const int root = m1 / 2 + (n1 / 2) * m1 + (o1 / 2) * m1 * n1;
    in_tree[root] = 1;
    int last = root;
    for (int added = 1; added < sz; added++) {
        for (int nb = 0; nb < 6; nb++) {
            const int v = nbr(last, nb);
            if (v >= 0) {
                heap.push_back(QueuedEdge{w[(size_t)nb * sz + last], (uint32_t)last * 8u + (uint32_t)nb});
                std::push_heap(heap.begin(), heap.end());
            }
        }
        int from = -1, to = -1;
        while (to < 0) {
            const QueuedEdge e = heap.front();
            std::pop_heap(heap.begin(), heap.end());
            heap.pop_back();
            const int ef = (int)(e.from_dir >> 3), et = nbr(ef, (int)(e.from_dir & 7u));
            const bool a = in_tree[ef], b = in_tree[et];
            if (a != b) { from = a ? ef : et; to = a ? et : ef; }
        }
        in_tree[to] = 1;
        depth[to] = depth[from] + 1;
        parents[to] = from;
        last = to;
    }
    // breadth-level order, stable in node id (src/primsMST.h:166-190)
    int maxd = 0;
    for (int v = 0; v < sz; v++) maxd = std::max(maxd, depth[v]);
    std::vector<int> start(maxd + 2, 0);
    for (int v = 0; v < sz; v++) start[depth[v] + 1]++;
    for (int l = 1; l <= maxd + 1; l++) start[l] += start[l - 1];
    for (int v = 0; v < sz; v++) ordered[start[depth[v]]++] = v;
    // weight of each child's edge to its parent (src/primsMST.h:198-211)
    for (int v = 0; v < sz; v++) edgemst[v] = 0.0f;
    for (int t = 1; t < sz; t++) {
        const int c = ordered[t], p = parents[c];
        for (int nb = 0; nb < 6; nb++)
            if (nbr(c, nb) == p) edgemst[c] = -w[(size_t)nb * sz + c];
    }
}

void build_schedule(const int* ordered, const int* parents, int sz, TreeSchedule& s) {
    // breadth levels from the ordering (src/regularisation.h:145-169)
    std::vector<int> depth(sz, 0), pos(sz, 0);
    for (int t = 0; t < sz; t++) pos[ordered[t]] = t;
    for (int t = 1; t < sz; t++) depth[ordered[t]] = depth[parents[ordered[t]]] + 1;
    int maxd = 0;
    for (int v = 0; v < sz; v++) maxd = std::max(maxd, depth[v]);
    s.n_levels = maxd + 1;
    s.level_start.assign(s.n_levels + 1, 0);
    for (int v = 0; v < sz; v++) s.level_start[depth[v] + 1]++;
    for (int l = 1; l <= s.n_levels; l++) s.level_start[l] += s.level_start[l - 1];
    s.max_width = 0;
    for (int l = 0; l < s.n_levels; l++) s.max_width = std::max(s.max_width, s.level_start[l + 1] - s.level_start[l]);
    // children per node in ordering order (ordering is breadth-level, so a
    // parent's children appear in the order the reference adds them)
    s.child_ptr.assign(sz + 1, 0);
    for (int t = 1; t < sz; t++) s.child_ptr[parents[ordered[t]] + 1]++;
    for (int v = 0; v < sz; v++) s.child_ptr[v + 1] += s.child_ptr[v];
    s.children.assign(sz > 0 ? sz - 1 : 0, 0);
    std::vector<int> fill(s.child_ptr.begin(), s.child_ptr.end() - 1);
    for (int t = 1; t < sz; t++) {
        const int c = ordered[t];
        s.children[fill[parents[c]]++] = c;
    }
    // leaves, deepest first (long chains start early)
    s.leaves.clear();
    for (int t = sz - 1; t >= 1; t--) {
        const int v = ordered[t];
        if (s.child_ptr[v + 1] == s.child_ptr[v]) s.leaves.push_back(v);
    }
    s.parent_pos.assign(sz, 0);
    for (int t = 1; t < sz; t++) s.parent_pos[t] = pos[parents[ordered[t]]];
}

}  // namespace deeds
