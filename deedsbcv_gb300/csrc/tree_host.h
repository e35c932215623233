// Host-side MST construction and BP schedule (see tree_host.cpp).
#pragma once
#include <cstddef>
#include <vector>

namespace deeds {

struct TreeSchedule {
    std::vector<int> child_ptr;    // [sz+1] CSR of children per node
    std::vector<int> children;     // in MST ordering order
    std::vector<int> leaves;       // nodes without children (root excluded), deepest first
    // Heavy-path chains for the downward pass: from each chain start (the root,
    // and every child that is not its parent's heavy child) down through heavy
    // children (the child with the deepest subtree, the first such on ties) to a
    // leaf; chains in breadth order of their starts, every node in exactly one.
    std::vector<int> chain_ptr;    // [n_chains+1] ranges into chain_nodes
    std::vector<int> chain_nodes;  // [sz]
};

void image_stats(const float* im, size_t sz, float* mean_out, float* std_out);
void prims_from_sad(const float* sad, float stddev, int m1, int n1, int o1, int g, int* ordered, int* parents,
                    float* edgemst);
// levels_by_id: `ordered` is breadth-level order with every level in increasing
// node id (prims_from_sad's ordering); any order where parents precede their
// children otherwise.  Both give the same schedule for such an ordering.
void build_schedule(const int* ordered, const int* parents, int sz, TreeSchedule& s, bool levels_by_id = false);
// Process-wide counts of the MST constructions: trees whose minimum spanning tree
// is unique (no Prim walk needed), trees with ambiguous ties (a Prim walk until
// its tie picks are made, or all of it when a weight is NaN), Prim steps walked
// for the latter (the walk starts while the tie analysis runs; for a unique tree
// those steps are discarded and not counted), and the steps full walks of the
// same trees would take.
void mst_path_counts(long long out[4]);

}  // namespace deeds
