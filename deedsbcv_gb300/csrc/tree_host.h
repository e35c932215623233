// Host-side MST construction and BP schedule (see tree_host.cpp).
#pragma once
#include <cstddef>
#include <vector>

namespace deeds {

struct TreeSchedule {
    int n_levels = 0;
    std::vector<int> depth;        // per node
    std::vector<int> level_start;  // [n_levels+1] ranges into ordered
    std::vector<int> up_nodes;     // upward work items (parents), deepest first
    std::vector<int> child_ptr;    // [n_up+1]
    std::vector<int> children;     // per item, in ordering order
    std::vector<int> wait_idx;     // per node: its item index or -1
};

void image_stats(const float* im, size_t sz, float* mean_out, float* std_out);
void prims_from_sad(const float* sad, float stddev, int m1, int n1, int o1, int g, int* ordered, int* parents,
                    float* edgemst);
void build_schedule(const int* ordered, const int* parents, int sz, TreeSchedule& s);

}  // namespace deeds
