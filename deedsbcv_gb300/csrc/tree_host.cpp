// Host half of the MST stage: image statistics, Prim's algorithm and the
// belief-propagation schedule (src/primsMST.h:52-223, src/regularisation.h:145-169).
//
// Prim's algorithm is a priority-queue walk whose tie handling decides the tree
// whenever two candidate edges have bit-equal weights, which is common on CT
// backgrounds (weights are exp() of block SADs quantised to float).  To give
// the reference's tree node for node, it runs on the host with the same binary
// heap algorithm as the reference's std::push_heap / std::pop_heap, over the same
// edge sequence and comparison.  The edge SADs come from the GPU (deeds_mst_edges_dev); the
// statistics are sequential float sums as in the reference.  Compiled with
// -ffp-contract=off.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <thread>
#include <vector>

#include "tree_host.h"

namespace deeds {

// The reference's statistics (src/primsMST.h:101-110) are sequential float sums:
// mean += im[i], then var = float(double(var) + double(im[i]-mean)^2) -- a double
// rounding per step.  Both are evaluated exactly, in parallel chunks, using one
// property of such chains.  Let every value of a chain lie in one binade
// [2^(e-1), 2^e) (or its negative), where floats are the multiples of u =
// 2^(e-24), at least one u inside its ends.  Then each step is "add the
// increment exactly, round to the u-grid" (for the variance first to the double
// grid u*2^-29, then to the u-grid), and shifting the running value by an even
// multiple of u shifts every later value by the same amount: rounding to a grid
// commutes with shifts by grid points, and ties to even see the same parity.
// So a chunk is run (the reference arithmetic, step for step) from two guessed
// start values in the binade of the estimated true start, one u apart; when the
// true start is known, the trajectory whose start differs from it by an even
// multiple of u gives the chunk's end by the same shift, provided both it and
// its shifted copy stay inside the binade.  Chunks where the guess or the check
// fails (the first ones, while the sum crosses binades quickly, or non-finite
// data) are replayed from the true start sequentially.  The result is always the
// reference's.
namespace {

struct Traj {
    float end, lo, hi;  // last, smallest and largest value of the trajectory (start included)
    bool exact;         // the variance's fast steps matched the reference formula
};

// binade exponent (|v| in [2^(e-1), 2^e)) and its grid step u; false for 0, tiny or non-finite v
bool binade(float v, int& e, float& u) {
    if (!std::isfinite(v) || std::fabs(v) < 0x1p-100f) return false;
    std::frexp(v, &e);
    u = std::ldexp(1.0f, e - 24);
    return true;
}

// every value of [lo, hi] (shifted by d) strictly inside the binade e of sign neg
bool inside(float lo, float hi, float d, int e, float u, bool neg) {
    const double l = (double)lo + d, h = (double)hi + d;  // exact: small integers of u
    const double inner = std::ldexp(1.0, e - 1) + u, outer = std::ldexp(1.0, e) - 2.0 * u;
    return neg ? (l >= -outer && h <= -inner) : (l >= inner && h <= outer);
}

inline float mean_step(float v, float x) { return v + x; }
inline float var_step(float v, float d) { return (float)((double)v + (double)d * (double)d); }

Traj run_mean(const float* x, size_t lo, size_t hi, float v) {
    Traj t{v, v, v, true};
    for (size_t i = lo; i < hi; i++) {
        v = mean_step(v, x[i]);
        t.lo = std::min(t.lo, v);
        t.hi = std::max(t.hi, v);
    }
    t.end = v;
    return t;
}

// Two independent mean trajectories in one loop (their dependency chains overlap;
// the running extremes use four accumulators each so that they add no chain).
void run_mean2(const float* x, size_t lo, size_t hi, float va, float vb, Traj& ta, Traj& tb) {
    float alo[4] = {va, va, va, va}, ahi[4] = {va, va, va, va};
    float blo[4] = {vb, vb, vb, vb}, bhi[4] = {vb, vb, vb, vb};
    size_t i = lo;
    for (; i + 4 <= hi; i += 4)
        for (int j = 0; j < 4; j++) {
            va = mean_step(va, x[i + j]);
            vb = mean_step(vb, x[i + j]);
            alo[j] = std::min(alo[j], va);
            ahi[j] = std::max(ahi[j], va);
            blo[j] = std::min(blo[j], vb);
            bhi[j] = std::max(bhi[j], vb);
        }
    for (; i < hi; i++) {
        va = mean_step(va, x[i]);
        vb = mean_step(vb, x[i]);
        alo[0] = std::min(alo[0], va);
        ahi[0] = std::max(ahi[0], va);
        blo[0] = std::min(blo[0], vb);
        bhi[0] = std::max(bhi[0], vb);
    }
    ta = Traj{va, std::min(std::min(alo[0], alo[1]), std::min(alo[2], alo[3])),
              std::max(std::max(ahi[0], ahi[1]), std::max(ahi[2], ahi[3])), true};
    tb = Traj{vb, std::min(std::min(blo[0], blo[1]), std::min(blo[2], blo[3])),
              std::max(std::max(bhi[0], bhi[1]), std::max(bhi[2], bhi[3])), true};
}

// The variance chain with fmaf (one rounding, shorter dependency) checked against
// the reference's double-rounded step; the exact formula when they ever differ.
// The chain never decreases (it adds squares): its extremes are start and end.
Traj run_var(const float* x, float mean, size_t lo, size_t hi, float v0) {
    float v = v0;
    unsigned bad = 0;
    for (size_t i = lo; i < hi; i++) {
        const float d = x[i] - mean;
        const float nv = std::fma(d, d, v);
        bad |= (unsigned)(nv != var_step(v, d));
        v = nv;
    }
    if (bad) {
        v = v0;
        for (size_t i = lo; i < hi; i++) v = var_step(v, x[i] - mean);
    }
    return Traj{v, v0, v, true};
}

// Two variance trajectories in one loop, each as run_var.  The chain never
// decreases (it adds squares), so its extremes are its start and end.
void run_var2(const float* x, float mean, size_t lo, size_t hi, float va, float vb, Traj& ta, Traj& tb) {
    const float a0 = va, b0 = vb;
    unsigned bad = 0;
    for (size_t i = lo; i < hi; i++) {
        const float d = x[i] - mean;
        const float na = std::fma(d, d, va), nb = std::fma(d, d, vb);
        bad |= (unsigned)(na != var_step(va, d)) | (unsigned)(nb != var_step(vb, d));
        va = na;
        vb = nb;
    }
    if (bad) {
        ta = run_var(x, mean, lo, hi, a0);
        tb = run_var(x, mean, lo, hi, b0);
        return;
    }
    ta = Traj{va, a0, va, true};
    tb = Traj{vb, b0, vb, true};
}

// The chunks of the two chains and their start estimates.
struct ChainPlan {
    size_t nch;
    std::vector<size_t> bnd;
    std::vector<double> sum_x, sum_x2;  // per chunk (estimates only: any order of addition)
};

template <class Fn>
void parallel_chunks(size_t nch, int threads, Fn fn) {
    const int nt = std::max(1, std::min<int>(threads, (int)nch));
    std::vector<std::thread> th;
    for (int t = 1; t < nt; t++) th.emplace_back(fn, nch * t / nt, nch * (t + 1) / nt);
    fn((size_t)0, nch / nt);
    for (auto& h : th) h.join();
}

// One chain over x: kind 0 = mean sum, 1 = variance sum around `mean`; `est[c]`
// estimates the chain's value at the start of chunk c.
float chain_sum(const float* x, const ChainPlan& P, int kind, float mean, const std::vector<float>& est,
                int threads) {
    const size_t nch = P.nch;
    const std::vector<size_t>& bnd = P.bnd;
    std::vector<float> alt(nch, 0.0f);
    std::vector<Traj> ta(nch), tb(nch);
    std::vector<char> spec(nch, 0);
    parallel_chunks(nch, threads, [&](size_t c0, size_t c1) {
        for (size_t c = c0; c < c1; c++) {
            int e;
            float u;
            if (!binade(est[c], e, u)) continue;
            // a second start one u away, in the same binade
            const float g2 = std::fabs(est[c] + u) < std::ldexp(1.0f, e) ? est[c] + u : est[c] - u;
            alt[c] = g2;
            if (kind == 0) run_mean2(x, bnd[c], bnd[c + 1], est[c], g2, ta[c], tb[c]);
            else run_var2(x, mean, bnd[c], bnd[c + 1], est[c], g2, ta[c], tb[c]);
            spec[c] = 1;
        }
    });
    // the true chain, chunk by chunk
    float v = 0.0f;
    for (size_t c = 0; c < nch; c++) {
        int e, eg;
        float u, ug;
        bool done = false;
        if (spec[c] && binade(v, e, u) && binade(est[c], eg, ug) && e == eg && std::signbit(v) == std::signbit(est[c])) {
            const double k = ((double)v - (double)est[c]) / u;  // exact integer
            const bool even = std::fmod(std::fabs(k), 2.0) == 0.0;
            const Traj& t = even ? ta[c] : tb[c];
            const float start = even ? est[c] : alt[c];
            const float d = v - start;  // exact: both multiples of u in one binade
            const bool neg = std::signbit(v);
            if (t.exact && inside(t.lo, t.hi, 0.0f, e, u, neg) && inside(t.lo, t.hi, d, e, u, neg)) {
                v = t.end + d;  // exact: a multiple of u inside the binade
                done = true;
            }
        }
        if (!done) v = kind == 0 ? run_mean(x, bnd[c], bnd[c + 1], v).end : run_var(x, mean, bnd[c], bnd[c + 1], v).end;
    }
    return v;
}

}  // namespace

void image_stats(const float* im, size_t sz, float* mean_out, float* std_out) {
    const int threads = sz >= ((size_t)1 << 20) ? std::max(1, (int)std::thread::hardware_concurrency() / 2) : 1;
    ChainPlan P;
    P.nch = std::max<size_t>(1, std::min<size_t>(256, sz / 32768));
    P.bnd.resize(P.nch + 1);
    for (size_t c = 0; c <= P.nch; c++) P.bnd[c] = sz * c / P.nch;
    P.sum_x.assign(P.nch, 0.0);
    P.sum_x2.assign(P.nch, 0.0);
    // one pass for both chains' estimates: per chunk sum of x and of x^2 (four
    // independent accumulators each)
    parallel_chunks(P.nch, threads, [&](size_t c0, size_t c1) {
        for (size_t c = c0; c < c1; c++) {
            double s[4] = {0, 0, 0, 0}, q[4] = {0, 0, 0, 0};
            size_t i = P.bnd[c];
            for (; i + 4 <= P.bnd[c + 1]; i += 4)
                for (int j = 0; j < 4; j++) {
                    const double v = im[i + j];
                    s[j] += v;
                    q[j] += v * v;
                }
            for (; i < P.bnd[c + 1]; i++) {
                s[0] += im[i];
                q[0] += (double)im[i] * im[i];
            }
            P.sum_x[c] = (s[0] + s[1]) + (s[2] + s[3]);
            P.sum_x2[c] = (q[0] + q[1]) + (q[2] + q[3]);
        }
    });
    std::vector<float> est(P.nch);
    double pre = 0.0, total = 0.0;
    for (size_t c = 0; c < P.nch; c++) total += P.sum_x[c];
    for (size_t c = 0; c < P.nch; c++) {
        est[c] = (float)pre;
        pre += P.sum_x[c];
    }
    float mean = chain_sum(im, P, 0, 0.0f, est, threads);
    mean /= (float)sz;
    // sum over a chunk of (x - m)^2 = sum x^2 - 2 m sum x + n m^2, m the estimated mean
    const double m = total / (double)sz;
    pre = 0.0;
    for (size_t c = 0; c < P.nch; c++) {
        est[c] = (float)pre;
        const double n = (double)(P.bnd[c + 1] - P.bnd[c]);
        pre += std::max(0.0, P.sum_x2[c] - 2.0 * m * P.sum_x[c] + n * m * m);
    }
    const float var = chain_sum(im, P, 1, mean, est, threads);
    *mean_out = mean;
    *std_out = std::sqrt(var / (float)sz);
}

#ifndef DEEDS_HEAP_LOOKAHEAD
#define DEEDS_HEAP_LOOKAHEAD 4  // levels ahead of the sift-down that are prefetched (two lines)
#endif

namespace {
// A candidate edge: weight and (from vertex, direction).  The reference stores
// the weight as double; comparing the float is the same order, and the heap
// only sees comparison results, so the pop order (ties included) is unchanged
// while the element shrinks to 8 bytes.
struct QueuedEdge {
    float weight;
    uint32_t from_dir;  // from * 8 + nb
};

// The reference's priority queue is a binary max-heap under an inverted
// comparison (src/primsMST.h:24-26) driven by std::push_heap / std::pop_heap.
// Which of several equal-weight edges pops first depends on the exact sequence
// of element moves, so this heap performs the same algorithm step for step:
//   push: append, then move the new element up while its parent compares
//         "less" (parent weight > new weight);
//   pop:  take the root; move a hole from the root down to a leaf, always into
//         the child that compares greater (the lighter edge; the right child
//         unless it is strictly heavier than the left one), including the
//         single-child case at the end of an even-length heap; then place the
//         former last element at the hole and move it up as in push.
// It differs only in how the descent is evaluated: branch-free, two levels per
// step while both are full levels (the four grandchildren are compared in the
// same step as the two children, which halves the dependent load-compare chain),
// and with the path prefetched ahead; that changes timing, not order.
class EdgeHeap {
  public:
    explicit EdgeHeap(size_t reserve) { grow(std::max<size_t>(reserve, 64)); }
    bool empty() const { return n_ == 0; }
    void push(QueuedEdge e) {
        if (n_ == cap_) grow(2 * cap_);
        a_[n_++] = e;
        sift_up(n_ - 1, 0, e);
    }
    QueuedEdge pop() {
        const QueuedEdge top = a_[0];
        const QueuedEdge last = a_[--n_];
        const size_t len = n_;
        if (len == 0) return top;
        QueuedEdge* d = a_;
        size_t hole = 0;
        const size_t lim = (len - 1) / 2;
        // Two levels per step while the deeper of the two possible children still
        // has children below it (both levels are then full descents).  Choices as
        // the single-level step below: right (c + 1) unless it is strictly heavier.
        while (2 * hole + 2 < lim) {
            {
                const size_t first = ((hole + 1) << DEEDS_HEAP_LOOKAHEAD) - 1;
                if (first < len) {
                    __builtin_prefetch(d + first);
                    if (first + 8 < len) __builtin_prefetch(d + first + 8);
                }
            }
            const size_t c = 2 * hole + 1, gc = 4 * hole + 3;
            const float lw = d[c].weight, rw = d[c + 1].weight;
            const float g0 = d[gc].weight, g1 = d[gc + 1].weight, g2 = d[gc + 2].weight, g3 = d[gc + 3].weight;
            const size_t p1 = (size_t)!(rw > lw);
            const size_t p2a = (size_t)!(g1 > g0), p2b = (size_t)!(g3 > g2);
            const size_t p2 = p2a ^ ((p2a ^ p2b) & (0 - p1));  // p1 ? p2b : p2a, without a branch
            const size_t c1 = c + p1, c2 = gc + 2 * p1 + p2;
            d[hole] = d[c1];
            d[c1] = d[c2];
            hole = c2;
        }
        size_t child = hole;
        while (child < lim) {
            // The descendants of the hole k levels down are the 2^k contiguous
            // entries from 2^k (hole + 1) - 1: prefetch those DEEDS_HEAP_LOOKAHEAD
            // levels ahead so the misses of a root-to-leaf walk overlap.
            {
                const size_t k = DEEDS_HEAP_LOOKAHEAD;
                const size_t first = ((hole + 1) << k) - 1;
                if (first < len) {
                    __builtin_prefetch(d + first);
                    if (k >= 4 && first + 8 < len) __builtin_prefetch(d + first + 8);
                }
            }
            child = 2 * (child + 1);  // right child
            const size_t gc = 2 * child + 1;
            if (gc < len) __builtin_prefetch(d + gc);
            if (gc - 2 < len) __builtin_prefetch(d + gc - 2);
            // the right child wins unless it is strictly heavier than the left one
            child -= (size_t)(d[child].weight > d[child - 1].weight);
            d[hole] = d[child];
            hole = child;
        }
        if ((len & 1) == 0 && child == (len - 2) / 2) {
            child = 2 * (child + 1);
            d[hole] = d[child - 1];
            hole = child - 1;
        }
        sift_up(hole, 0, last);
        return top;
    }

  private:
    // Storage with entry 1 on a 64-byte boundary: the siblings 2i+1, 2i+2 that
    // every sift-down level compares then share one cache line.
    void grow(size_t cap) {
        std::unique_ptr<QueuedEdge[]> mem(new QueuedEdge[cap + 16]);
        const uintptr_t b = reinterpret_cast<uintptr_t>(mem.get() + 1);
        QueuedEdge* a = mem.get() + ((64 - (b & 63)) & 63) / sizeof(QueuedEdge);
        if (n_) std::memcpy(a, a_, n_ * sizeof(QueuedEdge));
        mem_ = std::move(mem);
        a_ = a;
        cap_ = cap;
    }
    void sift_up(size_t hole, size_t top, QueuedEdge v) {
        QueuedEdge* d = a_;
        size_t parent = (hole - 1) / 2;
        while (hole > top && d[parent].weight > v.weight) {
            d[hole] = d[parent];
            hole = parent;
            parent = (hole - 1) / 2;
        }
        d[hole] = v;
    }
    std::unique_ptr<QueuedEdge[]> mem_;
    QueuedEdge* a_ = nullptr;
    size_t n_ = 0, cap_ = 0;
};
}  // namespace

namespace {

// Undirected grid edges are numbered 3 v + axis: axis 0 joins v and v + m1 (+x),
// 1 joins v and v + 1 (+y), 2 joins v and v + m1 n1 (+z).  `w` holds the
// reference's weight of each directed edge, vertex-major (w[v*6 + nb]); both
// directions of an edge carry the same weight (one block SAD).
inline float edge_weight(const float* w, int id) {
    static const int plus_dir[3] = {1, 3, 5};
    return w[(size_t)(id / 3) * 6 + plus_dir[id % 3]];
}

// Monotone map of a float to an unsigned key (ascending floats, ascending keys).
inline uint32_t float_key(float f) {
    uint32_t b;
    std::memcpy(&b, &f, 4);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
inline float key_float(uint32_t k) {
    const uint32_t b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    float f;
    std::memcpy(&f, &b, 4);
    return f;
}

// Kruskal's view of the minimum spanning trees of the grid.  Edges are taken in
// weight order, all edges of one weight w as a group.  The components of the
// edges lighter than w are the same for every spanning tree of minimum weight,
// and each such tree contains a spanning forest of the group's "useful" edges
// (those joining two different components), with the same number r of edges.
// When the useful edges form a forest themselves (k useful edges = r), every
// minimum tree contains all of them; otherwise the group is ambiguous and the
// trees differ only in the forest they pick from it, independently per group.
// So Prim's tree (the reference's) = the forced edges + Prim's picks in the
// ambiguous groups, and with no ambiguous group it is this tree outright.
struct MstGroups {
    std::vector<int> forced;       // tree edges of unambiguous groups
    std::vector<int> amb_of_edge;  // [3 sz] ambiguous group of a useful edge, -1 otherwise
    std::vector<int> amb_rank;     // per ambiguous group: edges every minimum tree takes from it
};

// False when a weight is NaN (the order is then the heap's own business).
bool mst_groups(const float* w, int m1, int n1, int o1, MstGroups& G) {
    const int sz = m1 * n1 * o1, mn1 = m1 * n1;
    std::vector<uint64_t> a, b;
    a.reserve((size_t)3 * sz);
    for (int v = 0; v < sz; v++) {
        const int k = v / mn1, rem = v - k * mn1, j = rem / m1, i = rem - j * m1;
        const bool has[3] = {j + 1 < n1, i + 1 < m1, k + 1 < o1};
        for (int ax = 0; ax < 3; ax++) {
            if (!has[ax]) continue;
            const float f = edge_weight(w, 3 * v + ax);
            if (std::isnan(f)) return false;
            a.push_back((uint64_t)float_key(f) << 32 | (uint32_t)(3 * v + ax));
        }
    }
    // LSD radix sort on the 32-bit key (three passes of 11 bits)
    b.resize(a.size());
    for (int pass = 0; pass < 3; pass++) {
        const int shift = 32 + 11 * pass;
        std::vector<size_t> cnt(2049, 0);
        for (uint64_t x : a) cnt[((x >> shift) & 2047u) + 1]++;
        for (int d = 0; d < 2048; d++) cnt[d + 1] += cnt[d];
        for (uint64_t x : a) b[cnt[(x >> shift) & 2047u]++] = x;
        a.swap(b);
    }
    // union-find: union by size, path halving
    std::vector<int> par(sz), size(sz, 1);
    for (int v = 0; v < sz; v++) par[v] = v;
    auto find = [&](int x) {
        while (par[x] != x) {
            par[x] = par[par[x]];
            x = par[x];
        }
        return x;
    };
    auto unite = [&](int rp, int rq) {
        if (size[rp] < size[rq]) std::swap(rp, rq);
        par[rq] = rp;
        size[rp] += size[rq];
    };
    auto ends = [&](int id, int& p, int& q) {
        const int v = id / 3, ax = id % 3;
        p = v;
        q = v + (ax == 0 ? m1 : ax == 1 ? 1 : mn1);
    };
    G.forced.clear();
    G.forced.reserve(sz);
    G.amb_rank.clear();
    G.amb_of_edge.assign((size_t)3 * sz, -1);
    std::vector<int> useful;
    size_t s = 0;
    while (s < a.size()) {
        const uint32_t key = (uint32_t)(a[s] >> 32);
        const float f = key_float(key);
        size_t e = s + 1;
        while (e < a.size() && ((uint32_t)(a[e] >> 32) == key || key_float((uint32_t)(a[e] >> 32)) == f)) e++;
        if (e == s + 1) {  // a weight of its own: never ambiguous
            const int id = (int)(uint32_t)a[s];
            int p, q;
            ends(id, p, q);
            const int rp = find(p), rq = find(q);
            if (rp != rq) {
                unite(rp, rq);
                G.forced.push_back(id);
            }
            s = e;
            continue;
        }
        useful.clear();
        for (size_t t = s; t < e; t++) {
            int p, q;
            ends((int)(uint32_t)a[t], p, q);
            if (find(p) != find(q)) useful.push_back((int)(uint32_t)a[t]);
        }
        const size_t first = G.forced.size();
        for (int id : useful) {
            int p, q;
            ends(id, p, q);
            const int rp = find(p), rq = find(q);
            if (rp != rq) {
                unite(rp, rq);
                G.forced.push_back(id);
            }
        }
        const int r = (int)(G.forced.size() - first);
        if ((size_t)r != useful.size()) {  // a cycle among the useful edges: Prim decides
            G.forced.resize(first);
            const int gi = (int)G.amb_rank.size();
            for (int id : useful) G.amb_of_edge[id] = gi;
            G.amb_rank.push_back(r);
        }
        s = e;
    }
    return true;
}

std::atomic<long long> g_mst_counts[4];  // trees without ambiguity, trees with, Prim steps run, Prim steps of a full run

}  // namespace

void mst_path_counts(long long out[4]) {
    for (int i = 0; i < 4; i++) out[i] = g_mst_counts[i].load();
}

void prims_from_sad(const float* sad, float stddev, int m1, int n1, int o1, int g, int* ordered, int* parents,
                    float* edgemst) {
    const int sz = m1 * n1 * o1;
    // -exp(-(sad/g^3) / (2 std)) in float, as edgecost2weight() (src/primsMST.h:48-50, :112-117);
    // stored vertex-major (w[v*6 + nb]): the six pushes of an added vertex read one
    // line; -1 for a direction that leaves the grid.  The two directions of an edge
    // normally have one SAD (computed once from the image), so one weight: where
    // the mirror entry is already evaluated it is reused.
    std::unique_ptr<float[]> w(new float[(size_t)sz * 6]);
    const float g3 = (float)std::pow((double)g, 3.0);
    const float twostd = 2.0f * stddev;
    const int mn1 = m1 * n1;
    // neighbour offsets in the reference's direction order -x,+x,-y,+y,-z,+z (src/primsMST.h:70-72)
    const int off[6] = {-m1, m1, -1, 1, -mn1, mn1};
    // All six entries of the vertices of z-slabs [k0, k1), in vertex order; false if
    // some edge whose lower end lies there has two different SADs.
    auto weights = [&](int k0, int k1) {
        bool sym = true;
        for (int k = k0; k < k1; k++)
            for (int j = 0; j < n1; j++)
                for (int i = 0; i < m1; i++) {
                    const int v = i + j * m1 + k * mn1;
                    const bool has[6] = {j > 0, j + 1 < n1, i > 0, i + 1 < m1, k > 0, k + 1 < o1};
                    float* wv = &w[(size_t)v * 6];
                    for (int nb = 0; nb < 6; nb++) {
                        if (!has[nb]) {
                            wv[nb] = -1.0f;
                            continue;
                        }
                        const float sv = sad[(size_t)nb * sz + v];
                        const int u = v + off[nb];
                        const float su = sad[(size_t)(nb ^ 1) * sz + u];  // the mirror direction's SAD
                        const bool same = std::memcmp(&sv, &su, 4) == 0;
                        if (nb & 1) {
                            sym = sym && same;
                            wv[nb] = -std::exp(-(sv / g3) / twostd);
                        } else {
                            // the lower neighbour u was evaluated before v when it lies in these slabs
                            const bool done = nb != 4 || k > k0;
                            wv[nb] = same && done ? w[(size_t)u * 6 + nb + 1] : -std::exp(-(sv / g3) / twostd);
                        }
                    }
                }
        return sym;
    };
    // Large trees: the slabs are evaluated in blocks, from the root's block outward,
    // by helper threads while the walk starts at the root; the walk waits for a
    // block's flag before it reads the weights of a vertex in it (only the vertex it
    // adds), the tie analysis and the edge weights at the end wait for all of them.
    const int root = m1 / 2 + (n1 / 2) * m1 + (o1 / 2) * m1 * n1;
    const bool lazy = sz >= (1 << 16);
    const int spb = lazy ? std::max(1, 8192 / mn1) : o1;  // slabs per block
    const int nblk = (o1 + spb - 1) / spb;
    std::unique_ptr<std::atomic<int>[]> blk_ready(new std::atomic<int>[nblk]);
    std::vector<char> blk_sym(nblk, 1);
    for (int b = 0; b < nblk; b++) blk_ready[b].store(0, std::memory_order_relaxed);
    std::vector<int> blk_order;
    {
        const int br = (o1 / 2) / spb;
        blk_order.push_back(br);
        for (int d = 1; (int)blk_order.size() < nblk; d++) {
            if (br + d < nblk) blk_order.push_back(br + d);
            if (br - d >= 0) blk_order.push_back(br - d);
        }
    }
    std::atomic<int> blk_next{0};
    auto helper = [&]() {
        for (;;) {
            const int t = blk_next.fetch_add(1);
            if (t >= nblk) return;
            const int b = blk_order[t];
            blk_sym[b] = weights(b * spb, std::min(o1, (b + 1) * spb));
            blk_ready[b].store(1, std::memory_order_release);
        }
    };
    auto wait_block = [&](int b) {
        while (!blk_ready[b].load(std::memory_order_acquire)) std::this_thread::yield();
    };
    std::vector<std::thread> helpers;
    struct JoinHelpers {
        std::vector<std::thread>& t;
        ~JoinHelpers() {
            for (auto& x : t)
                if (x.joinable()) x.join();
        }
    } join_helpers{helpers};
    if (lazy) {
        try {
            for (int t = 0; t < 4; t++) helpers.emplace_back(helper);
        } catch (...) {
            helper();  // no threads: the rest here
        }
    } else {
        helper();
    }
    auto all_weights = [&]() {
        bool sym = true;
        for (int b = 0; b < nblk; b++) {
            wait_block(b);
            sym = sym && blk_sym[b];
        }
        return sym;
    };
    std::vector<int> depth(sz, 0);
    for (int v = 0; v < sz; v++) parents[v] = -1;

    // The tree Prim's walk would give (src/primsMST.h:120-165): Kruskal's forced
    // edges, plus the walk itself only until it has made its picks in every
    // ambiguous tie group (its heap decides those ties); no walk when no group is
    // ambiguous.  A NaN weight, or an edge whose two directions differ: the whole
    // walk.  The tie-group analysis runs on its own thread while the walk starts;
    // the walk records its picks until the analysis is in, then counts them.
    MstGroups G;
    std::atomic<int> g_state{sz > 1 ? 0 : 2};  // 0 running, 1 grouped, 2 no grouping
    auto analyse = [&]() {
        bool ok = false;
        try {
            // every weight is in; an edge whose two directions differ: no grouping
            ok = all_weights() && mst_groups(w.get(), m1, n1, o1, G);
        } catch (...) {
            ok = false;
        }
        g_state.store(ok ? 1 : 2, std::memory_order_release);
    };
    // its own thread for large trees only: a registration builds ten trees at once,
    // and the long walks of the finest two should not share cores with helpers
    std::thread grouper;
    if (g_state.load() == 0) {
        if (sz >= (1 << 16)) grouper = std::thread(analyse);
        else analyse();
    }
    struct JoinAtExit {
        std::thread& t;
        ~JoinAtExit() { if (t.joinable()) t.join(); }
    } join_grouper{grouper};
    std::vector<int> picks;           // edges the walk took before the analysis was in
    std::vector<int> tree_edges;
    std::vector<int> taken;
    bool grouped = false;
    int pending = -2;  // ambiguous groups still open; -1: full walk; -2: analysis not in yet
    // the analysis is in: forced edges, and the walk's picks so far counted per group
    auto settle = [&]() {
        grouped = g_state.load(std::memory_order_acquire) == 1;
        if (!grouped) {
            pending = -1;
            return;
        }
        tree_edges = G.forced;
        taken.assign(G.amb_rank.size(), 0);
        pending = (int)G.amb_rank.size();
        for (int id : picks) {
            const int gi = G.amb_of_edge[id];
            if (gi >= 0) {
                tree_edges.push_back(id);
                if (++taken[gi] == G.amb_rank[gi]) pending--;
            }
        }
    };
    long long steps = 0;
    // the walk's vertices; their parents and depths from the walk are final
    std::vector<uint8_t> in_tree(sz, 0);
    in_tree[root] = 1;
    int walked = 1;
    {
        EdgeHeap heap((size_t)sz * 3);
        int last = root;
        picks.reserve(sz);
        for (int added = 1; added < sz && pending != 0; added++) {
            if (pending == -2 && (added & 1023) == 0 && g_state.load(std::memory_order_acquire) != 0) {
                settle();
                if (pending == 0) break;
            }
            // push the new vertex's edges to its in-grid neighbours, in direction order
            const int k = last / mn1, rem = last - k * mn1, j = rem / m1, i = rem - j * m1;
            if (lazy) wait_block(k / spb);  // the added vertex's weights
            const bool ok[6] = {j > 0, j + 1 < n1, i > 0, i + 1 < m1, k > 0, k + 1 < o1};
            for (int nb = 0; nb < 6; nb++)
                if (ok[nb]) heap.push(QueuedEdge{w[(size_t)last * 6 + nb], (uint32_t)last * 8u + (uint32_t)nb});
            int from = -1, to = -1;
            uint32_t dir = 0;
            while (to < 0) {
                if (heap.empty()) throw std::runtime_error("Prim: candidate heap exhausted (disconnected grid)");
                const QueuedEdge e = heap.pop();
                const int ef = (int)(e.from_dir >> 3), et = ef + off[e.from_dir & 7u];
                const bool a = in_tree[ef], b = in_tree[et];
                if (a != b) {
                    from = a ? ef : et;
                    to = a ? et : ef;
                    dir = e.from_dir;
                }
            }
            in_tree[to] = 1;
            walked++;
            depth[to] = depth[from] + 1;
            parents[to] = from;
            last = to;
            steps++;
            if (pending != -1) {
                // the undirected id of the edge just added: from its pushing end and direction
                const int ef = (int)(dir >> 3), nb = (int)(dir & 7u);
                const int id = (nb & 1) ? 3 * ef + nb / 2 : 3 * (ef + off[nb]) + nb / 2;
                if (pending == -2) {
                    picks.push_back(id);
                } else {
                    const int gi = G.amb_of_edge[id];
                    if (gi >= 0) {
                        tree_edges.push_back(id);
                        if (++taken[gi] == G.amb_rank[gi]) pending--;
                    }
                }
            }
        }
    }
    if (grouper.joinable()) grouper.join();
    if (pending == -2) settle();  // the walk ended first (small trees)
    g_mst_counts[grouped && G.amb_rank.empty() ? 0 : 1]++;
    // a unique tree's walk only ran while the analysis was out: it counts no steps
    g_mst_counts[2] += grouped && G.amb_rank.empty() ? 0 : steps;
    g_mst_counts[3] += sz - 1;
    if (grouped) {
        // Parents and depths of the assembled tree.  Every edge the walk added is a
        // tree edge and no other tree edge joins two walked vertices (it would close
        // a cycle with the walk's tree), so the walked vertices keep the parents and
        // depths the walk gave them, and the remaining tree edges (those with an end
        // outside the walk) attach the other vertices as subtrees of walked ones:
        // breadth-first from those attachment edges.
        if ((int)tree_edges.size() != sz - 1) throw std::runtime_error("MST assembly: wrong edge count");
        if (walked < sz) {
            // the tree's edges as a bitmap over the undirected edge ids
            std::vector<uint64_t> is_tree(((size_t)3 * sz + 63) / 64, 0);
            for (int id : tree_edges) is_tree[(size_t)id >> 6] |= 1ull << (id & 63);
            auto tree_nb = [&](int v, int nb, int& u) {  // v's tree neighbour in direction nb, if any
                const int k = v / mn1, rem = v - k * mn1, j = rem / m1, i = rem - j * m1;
                const bool in_grid = nb == 0 ? j > 0 : nb == 1 ? j + 1 < n1 : nb == 2 ? i > 0 : nb == 3 ? i + 1 < m1
                                   : nb == 4 ? k > 0 : k + 1 < o1;
                if (!in_grid) return false;
                u = v + off[nb];
                const int id = (nb & 1) ? 3 * v + nb / 2 : 3 * u + nb / 2;
                return ((is_tree[(size_t)id >> 6] >> (id & 63)) & 1ull) != 0;
            };
            // attachment edges (one end walked, which is the parent), then breadth-first
            std::vector<int> queue;
            queue.reserve((size_t)(sz - walked));
            std::vector<uint8_t> walked_at_end(in_tree);
            for (int v = 0; v < sz; v++) {
                if (walked_at_end[v]) continue;
                for (int nb = 0; nb < 6; nb++) {
                    int u;
                    if (tree_nb(v, nb, u) && walked_at_end[u]) {
                        in_tree[v] = 1;
                        parents[v] = u;
                        depth[v] = depth[u] + 1;
                        queue.push_back(v);
                        break;
                    }
                }
            }
            for (size_t qh = 0; qh < queue.size(); qh++) {
                const int v = queue[qh];
                for (int nb = 0; nb < 6; nb++) {
                    int u;
                    if (!tree_nb(v, nb, u) || in_tree[u]) continue;
                    in_tree[u] = 1;
                    parents[u] = v;
                    depth[u] = depth[v] + 1;
                    queue.push_back(u);
                }
            }
            if ((int)queue.size() != sz - walked) throw std::runtime_error("MST assembly: tree does not span the grid");
        }
    }
    // breadth-level order, stable in node id (src/primsMST.h:166-190)
    int maxd = 0;
    for (int v = 0; v < sz; v++) maxd = std::max(maxd, depth[v]);
    std::vector<int> start(maxd + 2, 0);
    for (int v = 0; v < sz; v++) start[depth[v] + 1]++;
    for (int l = 1; l <= maxd + 1; l++) start[l] += start[l - 1];
    for (int v = 0; v < sz; v++) ordered[start[depth[v]]++] = v;
    all_weights();  // (the analysis waited for them already, unless it never ran)
    // weight of each child's edge to its parent (src/primsMST.h:198-211)
    // The reference forms the neighbour index without a bounds check here, so on
    // grids with a dimension of 1 an out-of-grid direction can alias the parent;
    // the same unchecked index (last match wins) is used.  That index is the child's
    // plus the direction's offset, so the direction is found from parent - child.
    for (int c = 0; c < sz; c++) {
        float e = 0.0f;
        if (c != root) {
            const int d = parents[c] - c;
            int sel = -1;
            for (int nb = 0; nb < 6; nb++) {  // masks: no data-dependent branch
                const int mk = -(int)(d == off[nb]);
                sel = (sel & ~mk) | (nb & mk);
            }
            if (sel >= 0) e = -w[(size_t)c * 6 + sel];
        }
        edgemst[c] = e;
    }
}

void build_schedule(const int* ordered, const int* parents, int sz, TreeSchedule& s, bool levels_by_id) {
    // children per node in ordering order (ordering is breadth-level, so a
    // parent's children appear in the order the reference adds them); every node
    // but ordered[0] is a child, so the counts can be taken in node order
    s.child_ptr.assign(sz + 1, 0);
    const int r0 = sz > 0 ? ordered[0] : -1;
    for (int v = 0; v < sz; v++)
        if (v != r0) s.child_ptr[parents[v] + 1]++;
    for (int v = 0; v < sz; v++) s.child_ptr[v + 1] += s.child_ptr[v];
    s.children.assign(sz > 0 ? sz - 1 : 0, 0);
    {
        std::vector<int> fill(s.child_ptr.begin(), s.child_ptr.end() - 1);
        if (levels_by_id) {
            // a node's children share a breadth level, ordered there by node id:
            // node order gives each parent its children in ordering order
            for (int v = 0; v < sz; v++)
                if (v != r0) s.children[fill[parents[v]]++] = v;
        } else {
            for (int t = 1; t < sz; t++) {
                const int c = ordered[t];
                s.children[fill[parents[c]]++] = c;
            }
        }
    }
    // leaves, deepest first (long chains start early), and the heavy children:
    // subtree heights bottom-up (ordering is breadth-level, so every child is
    // visited before its parent; a node visited with height 0 has no children);
    // in reverse order '>=' keeps the first child of equal height.  A node's
    // height, heavy child and chain slot share one 16-byte record.
    struct Aux {
        int height, heavy, slot, pad;
    };
    std::vector<Aux> aux((size_t)sz, Aux{0, -1, 0, 0});
    s.leaves.clear();
    s.leaves.reserve((size_t)sz);
    for (int t = sz - 1; t >= 1; t--) {
        const int c = ordered[t], p = parents[c];
        const int h = aux[c].height;
        if (h == 0) s.leaves.push_back(c);
        const int hc = h + 1, hp = aux[p].height, kp = aux[p].heavy;
        const bool take = hc >= hp;  // selects: the outcome is data-dependent
        aux[p].height = take ? hc : hp;
        aux[p].heavy = take ? c : kp;
    }
    // Chains in ordering order of their starts, each from its start down through
    // heavy children to a leaf.  A heavy child's subtree is one level lower than
    // its parent's, so a chain starting at v holds height[v] + 1 nodes: the chains'
    // ranges follow from the starts alone, and a node's slot is its parent's + 1
    // (no walk along the chain).
    s.chain_ptr.clear();
    s.chain_nodes.assign((size_t)sz, 0);
    {
        int next = 0;
        for (int t = 0; t < sz; t++) {
            const int v = ordered[t];
            int k;
            if (t > 0 && aux[parents[v]].heavy == v) {  // continues its parent's chain
                k = aux[parents[v]].slot + 1;
            } else {
                s.chain_ptr.push_back(next);
                k = next;
                next += aux[v].height + 1;
            }
            aux[v].slot = k;
            s.chain_nodes[(size_t)k] = v;
        }
        s.chain_ptr.push_back(next);
        if (next != sz) throw std::runtime_error("tree schedule: chains do not cover the tree");
    }
}

}  // namespace deeds
