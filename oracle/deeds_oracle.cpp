// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// A CPU restatement of the deedsBCV dense-registration hot path, used as the
// checker for the GPU library's parity tests, by __graft_entry__.smoke(), and
// as bench.py's timed CPU baseline when the reference binaries are absent.
// Nothing in the product (deedsbcv_gb300/) links, loads or calls this file.
//
// Parity pin: every function below is compared bit-for-bit with the unmodified
// reference sources (compiled by oracle/Makefile into oracle/_ref/) on the
// committed golden vectors in tests/golden/ (made by tests/golden/make_golden.py).
//
// Numerics.  The reference relies on IEEE float evaluation in source order with
// no FMA contraction (ISO C++ mode) and on implicit promotion to double in a few
// places (interpolation weights, alpha scaling, consistent-mapping update).  The
// expressions below keep exactly those types and that order; the build uses
// -ffp-contract=off.  Each function cites the reference file:line it restates.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <vector>

namespace {

inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Trilinear 8-term blend with the reference's mixed float/double evaluation
// (src/transformations.h:15-22, src/dataCostD.h:288-295).  Products whose
// operands are all float stay float; anything touching the literal 1.0 is double;
// the running sum is double, left to right, rounded to float once at the end.
inline float blend8(float dx, float dy, float dz, float c000, float c100, float c010, float c001,
                    float c110, float c101, float c011, float c111) {
    // cXYZ: X = y+1 step, Y = x+1 step, Z = z+1 step
    double acc = (1.0 - dx) * (1.0 - dy) * (1.0 - dz) * (double)c000;
    acc = acc + (1.0 - dx) * (double)dy * (1.0 - dz) * (double)c100;
    acc = acc + (double)dx * (1.0 - dy) * (1.0 - dz) * (double)c010;
    acc = acc + (1.0 - dx) * (1.0 - dy) * (double)dz * (double)c001;
    acc = acc + (double)(dx * dy) * (1.0 - dz) * (double)c110;
    acc = acc + (1.0 - dx) * (double)dy * (double)dz * (double)c101;
    acc = acc + (double)dx * (1.0 - dy) * (double)dz * (double)c011;
    acc = acc + (double)(dx * dy * dz * c111);
    return (float)acc;
}

// Sample `vol` (m2 x n2 x o2, i fastest) at integer corner (y,x,z) with
// clamp-to-edge and fractional offsets; restates the body of interp3
// (src/transformations.h:9-22) after the floor() split.
inline float sample_trilinear(const float* vol, int m2, int n2, int o2, int y, int x, int z,
                              float dx, float dy, float dz) {
    const int y0 = clampi(y, 0, m2 - 1), y1 = clampi(y + 1, 0, m2 - 1);
    const int x0 = clampi(x, 0, n2 - 1), x1 = clampi(x + 1, 0, n2 - 1);
    const int z0 = clampi(z, 0, o2 - 1), z1 = clampi(z + 1, 0, o2 - 1);
    const size_t s1 = (size_t)m2, s2 = (size_t)m2 * n2;
    return blend8(dx, dy, dz,
                  vol[y0 + x0 * s1 + z0 * s2], vol[y1 + x0 * s1 + z0 * s2],
                  vol[y0 + x1 * s1 + z0 * s2], vol[y0 + x0 * s1 + z1 * s2],
                  vol[y1 + x1 * s1 + z0 * s2], vol[y1 + x0 * s1 + z1 * s2],
                  vol[y0 + x1 * s1 + z1 * s2], vol[y1 + x1 * s1 + z1 * s2]);
}

// One separable box-filter pass along an axis of length L and element stride
// `stride`, over `nlines` lines whose first elements are given by line_base().
// Sequential running sum, then the windowed difference with the reference's
// edge rules (src/MINDSSCbox.h:9-29 for the first axis; :31-51, :53-73 repeat
// it for the other two axes).  `a` holds the input and is left holding the
// prefix sums; the filtered line is written to `b`.
template <class BaseFn>
void box_pass(float* a, float* b, int L, size_t stride, size_t nlines, int r, BaseFn line_base) {
#pragma omp parallel for schedule(static)
    for (long long ln = 0; ln < (long long)nlines; ln++) {
        const size_t base = line_base((size_t)ln);
        float* p = a + base;
        float* q = b + base;
        for (int i = 1; i < L; i++) p[i * stride] += p[(i - 1) * stride];
        for (int i = 0; i < r + 1; i++) q[i * stride] = p[(i + r) * stride];
        for (int i = r + 1; i < L - r; i++) q[i * stride] = p[(i + r) * stride] - p[(i - r - 1) * stride];
        for (int i = L - r; i < L; i++) q[i * stride] = p[(L - 1) * stride] - p[(i - r - 1) * stride];
    }
}

// 3-D box sum of half-width r, in place on `vol` (src/MINDSSCbox.h:2-76).
void box_filter3(float* vol, int m, int n, int o, int r) {
    const size_t sz = (size_t)m * n * o;
    std::vector<float> t1(vol, vol + sz), t2(sz);
    // i-axis: lines indexed by (j,k)
    box_pass(t1.data(), t2.data(), m, 1, (size_t)n * o, r, [&](size_t ln) { return ln * m; });
    // j-axis: lines indexed by (i,k)
    box_pass(t2.data(), t1.data(), n, (size_t)m, (size_t)m * o, r,
             [&](size_t ln) { return (ln % m) + (ln / m) * (size_t)m * n; });
    // k-axis: lines indexed by (i,j)
    box_pass(t1.data(), vol, o, (size_t)m * n, (size_t)m * n, r, [&](size_t ln) { return ln; });
}

// Six self-similarity shift vectors and the twelve (channel, offset) pairs of
// MIND-SSC (src/MINDSSCbox.h:110-112, :132-140).
struct MindLayout {
    int dx[6], dy[6], dz[6];
    int sx[12], sy[12], sz[12], ch[12];
    explicit MindLayout(int q) {
        const int DX[6] = {1, 1, -1, 0, 1, 0}, DY[6] = {1, -1, 0, -1, 0, 1}, DZ[6] = {0, 0, 1, 1, 1, 1};
        const int SX[12] = {-1, 0, -1, 0, 0, 1, 0, 0, 0, -1, 0, 0};
        const int SY[12] = {0, -1, 0, 1, 0, 0, 0, 1, 0, 0, 0, -1};
        const int SZ[12] = {0, 0, 0, 0, -1, 0, -1, 0, -1, 0, -1, 0};
        for (int l = 0; l < 6; l++) { dx[l] = DX[l] * q; dy[l] = DY[l] * q; dz[l] = DZ[l] * q; }
        for (int l = 0; l < 12; l++) { sx[l] = SX[l] * q; sy[l] = SY[l] * q; sz[l] = SZ[l] * q; ch[l] = l / 2; }
    }
};

}  // namespace

extern "C" {

// floor(0.5*Q+1) patch radius per level (src/deedsBCV0.cpp:183-186).
int orc_mind_step(int quant) { return (int)std::floor(0.5f * (float)quant + 1.0f); }

// The five quantisation thresholds -log((c+1.5)/6) in float (src/MINDSSCbox.h:177-180).
void orc_mind_thresholds(float* out5) {
    for (int c = 0; c < 5; c++) out5[c] = -std::log(((float)c + 1.5f) / 6);
}

// MIND-SSC descriptor -> one 64-bit code per voxel (src/MINDSSCbox.h:127-232,
// distances :104-124, imshift :79-90, boxfilter :2-76).
void orc_descriptor(uint64_t* codes, const float* im, int m, int n, int o, int qs) {
    const size_t sz = (size_t)m * n * o;
    const MindLayout L(qs);
    std::vector<float> d(sz * 6);
    for (int l = 0; l < 6; l++) {
        float* dl = d.data() + (size_t)l * sz;
        // shifted squared difference; out-of-volume shifts read the voxel itself
#pragma omp parallel for schedule(static)
        for (int k = 0; k < o; k++)
            for (int j = 0; j < n; j++)
                for (int i = 0; i < m; i++) {
                    const size_t p = i + (size_t)j * m + (size_t)k * m * n;
                    const int ii = i + L.dy[l], jj = j + L.dx[l], kk = k + L.dz[l];
                    float s = (ii >= 0 && ii < m && jj >= 0 && jj < n && kk >= 0 && kk < o)
                                  ? im[ii + (size_t)jj * m + (size_t)kk * m * n] : im[p];
                    float diff = s - im[p];
                    dl[p] = diff * diff;
                }
        box_filter3(dl, m, n, o, qs);
    }
    float thr[5];
    orc_mind_thresholds(thr);
    static const unsigned therm[6] = {0, 1, 3, 7, 15, 31};
#pragma omp parallel for schedule(static)
    for (int k = 0; k < o; k++)
        for (int j = 0; j < n; j++)
            for (int i = 0; i < m; i++) {
                const size_t p = i + (size_t)j * m + (size_t)k * m * n;
                float v[12];
                for (int l = 0; l < 12; l++) {
                    const int ii = i + L.sy[l], jj = j + L.sx[l], kk = k + L.sz[l];
                    const float* dl = d.data() + (size_t)L.ch[l] * sz;
                    v[l] = (ii >= 0 && ii < m && jj >= 0 && jj < n && kk >= 0 && kk < o)
                               ? dl[ii + (size_t)jj * m + (size_t)kk * m * n] : dl[p];
                }
                float mn = v[0];
                for (int l = 1; l < 12; l++) mn = v[l] < mn ? v[l] : mn;
                float noise = 0.0f;
                for (int l = 0; l < 12; l++) { v[l] -= mn; noise += v[l]; }
                noise = std::max(noise / 12.0f, 1e-6f);
                uint64_t code = 0;
                for (int l = 0; l < 12; l++) {
                    const float x = v[l] / noise;
                    int lvl = 0;
                    for (int c = 0; c < 5; c++) lvl += thr[c] > x ? 1 : 0;
                    code |= (uint64_t)therm[lvl] << (5 * l);
                }
                codes[p] = code;
            }
}

// Sampling strides of the cost volume for RAND_SAMPLES=1 (src/dataCostD.h:141-155).
void orc_datacost_skips(int g, int* sy, int* sx, int* sz) {
    *sy = 1; *sx = 1; *sz = 1;
    if (g > 4) { *sx = 2; *sz = 2; }
}

// Per-sample cost scale alpha1 = float(0.5*(g/(alpha*q))/maxsamp) (src/dataCostD.h:157-163).
float orc_datacost_alpha1(int g, float q, float alpha) {
    int sy, sx, sz;
    orc_datacost_skips(g, &sy, &sx, &sz);
    const float maxsamp = std::ceil((float)g / (float)sx) * std::ceil((float)g / (float)sz) *
                          std::ceil((float)g / (float)sy);
    const float alphai = (float)g / (alpha * q);
    return (float)(0.5 * alphai / (float)maxsamp);
}

// Hamming cost volume cost[node][label] (src/dataCostD.h:108-210).  The moving
// codes are padded by q*hw with clamp-to-edge (:124-138).
void orc_data_cost(const uint64_t* F, const uint64_t* M, float* cost, int m, int n, int o, int g,
                   int hw, int q, float alpha) {
    const int len = 2 * hw + 1, len3 = len * len * len;
    const int m1 = m / g, n1 = n / g, o1 = o / g;
    const int pad = q * hw;
    const int mp = m + 2 * pad, np = n + 2 * pad, op = o + 2 * pad;
    std::vector<uint64_t> Mp((size_t)mp * np * op);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < op; k++)
        for (int j = 0; j < np; j++)
            for (int i = 0; i < mp; i++)
                Mp[i + (size_t)j * mp + (size_t)k * mp * np] =
                    M[clampi(i - pad, 0, m - 1) + (size_t)clampi(j - pad, 0, n - 1) * m +
                      (size_t)clampi(k - pad, 0, o - 1) * m * n];
    int sy, sx, sz;
    orc_datacost_skips(g, &sy, &sx, &sz);
    const float alpha1 = orc_datacost_alpha1(g, (float)q, alpha);
#pragma omp parallel for schedule(static)
    for (int z = 0; z < o1; z++)
        for (int x = 0; x < n1; x++)
            for (int y = 0; y < m1; y++) {
                const size_t node = y + (size_t)x * m1 + (size_t)z * m1 * n1;
                for (int l = 0; l < len3; l++) {
                    const int lz = l / (len * len), lx = (l / len) % len, ly = l % len;
                    const size_t shift = (size_t)(y * g + ly * q) + (size_t)(x * g + lx * q) * mp +
                                         (size_t)(z * g + lz * q) * mp * np;
                    int acc = 0;
                    for (int k = 0; k < g; k += sz)
                        for (int j = 0; j < g; j += sx)
                            for (int i = 0; i < g; i += sy) {
                                const uint64_t a = F[(y * g + i) + (size_t)(x * g + j) * m + (size_t)(z * g + k) * m * n];
                                const uint64_t b = Mp[shift + i + (size_t)j * mp + (size_t)k * mp * np];
                                acc += __builtin_popcountll(a ^ b);
                            }
                    cost[node * len3 + l] = (float)acc * alpha1;
                }
            }
}

// Intensity statistics used for the MST edge weights: sequential float mean and
// sqrt of the double-promoted squared deviations (src/primsMST.h:101-110).
void orc_image_stats(const float* im, size_t sz, float* mean_out, float* std_out) {
    float mean = 0.0f;
    for (size_t i = 0; i < sz; i++) mean += im[i];
    mean /= (float)sz;
    float var = 0.0f;
    for (size_t i = 0; i < sz; i++) {
        const double dv = (double)(im[i] - mean);
        var = (float)((double)var + dv * dv);
    }
    *mean_out = mean;
    *std_out = std::sqrt(var / (float)sz);
}

// Block sum of absolute differences between a grid node's g^3 block and its
// neighbour's block, summed in k,j,i order (src/primsMST.h:75-100).  Output layout
// edge[nb*sz1 + node], nb in the reference's order (-x,+x,-y,+y,-z,+z); missing
// neighbours get 0.
void orc_edge_sad(const float* im, float* edge, int m, int n, int o, int g) {
    const int m1 = m / g, n1 = n / g, o1 = o / g;
    const size_t sz1 = (size_t)m1 * n1 * o1;
    const int ddx[6] = {-1, 1, 0, 0, 0, 0}, ddy[6] = {0, 0, -1, 1, 0, 0}, ddz[6] = {0, 0, 0, 0, -1, 1};
#pragma omp parallel for schedule(static)
    for (int k = 0; k < o1; k++)
        for (int j = 0; j < n1; j++)
            for (int i = 0; i < m1; i++) {
                const size_t node = i + (size_t)j * m1 + (size_t)k * m1 * n1;
                for (int nb = 0; nb < 6; nb++) {
                    const int ii = i + ddy[nb], jj = j + ddx[nb], kk = k + ddz[nb];
                    float s = 0.0f;
                    if (ii >= 0 && ii < m1 && jj >= 0 && jj < n1 && kk >= 0 && kk < o1) {
                        for (int c = 0; c < g; c++)
                            for (int b = 0; b < g; b++)
                                for (int a = 0; a < g; a++) {
                                    const float p = im[(i * g + a) + (size_t)(j * g + b) * m + (size_t)(k * g + c) * m * n];
                                    const float r = im[(ii * g + a) + (size_t)(jj * g + b) * m + (size_t)(kk * g + c) * m * n];
                                    s += std::fabs(p - r);
                                }
                    }
                    edge[nb * sz1 + node] = s;
                }
            }
}

// Prim's MST on the 6-connected control grid from per-edge SADs, then the
// breadth-level ordering and per-child edge weights (src/primsMST.h:52-223).
// `sad` is orc_edge_sad's output; `stdim` the image standard deviation.
void orc_prims_from_sad(const float* sad, float stdim, int m1, int n1, int o1, int g,
                        int* ordered, int* parents, float* edgemst) {
    const int sz = m1 * n1 * o1;
    const int ddx[6] = {-1, 1, 0, 0, 0, 0}, ddy[6] = {0, 0, -1, 1, 0, 0}, ddz[6] = {0, 0, 0, 0, -1, 1};
    // edge weight -exp(-(sad/g^3)/(2 std)) in float (src/primsMST.h:112-117)
    std::vector<float> w((size_t)sz * 6);
    const float g3 = (float)std::pow(g, 3);
    const float twostd = 2.0f * stdim;
    for (size_t e = 0; e < (size_t)sz * 6; e++) {
        const float c = sad[e] / g3;
        w[e] = -std::exp(-c / twostd);
    }
    auto nbr = [&](int v, int nb) -> int {
        const int k = v / (m1 * n1), j = (v - k * m1 * n1) / m1, i = v - k * m1 * n1 - j * m1;
        const int ii = i + ddy[nb], jj = j + ddx[nb], kk = k + ddz[nb];
        if (ii < 0 || ii >= m1 || jj < 0 || jj >= n1 || kk < 0 || kk >= o1) return -1;
        return ii + jj * m1 + kk * m1 * n1;
    };
    // Heap entries ordered so that std::push_heap/pop_heap yield the lightest
    // edge first, with the standard library's tie handling (src/primsMST.h:7-26).
    struct HeapEdge {
        double weight; int from; int to;
        bool operator<(const HeapEdge& b) const { return weight > b.weight; }
    };
    std::vector<HeapEdge> heap;
    std::vector<char> in_tree(sz, 0);
    std::vector<int> level(sz, 0);
    for (int v = 0; v < sz; v++) parents[v] = -1;
    const int root = m1 / 2 + (n1 / 2) * m1 + (o1 / 2) * m1 * n1;
    in_tree[root] = 1;
    level[root] = 0;
    int last = root;
    for (int added = 0; added < sz - 1; added++) {
        for (int nb = 0; nb < 6; nb++) {
            const int v = nbr(last, nb);
            if (v >= 0) {
                heap.push_back(HeapEdge{(double)w[(size_t)nb * sz + last], last, v});
                std::push_heap(heap.begin(), heap.end());
            }
        }
        int from = -1, to = -1;
        while (to < 0) {
            const HeapEdge e = heap.front();
            std::pop_heap(heap.begin(), heap.end());
            heap.pop_back();
            const bool a = in_tree[e.from], b = in_tree[e.to];
            if (a != b) {
                from = a ? e.from : e.to;
                to = a ? e.to : e.from;
            }
        }
        in_tree[to] = 1;
        level[to] = level[from] + 1;
        parents[to] = from;
        last = to;
    }
    // counting sort by depth, stable in node id (src/primsMST.h:166-190)
    int maxlev = 0;
    for (int v = 0; v < sz; v++) maxlev = std::max(maxlev, level[v]);
    std::vector<int> start(maxlev + 2, 0);
    for (int v = 0; v < sz; v++) start[level[v] + 1]++;
    for (int l = 1; l <= maxlev + 1; l++) start[l] += start[l - 1];
    for (int v = 0; v < sz; v++) ordered[start[level[v]]++] = v;
    // weight of the edge to the parent, exp(-c) in (0,1] (src/primsMST.h:198-211)
    // the neighbour index is formed without a bounds check, as the reference does
    // (last match wins; matters only on grids with a dimension of 1)
    for (int v = 0; v < sz; v++) edgemst[v] = 0.0f;
    for (int t = 1; t < sz; t++) {
        const int c = ordered[t], p = parents[c];
        const int k = c / (m1 * n1), j = (c - k * m1 * n1) / m1, i = c - k * m1 * n1 - j * m1;
        for (int nb = 0; nb < 6; nb++) {
            const int idx = i + ddy[nb] + (j + ddx[nb]) * m1 + (k + ddz[nb]) * m1 * n1;
            if (idx == p) edgemst[c] = -w[(size_t)nb * sz + c];
        }
    }
}

// primsGraph(im, ...) end to end (src/primsMST.h:52).
void orc_prims_graph(const float* im, int m, int n, int o, int g, int* ordered, int* parents, float* edgemst) {
    const int m1 = m / g, n1 = n / g, o1 = o / g;
    std::vector<float> sad((size_t)m1 * n1 * o1 * 6);
    orc_edge_sad(im, sad.data(), m, n, o, g);
    float mean, sd;
    orc_image_stats(im, (size_t)m * n * o, &mean, &sd);
    orc_prims_from_sad(sad.data(), sd, m1, n1, o1, g, ordered, parents, edgemst);
}

// Separable min-convolution of one node's len^3 costs with (d+offset)^2 per axis,
// first y (fastest), then x, then z; strict '<' keeps the first minimiser.
// In place on `row`; `arg[l]` receives the source label for parent label l
// (src/regularisation.h:6-113).
void orc_message_dt(float* row, short* arg, int len, float offx, float offy, float offz) {
    const int len2 = len * len, len3 = len2 * len;
    std::vector<float> a(len3), b(len3), zt(2 * len + 1);
    std::vector<int> ia(len3), ib(len3);
    auto parab = [&](float off) {
        for (int t = 0; t < 2 * len; t++) {
            const float d = (float)(t - len) + off;
            zt[t] = d * d;
        }
    };
    // y pass: row -> a
    parab(offy);
    for (int k = 0; k < len; k++)
        for (int j = 0; j < len; j++) {
            const int base = j * len + k * len2;
            for (int i = 0; i < len; i++) {
                float best = row[base] + zt[i + len];
                int bi = 0;
                for (int s = 0; s < len; s++) {
                    const float c = row[base + s] + zt[i - s + len];
                    if (c < best) { best = c; bi = s; }
                }
                a[base + i] = best;
                ia[base + i] = base + bi;
            }
        }
    // x pass: a -> b
    parab(offx);
    for (int k = 0; k < len; k++)
        for (int i = 0; i < len; i++) {
            const int base = i + k * len2;
            for (int j = 0; j < len; j++) {
                float best = a[base] + zt[j + len];
                int bj = 0;
                for (int s = 0; s < len; s++) {
                    const float c = a[base + s * len] + zt[j - s + len];
                    if (c < best) { best = c; bj = s; }
                }
                b[base + j * len] = best;
                ib[base + j * len] = ia[base + bj * len];
            }
        }
    // z pass: b -> row
    parab(offz);
    for (int j = 0; j < len; j++)
        for (int i = 0; i < len; i++) {
            const int base = i + j * len;
            for (int k = 0; k < len; k++) {
                float best = b[base] + zt[k + len];
                int bk = 0;
                for (int s = 0; s < len; s++) {
                    const float c = b[base + s * len2] + zt[k - s + len];
                    if (c < best) { best = c; bk = s; }
                }
                row[base + k * len2] = best;
                arg[base + k * len2] = (short)ib[base + bk * len2];
            }
        }
}

// Exact min-sum belief propagation on the MST (src/regularisation.h:115-303).
// `cost` is overwritten with the upward-pass state: each non-root row holds that
// node's outgoing message (after the distance transform), the root row its
// total.  Outputs the displacement u1 = label offset + u0 per node.  If
// `allinds_out` is non-null it receives the argmin tables (sz1*len3 shorts).
void orc_regularisation(float* cost, const float* u0, const float* v0, const float* w0,
                        float* u1, float* v1, float* w1, int m1, int n1, int o1, int hw, float q,
                        const int* ordered, const int* parents, const float* edgemst, short* allinds_out) {
    const int sz = m1 * n1 * o1;
    const int len = 2 * hw + 1, len3 = len * len * len;
    std::vector<short> own;
    short* allinds = allinds_out;
    if (!allinds) { own.resize((size_t)sz * len3); allinds = own.data(); }
    // depth of every node from the ordering (src/regularisation.h:145-169)
    std::vector<int> depth(sz, 0);
    for (int t = 1; t < sz; t++) depth[ordered[t]] = depth[parents[ordered[t]]] + 1;
    int maxlev = 1 + *std::max_element(depth.begin(), depth.end());
    std::vector<int> first(maxlev + 1, 0);
    for (int v = 0; v < sz; v++) first[depth[v] + 1]++;
    for (int l = 1; l <= maxlev; l++) first[l] += first[l - 1];
    // leaves to root, one breadth level at a time (src/regularisation.h:190-238)
    for (int lev = maxlev - 1; lev > 0; lev--) {
        const int b = first[lev], e = first[lev + 1];
        for (int t = b; t < e; t++) {
            const int c = ordered[t];
            for (int l = 0; l < len3; l++) cost[(size_t)c * len3 + l] *= edgemst[c];
        }
#pragma omp parallel for schedule(static)
        for (int t = b; t < e; t++) {
            const int c = ordered[t], p = parents[c];
            const float ox = (u0[p] - u0[c]) / q;
            const float oy = (v0[p] - v0[c]) / q;
            const float oz = (w0[p] - w0[c]) / q;
            orc_message_dt(cost + (size_t)c * len3, allinds + (size_t)c * len3, len, ox, oy, oz);
        }
        // parents accumulate (message - min) in ordering order
        for (int t = b; t < e; t++) {
            const int c = ordered[t], p = parents[c];
            const float* cr = cost + (size_t)c * len3;
            const float mn = *std::min_element(cr, cr + len3);
            float* pr = cost + (size_t)p * len3;
            for (int l = 0; l < len3; l++) pr[l] += (cr[l] - mn);
        }
    }
    // label -> displacement tables (src/regularisation.h:242-254)
    auto disp = [&](int l, float* dx, float* dy, float* dz) {
        const int i = l % len, j = (l / len) % len, k = l / (len * len);
        *dx = (float)(j - hw) * q; *dy = (float)(i - hw) * q; *dz = (float)(k - hw) * q;
    };
    std::vector<int> sel(sz);
    const int root = ordered[0];
    const float* rr = cost + (size_t)root * len3;
    int best = 0;
    float bv = rr[0];
    for (int l = 0; l < len3; l++) {
        if (rr[l] < bv) { bv = rr[l]; best = l; }
        allinds[(size_t)root * len3 + l] = (short)l;
    }
    float dx, dy, dz;
    sel[root] = best;
    disp(best, &dx, &dy, &dz);
    u1[root] = dx + u0[root]; v1[root] = dy + v0[root]; w1[root] = dz + w0[root];
    for (int t = 1; t < sz; t++) {
        const int c = ordered[t], p = parents[c];
        const int l = allinds[(size_t)c * len3 + sel[p]];
        sel[c] = l;
        disp(l, &dx, &dy, &dz);
        u1[c] = dx + u0[c]; v1[c] = dy + v0[c]; w1[c] = dz + w0[c];
    }
}

// interp3 (src/transformations.h:5-26): resample `in` (m2 x n2 x o2) at per-voxel
// coordinates (x=x1 along n, y=y1 along m, z=z1 along o) of an m x n x o output;
// with `relative` the coordinates are offsets from the voxel position.
void orc_interp3(float* out, const float* in, const float* x1, const float* y1, const float* z1,
                 int m, int n, int o, int m2, int n2, int o2, int relative) {
#pragma omp parallel for schedule(static)
    for (int k = 0; k < o; k++)
        for (int j = 0; j < n; j++)
            for (int i = 0; i < m; i++) {
                const size_t p = i + (size_t)j * m + (size_t)k * m * n;
                int x = (int)std::floor(x1[p]), y = (int)std::floor(y1[p]), z = (int)std::floor(z1[p]);
                const float dx = x1[p] - x, dy = y1[p] - y, dz = z1[p] - z;
                if (relative) { x += j; y += i; z += k; }
                out[p] = sample_trilinear(in, m2, n2, o2, y, x, z, dx, dy, dz);
            }
}

// upsampleDeformationsCL (src/transformations.h:245-279): grid (m2,n2,o2) field to
// (m,n,o) at coordinate index/scale with scale=(float)m/(float)m2.
void orc_upsample(float* u1, float* v1, float* w1, const float* u0, const float* v0, const float* w0,
                  int m, int n, int o, int m2, int n2, int o2) {
    const float sm = (float)m / (float)m2, sn = (float)n / (float)n2, so = (float)o / (float)o2;
    const size_t sz = (size_t)m * n * o;
    std::vector<float> xs(sz), ys(sz), zs(sz);
    for (int k = 0; k < o; k++)
        for (int j = 0; j < n; j++)
            for (int i = 0; i < m; i++) {
                const size_t p = i + (size_t)j * m + (size_t)k * m * n;
                xs[p] = j / sn; ys[p] = i / sm; zs[p] = k / so;
            }
    orc_interp3(u1, u0, xs.data(), ys.data(), zs.data(), m, n, o, m2, n2, o2, 0);
    orc_interp3(v1, v0, xs.data(), ys.data(), zs.data(), m, n, o, m2, n2, o2, 0);
    orc_interp3(w1, w0, xs.data(), ys.data(), zs.data(), m, n, o, m2, n2, o2, 0);
}

// Affine + dense-field trilinear warp, clamp-to-edge (src/dataCostD.h:267-298).
// X is the 16-float matrix with rows y,x,z at X[0..3], X[4..7], X[8..11].
void orc_warp_affine(float* out, const float* in, const float* X, const float* u, const float* v,
                     const float* w, int m, int n, int o) {
#pragma omp parallel for schedule(static)
    for (int k = 0; k < o; k++)
        for (int j = 0; j < n; j++)
            for (int i = 0; i < m; i++) {
                const size_t p = i + (size_t)j * m + (size_t)k * m * n;
                const float y1 = (float)i * X[0] + (float)j * X[1] + (float)k * X[2] + X[3] + v[p];
                const float x1 = (float)i * X[4] + (float)j * X[5] + (float)k * X[6] + X[7] + u[p];
                const float z1 = (float)i * X[8] + (float)j * X[9] + (float)k * X[10] + X[11] + w[p];
                const int x = (int)std::floor(x1), y = (int)std::floor(y1), z = (int)std::floor(z1);
                const float dx = x1 - x, dy = y1 - y, dz = z1 - z;
                out[p] = sample_trilinear(in, m, n, o, y, x, z, dx, dy, dz);
            }
}

// warpImageCL (src/dataCostD.h:213-239): the field is relative to the voxel position.
void orc_warp_image(float* out, const float* in, const float* u, const float* v, const float* w,
                    int m, int n, int o) {
    orc_interp3(out, in, u, v, w, m, n, o, m, n, o, 1);
}

// Nearest-neighbour label warp, round half away from zero (src/dataCostD.h:241-266).
void orc_warp_affine_s(short* out, const short* in, const float* X, const float* u, const float* v,
                       const float* w, int m, int n, int o) {
#pragma omp parallel for schedule(static)
    for (int k = 0; k < o; k++)
        for (int j = 0; j < n; j++)
            for (int i = 0; i < m; i++) {
                const size_t p = i + (size_t)j * m + (size_t)k * m * n;
                const float y1 = (float)i * X[0] + (float)j * X[1] + (float)k * X[2] + X[3] + v[p];
                const float x1 = (float)i * X[4] + (float)j * X[5] + (float)k * X[6] + X[7] + u[p];
                const float z1 = (float)i * X[8] + (float)j * X[9] + (float)k * X[10] + X[11] + w[p];
                const int x = (int)std::round(x1), y = (int)std::round(y1), z = (int)std::round(z1);
                out[p] = in[clampi(y, 0, m - 1) + (size_t)clampi(x, 0, n - 1) * m + (size_t)clampi(z, 0, o - 1) * m * n];
            }
}

// Inverse-consistent symmetrisation, 10 fixed-point iterations, in place on both
// grid fields (src/transformations.h:189-242).
void orc_consistent_mapping(float* u, float* v, float* w, float* u2, float* v2, float* w2,
                            int m, int n, int o, int g) {
    const float f1 = (float)(1.0 / (float)g);
    const size_t sz = (size_t)m * n * o;
    std::vector<float> us(sz), vs(sz), ws(sz), us2(sz), vs2(sz), ws2(sz);
    for (size_t i = 0; i < sz; i++) {
        us[i] = u[i] * f1; vs[i] = v[i] * f1; ws[i] = w[i] * f1;
        us2[i] = u2[i] * f1; vs2[i] = v2[i] * f1; ws2[i] = w2[i] * f1;
    }
    for (int it = 0; it < 10; it++) {
        orc_interp3(u, us2.data(), us.data(), vs.data(), ws.data(), m, n, o, m, n, o, 1);
        orc_interp3(v, vs2.data(), us.data(), vs.data(), ws.data(), m, n, o, m, n, o, 1);
        orc_interp3(w, ws2.data(), us.data(), vs.data(), ws.data(), m, n, o, m, n, o, 1);
        for (size_t i = 0; i < sz; i++) {
            u[i] = (float)(0.5 * us[i] - 0.5 * u[i]);
            v[i] = (float)(0.5 * vs[i] - 0.5 * v[i]);
            w[i] = (float)(0.5 * ws[i] - 0.5 * w[i]);
        }
        orc_interp3(u2, us.data(), us2.data(), vs2.data(), ws2.data(), m, n, o, m, n, o, 1);
        orc_interp3(v2, vs.data(), us2.data(), vs2.data(), ws2.data(), m, n, o, m, n, o, 1);
        orc_interp3(w2, ws.data(), us2.data(), vs2.data(), ws2.data(), m, n, o, m, n, o, 1);
        for (size_t i = 0; i < sz; i++) {
            u2[i] = (float)(0.5 * us2[i] - 0.5 * u2[i]);
            v2[i] = (float)(0.5 * vs2[i] - 0.5 * v2[i]);
            w2[i] = (float)(0.5 * ws2[i] - 0.5 * w2[i]);
        }
        for (size_t i = 0; i < sz; i++) {
            us[i] = u[i]; vs[i] = v[i]; ws[i] = w[i];
            us2[i] = u2[i]; vs2[i] = v2[i]; ws2[i] = w2[i];
        }
    }
    const float fg = (float)g;
    for (size_t i = 0; i < sz; i++) {
        u[i] *= fg; v[i] *= fg; w[i] *= fg;
        u2[i] *= fg; v2[i] *= fg; w2[i] *= fg;
    }
}

// Jacobian determinant statistics of a grid field (src/transformations.h:84-185):
// returns std(J); *neg_frac receives the fraction of J<0.
float orc_jacobian(const float* u, const float* v, const float* w, int m, int n, int o, int g, float* neg_frac) {
    const size_t sz = (size_t)m * n * o;
    const float f1 = (float)(1.0 / (float)g);
    const float gr[3] = {-0.5f, 0.0f, 0.5f};
    // central difference with replicate padding along axis 1=i, 2=j, 3=k (filter1 :30-54)
    auto deriv = [&](const float* in, std::vector<float>& out, int axis) {
        out.assign(sz, 0.0f);
        for (int k = 0; k < o; k++)
            for (int j = 0; j < n; j++)
                for (int i = 0; i < m; i++) {
                    const size_t p = i + (size_t)j * m + (size_t)k * m * n;
                    for (int f = 0; f < 3; f++) {
                        size_t q;
                        if (axis == 1) q = clampi(i + f - 1, 0, m - 1) + (size_t)j * m + (size_t)k * m * n;
                        else if (axis == 2) q = i + (size_t)clampi(j + f - 1, 0, n - 1) * m + (size_t)k * m * n;
                        else q = i + (size_t)j * m + (size_t)clampi(k + f - 1, 0, o - 1) * m * n;
                        out[p] += gr[f] * in[q];
                    }
                }
    };
    std::vector<float> J11, J12, J13, J21, J22, J23, J31, J32, J33;
    deriv(u, J11, 2); deriv(u, J12, 1); deriv(u, J13, 3);
    deriv(v, J21, 2); deriv(v, J22, 1); deriv(v, J23, 3);
    deriv(w, J31, 2); deriv(w, J32, 1); deriv(w, J33, 3);
    std::vector<float> Jd(sz);
    float jmean = 0.0f, neg = 0.0f, count = 0.0f;
    for (size_t p = 0; p < sz; p++) {
        const float a11 = (float)(J11[p] * f1 + 1.0), a12 = J12[p] * f1, a13 = J13[p] * f1;
        const float a21 = J21[p] * f1, a22 = (float)(J22[p] * f1 + 1.0), a23 = J23[p] * f1;
        const float a31 = J31[p] * f1, a32 = J32[p] * f1, a33 = (float)(J33[p] * f1 + 1.0);
        const float J = a11 * (a22 * a33 - a23 * a32) - a21 * (a12 * a33 - a13 * a32) + a31 * (a12 * a23 - a13 * a22);
        jmean += J;
        if (J < 0) neg++;
        count++;
        Jd[p] = J;
    }
    jmean /= (float)sz;
    float jstd = 0.0f;
    for (size_t p = 0; p < sz; p++) {
        const double d = (double)(Jd[p] - jmean);
        jstd = (float)((double)jstd + d * d);
    }
    jstd /= (float)(sz - 1);
    jstd = std::sqrt(jstd);
    if (neg_frac) *neg_frac = neg / count;
    return jstd;
}

// Full deeds nonlinear registration of one pair, mirroring the level loop of
// main() (src/deedsBCV0.cpp:183-349).  `fixed`/`moving` are intensities with the
// +1024 shift already applied (:139-144).  G/L/Q hold `levels` entries.
// Outputs: flow (3*sz1 of the last level, [u|v|w]), optional full-resolution
// field ux/vx/wx (may be null), optional warped moving image (may be null).
// Returns the last level's sz1.
int orc_register(const float* fixed, const float* moving, int m, int n, int o, const float* X,
                 int levels, const int* G, const int* Lr, const int* Q, float alpha,
                 float* flow, float* ux_out, float* vx_out, float* wx_out, float* warped_out, int verbose) {
    const size_t sz = (size_t)m * n * o;
    std::vector<int> mind_step(levels);
    for (int l = 0; l < levels; l++) mind_step[l] = orc_mind_step(Q[l]);
    std::vector<float> ux(sz, 0.0f), vx(sz, 0.0f), wx(sz, 0.0f), warped1(sz), warped0(sz);
    int m2 = m / G[0], n2 = n / G[0], o2 = o / G[0];
    std::vector<float> u1((size_t)m2 * n2 * o2, 0.0f), v1(u1), w1(u1), u1i(u1), v1i(u1), w1i(u1);
    orc_warp_affine(warped0.data(), moving, X, ux.data(), vx.data(), wx.data(), m, n, o);
    std::vector<uint64_t> mov_mind(sz), fix_mind(sz), warped_mind(sz);
    int m1 = m2, n1 = n2, o1 = o2;
    for (int level = 0; level < levels; level++) {
        const int q = Q[level];
        const int prev = mind_step[std::max(level - 1, 0)], curr = mind_step[level];
        if (level == 0 || prev != curr) {
            orc_descriptor(mov_mind.data(), warped0.data(), m, n, o, curr);
            orc_descriptor(fix_mind.data(), fixed, m, n, o, curr);
        }
        const int g = G[level], hw = Lr[level];
        const int len = 2 * hw + 1, len3 = len * len * len;
        m1 = m / g; n1 = n / g; o1 = o / g;
        const size_t sz1 = (size_t)m1 * n1 * o1;
        std::vector<float> cost(sz1 * len3), u0(sz1), v0(sz1), w0(sz1), edgemst(sz1);
        std::vector<int> ordered(sz1), parents(sz1);
        if (verbose) printf("level %d grid=%d %dx%dx%d hw=%d quant=%d\n", level, g, m1, n1, o1, hw, q);
        // forward
        orc_upsample(u0.data(), v0.data(), w0.data(), u1.data(), v1.data(), w1.data(), m1, n1, o1, m2, n2, o2);
        orc_upsample(ux.data(), vx.data(), wx.data(), u0.data(), v0.data(), w0.data(), m, n, o, m1, n1, o1);
        orc_warp_affine(warped1.data(), moving, X, ux.data(), vx.data(), wx.data(), m, n, o);
        std::vector<float> nu1(sz1), nv1(sz1), nw1(sz1);
        orc_descriptor(warped_mind.data(), warped1.data(), m, n, o, curr);
        orc_data_cost(fix_mind.data(), warped_mind.data(), cost.data(), m, n, o, g, hw, q, alpha);
        orc_prims_graph(fixed, m, n, o, g, ordered.data(), parents.data(), edgemst.data());
        orc_regularisation(cost.data(), u0.data(), v0.data(), w0.data(), nu1.data(), nv1.data(), nw1.data(),
                           m1, n1, o1, hw, (float)q, ordered.data(), parents.data(), edgemst.data(), nullptr);
        // backward
        orc_upsample(u0.data(), v0.data(), w0.data(), u1i.data(), v1i.data(), w1i.data(), m1, n1, o1, m2, n2, o2);
        orc_upsample(ux.data(), vx.data(), wx.data(), u0.data(), v0.data(), w0.data(), m, n, o, m1, n1, o1);
        orc_warp_image(warped1.data(), fixed, ux.data(), vx.data(), wx.data(), m, n, o);
        std::vector<float> nu1i(sz1), nv1i(sz1), nw1i(sz1);
        orc_descriptor(warped_mind.data(), warped1.data(), m, n, o, curr);
        orc_data_cost(mov_mind.data(), warped_mind.data(), cost.data(), m, n, o, g, hw, q, alpha);
        orc_prims_graph(warped0.data(), m, n, o, g, ordered.data(), parents.data(), edgemst.data());
        orc_regularisation(cost.data(), u0.data(), v0.data(), w0.data(), nu1i.data(), nv1i.data(), nw1i.data(),
                           m1, n1, o1, hw, (float)q, ordered.data(), parents.data(), edgemst.data(), nullptr);
        orc_consistent_mapping(nu1.data(), nv1.data(), nw1.data(), nu1i.data(), nv1i.data(), nw1i.data(),
                               m1, n1, o1, g);
        if (verbose) {
            float negf = 0;
            float js = orc_jacobian(nu1.data(), nv1.data(), nw1.data(), m1, n1, o1, g, &negf);
            printf("  std(J)=%.2f (J<0)=%.2fe-7\n", std::round(js * 100) / 100.0, std::round(negf * 1e7) / 100.0);
        }
        u1.swap(nu1); v1.swap(nv1); w1.swap(nw1);
        u1i.swap(nu1i); v1i.swap(nv1i); w1i.swap(nw1i);
        m2 = m1; n2 = n1; o2 = o1;
    }
    const size_t sz1 = (size_t)m1 * n1 * o1;
    orc_upsample(ux.data(), vx.data(), wx.data(), u1.data(), v1.data(), w1.data(), m, n, o, m1, n1, o1);
    for (size_t i = 0; i < sz1; i++) { flow[i] = u1[i]; flow[i + sz1] = v1[i]; flow[i + 2 * sz1] = w1[i]; }
    if (ux_out) std::copy(ux.begin(), ux.end(), ux_out);
    if (vx_out) std::copy(vx.begin(), vx.end(), vx_out);
    if (wx_out) std::copy(wx.begin(), wx.end(), wx_out);
    if (warped_out) orc_warp_affine(warped_out, moving, X, ux.data(), vx.data(), wx.data(), m, n, o);
    return (int)sz1;
}

// ---------------------------------------------------------------------------
// linearBCV (src/linearBCV.cpp:163-262): affine / rigid pre-registration from the
// per-node best labels of two smoothed cost volumes, fitted by least trimmed
// squares.  pow(x, 2) of a float is exact in double and sqrt of a float is the
// float overload (the reference's `using namespace std` with <cmath>).

// warpAffine of src/affineLTS1.h:39-68: trilinear with the affine map only, zero
// where the floor corner leaves [0, dim-2].
void orc_lin_warp(float* out, const float* in, const float* X, int m, int n, int o) {
#pragma omp parallel for schedule(static)
    for (int k = 0; k < o; k++)
        for (int j = 0; j < n; j++)
            for (int i = 0; i < m; i++) {
                const size_t p = i + (size_t)j * m + (size_t)k * m * n;
                const float y1 = (float)i * X[0] + (float)j * X[1] + (float)k * X[2] + X[3];
                const float x1 = (float)i * X[4] + (float)j * X[5] + (float)k * X[6] + X[7];
                const float z1 = (float)i * X[8] + (float)j * X[9] + (float)k * X[10] + X[11];
                const int x = (int)std::floor(x1), y = (int)std::floor(y1), z = (int)std::floor(z1);
                const float dx = x1 - x, dy = y1 - y, dz = z1 - z;
                if (y < 0 || y >= m - 1 || x < 0 || x >= n - 1 || z < 0 || z >= o - 1) out[p] = 0.0f;
                else out[p] = sample_trilinear(in, m, n, o, y, x, z, dx, dy, dz);
            }
}

}  // extern "C"

namespace {

float lin_norm(const float* v, int len) {  // src/QRsolve.h:2-8
    float s = 0;
    for (int i = 0; i < len; i++) s = (float)((double)s + (double)v[i] * (double)v[i]);
    return std::sqrt(s);
}

float lin_dot(const float* a, const float* b, int len) {  // src/QRsolve.h:10-16
    float d = 0;
    for (int i = 0; i < len; i++) d += a[i] * b[i];
    return d;
}

// Classical Gram-Schmidt QR of A (len x 4, column c at A + c*len) and the
// back-substitution for len2 right-hand sides (src/QRsolve.h:18-84).
void lin_qrsolve(float* X, const float* A, const float* b, int len, int len2) {
    std::vector<float> Q(4 * (size_t)len);
    const float r11 = lin_norm(A, len);
    for (int i = 0; i < len; i++) Q[i] = A[i] / r11;
    const float r12 = lin_dot(Q.data(), A + len, len);
    const float r13 = lin_dot(Q.data(), A + 2 * len, len);
    const float r14 = lin_dot(Q.data(), A + 3 * len, len);
    for (int i = 0; i < len; i++) {
        Q[i + len] = A[i + len] - Q[i] * r12;
        Q[i + 2 * len] = A[i + 2 * len] - Q[i] * r13;
        Q[i + 3 * len] = A[i + 3 * len] - Q[i] * r14;
    }
    const float r22 = lin_norm(Q.data() + len, len);
    for (int i = 0; i < len; i++) Q[i + len] = Q[i + len] / r22;
    const float r23 = lin_dot(Q.data() + len, A + 2 * len, len);
    const float r24 = lin_dot(Q.data() + len, A + 3 * len, len);
    for (int i = 0; i < len; i++) {
        Q[i + 2 * len] = A[i + 2 * len] - Q[i] * r13 - Q[i + len] * r23;
        Q[i + 3 * len] = A[i + 3 * len] - Q[i] * r14 - Q[i + len] * r24;
    }
    const float r33 = lin_norm(Q.data() + 2 * len, len);
    for (int i = 0; i < len; i++) Q[i + 2 * len] = Q[i + 2 * len] / r33;
    const float r34 = lin_dot(Q.data() + 2 * len, A + 3 * len, len);
    for (int i = 0; i < len; i++) Q[i + 3 * len] = A[i + 3 * len] - Q[i] * r14 - Q[i + len] * r24 - Q[i + 2 * len] * r34;
    const float r44 = lin_norm(Q.data() + 3 * len, len);
    for (int i = 0; i < len; i++) Q[i + 3 * len] = Q[i + 3 * len] / r44;
    for (int j = 0; j < len2; j++) {
        const float d1 = lin_dot(Q.data(), b + (size_t)j * len, len);
        const float d2 = lin_dot(Q.data() + len, b + (size_t)j * len, len);
        const float d3 = lin_dot(Q.data() + 2 * len, b + (size_t)j * len, len);
        const float d4 = lin_dot(Q.data() + 3 * len, b + (size_t)j * len, len);
        const float x4 = d4 / r44;
        const float x3 = (d3 - r34 * x4) / r33;
        const float x2 = (d2 - r23 * x3 - r24 * x4) / r22;
        const float x1 = (d1 - r12 * x2 - r13 * x3 - r14 * x4) / r11;
        X[0 + j * 4] = x1; X[1 + j * 4] = x2; X[2 + j * 4] = x3; X[3 + j * 4] = x4;
    }
}

// One-sided Jacobi SVD of a 3x3 matrix, 4 sweeps (src/QRsolve.h:86-141).
void lin_jacobi3(const float* A, float* U, float* V) {
    for (int i = 0; i < 9; i++) { U[i] = A[i]; V[i] = 0; }
    V[0] = 1; V[4] = 1; V[8] = 1;
    float T[3];
    for (int iter = 0; iter < 4; iter++)
        for (int j = 1; j < 3; j++)
            for (int i = 0; i < j; i++) {
                const float al = lin_dot(U + i * 3, U + i * 3, 3);
                const float be = lin_dot(U + j * 3, U + j * 3, 3);
                const float ga = lin_dot(U + i * 3, U + j * 3, 3);
                const float zeta = (float)((double)(be - al) / (2.0 * (double)ga));
                const float t = (float)((zeta > 0 ? 1.0 : -1.0) /
                                        ((double)std::fabs(zeta) + std::sqrt(1.0 + (double)(zeta * zeta))));
                const float c = (float)(1.0 / (double)std::sqrt(1.0f + t * t));
                const float sn = c * t;
                for (int k = 0; k < 3; k++) T[k] = U[k + i * 3];
                for (int k = 0; k < 3; k++) U[k + i * 3] = c * T[k] - sn * U[k + j * 3];
                for (int k = 0; k < 3; k++) U[k + j * 3] = sn * T[k] + c * U[k + j * 3];
                for (int k = 0; k < 3; k++) T[k] = V[k + i * 3];
                for (int k = 0; k < 3; k++) V[k + i * 3] = c * T[k] - sn * V[k + j * 3];
                for (int k = 0; k < 3; k++) V[k + j * 3] = sn * T[k] + c * V[k + j * 3];
            }
    for (int j = 0; j < 3; j++) {
        const float sv = lin_norm(U + j * 3, 3);
        for (int i = 0; i < 3; i++) U[i + j * 3] /= sv;
    }
}

// Rigid fit (rotation from the SVD of the cross-covariance, translation from the
// means) of point sets in column layout (src/QRsolve.h:143-254).
void lin_find_rigid(float* RT, const float* p1t, const float* p2t, int len) {
    std::vector<float> p1(4 * (size_t)len), p2(4 * (size_t)len);
    for (int i = 0; i < 4; i++)
        for (int k = 0; k < len; k++) {
            p1[i + k * 4] = p1t[k + (size_t)i * len];
            p2[i + k * 4] = p2t[k + (size_t)i * len];
        }
    float m1[3] = {0, 0, 0}, m2[3] = {0, 0, 0};
    for (int k = 0; k < len; k++)
        for (int c = 0; c < 3; c++) { m1[c] += p1[c + k * 4]; m2[c] += p2[c + k * 4]; }
    for (int c = 0; c < 3; c++) { m1[c] /= (float)len; m2[c] /= (float)len; }
    float K[9] = {0}, U[9], V[9], R[16] = {0};
    for (int k = 0; k < len; k++)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) K[i + j * 3] += (p1[j + k * 4] - m1[j]) * (p2[i + k * 4] - m2[i]);
    lin_jacobi3(K, U, V);
    for (int i = 0; i < 16; i++) RT[i] = 0.0f;
    R[15] = 1.0f;
    RT[15] = 1.0f;
    for (int k = 0; k < 3; k++)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) R[j + i * 4] += U[j + k * 3] * V[i + k * 3];
    std::vector<float> Rp2(4 * (size_t)len);
    lin_qrsolve(Rp2.data(), R, p2.data(), 4, len);
    float t1[3] = {0, 0, 0};
    for (int i = 0; i < len; i++)
        for (int c = 0; c < 3; c++) t1[c] += Rp2[c + i * 4];
    for (int c = 0; c < 3; c++) t1[c] = t1[c] / (float)len - m1[c];
    float t0[3] = {0, 0, 0};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) t0[i] += R[i + j * 4] * t1[j];
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) RT[i + j * 4] += R[j + i * 4];
        RT[3 + i * 4] = t0[i];
    }
}

void lin_fit(float* RT, const float* p1, const float* p2, int len, bool rigid) {
    if (rigid) lin_find_rigid(RT, p1, p2, len);
    else lin_qrsolve(RT, p1, p2, len, 4);
}

}  // namespace

extern "C" {

// affineRobust (src/QRsolve.h:258-296): a fit to all points, then 15 rounds of
// refitting to the half with the smallest squared residuals.
void orc_affine_robust(float* RT, const float* p1, const float* p2, int len, int rigid) {
    if (len < 8) return;  // the reference indexes an empty trimmed half here (undefined); not fitted
    lin_fit(RT, p1, p2, len, rigid != 0);
    const int lenh = len / 2;
    std::vector<float> err(len), err2(len), p1b(4 * (size_t)lenh, 1.0f), p2b(4 * (size_t)lenh, 1.0f);
    for (int iter = 0; iter < 15; iter++) {
        for (int l = 0; l < len; l++) {
            float x = 0, y = 0, z = 0;
            for (int i = 0; i < 3; i++) {
                y += p1[l + (size_t)i * len] * RT[i];
                x += p1[l + (size_t)i * len] * RT[i + 4];
                z += p1[l + (size_t)i * len] * RT[i + 8];
            }
            y += p1[l + 3 * (size_t)len] * RT[3];
            x += p1[l + 3 * (size_t)len] * RT[7];
            z += p1[l + 3 * (size_t)len] * RT[11];
            const double ey = (double)(y - p2[l]), ex = (double)(x - p2[l + len]), ez = (double)(z - p2[l + 2 * (size_t)len]);
            err[l] = (float)(ey * ey + ex * ex + ez * ez);
            err2[l] = err[l];
        }
        std::nth_element(err.begin(), err.begin() + len / 2, err.end());
        const float median = err[len / 2];
        int count = 0;
        for (int i = 0; i < len; i++) {
            const int l = std::min(count, lenh - 1);
            if (err2[i] <= median) {
                for (int c = 0; c < 3; c++) {
                    p1b[l + (size_t)c * lenh] = p1[i + (size_t)c * len];
                    p2b[l + (size_t)c * lenh] = p2[i + (size_t)c * len];
                }
                count++;
            }
        }
        lin_fit(RT, p1b.data(), p2b.data(), lenh, rigid != 0);
    }
}

void orc_qrsolve(float* X, const float* A, const float* b, int len, int len2) { lin_qrsolve(X, A, b, len, len2); }

// The three in-place smoothing passes of estimateAffine2 (src/affineLTS1.h:124-158):
// along y, then x, then z, each node gets half its two neighbours added, the
// lower neighbour already updated by the same pass (sequential node order).
void orc_lin_smooth(float* cost, int m1, int n1, int o1, int len3) {
    const int sz1 = m1 * n1 * o1;
    for (int axis = 0; axis < 3; axis++)
        for (int i = 0; i < sz1; i++) {
            const int z1 = i / (m1 * n1), x1 = (i - z1 * m1 * n1) / m1, y1 = i - z1 * m1 * n1 - x1 * m1;
            int i1, i2;
            if (axis == 0) {
                i1 = std::min(y1 + 1, m1 - 1) + x1 * m1 + z1 * m1 * n1;
                i2 = std::max(y1 - 1, 0) + x1 * m1 + z1 * m1 * n1;
            } else if (axis == 1) {
                i1 = y1 + std::min(x1 + 1, n1 - 1) * m1 + z1 * m1 * n1;
                i2 = y1 + std::max(x1 - 1, 0) * m1 + z1 * m1 * n1;
            } else {
                i1 = y1 + x1 * m1 + std::min(z1 + 1, o1 - 1) * m1 * n1;
                i2 = y1 + x1 * m1 + std::max(z1 - 1, 0) * m1 * n1;
            }
            for (int l = 0; l < len3; l++) {
                const double add = 0.5 * (double)cost[(size_t)i1 * len3 + l] + 0.5 * (double)cost[(size_t)i2 * len3 + l];
                cost[(size_t)i * len3 + l] = (float)((double)cost[(size_t)i * len3 + l] + add);
            }
        }
}

// estimateAffine2 (src/affineLTS1.h:91-236) on the two cost volumes of a level
// (smoothed in place), the +1024-shifted fixed and moving images and the previous
// matrix; X = fit * Xprev.  Returns the number of points used.
int orc_estimate_affine(float* X, const float* Xprev, const float* fixed, const float* moving, float* cost,
                        float* cost2, int m, int n, int o, int g, float q, int hw, int rigid) {
    const int m1 = m / g, n1 = n / g, o1 = o / g, sz1 = m1 * n1 * o1;
    const int len = 2 * hw + 1, len3 = len * len * len, stephw = (g - 1) / 2;
    std::vector<float> xs(len3), ys(len3), zs(len3);
    for (int l = 0; l < len3; l++) {
        const int i = l % len, j = (l / len) % len, k = l / (len * len);
        xs[l] = (j - hw) * q; ys[l] = (i - hw) * q; zs[l] = (k - hw) * q;
    }
    orc_lin_smooth(cost, m1, n1, o1, len3);
    orc_lin_smooth(cost2, m1, n1, o1, len3);
    std::vector<float> minval(sz1), minval2(sz1);
    std::vector<int> minind(sz1), minind2(sz1);
    int allcount = 0;
    for (int i = 0; i < sz1; i++) {
        const float* c1 = cost + (size_t)i * len3;
        const float* c2 = cost2 + (size_t)i * len3;
        minind[i] = (int)(std::min_element(c1, c1 + len3) - c1);
        minval[i] = c1[minind[i]];
        minind2[i] = (int)(std::min_element(c2, c2 + len3) - c2);
        minval2[i] = c2[minind2[i]];
        const int z1 = i / (m1 * n1), x1 = (i - z1 * m1 * n1) / m1, y1 = i - z1 * m1 * n1 - x1 * m1;
        float mean1 = 0.0f, mean2 = 0.0f;
        for (int k1 = 0; k1 < g; k1++)
            for (int j1 = 0; j1 < g; j1++)
                for (int i1 = 0; i1 < g; i1++) {
                    const size_t ind = y1 * g + i1 + (size_t)(x1 * g + j1) * m + (size_t)(z1 * g + k1) * m * n;
                    mean1 += fixed[ind];
                    mean2 += moving[ind];
                }
        mean1 /= (float)(g * g * g);
        mean2 /= (float)(g * g * g);
        if (mean1 < 5.0f) minval[i] = 1e20f;
        if (mean2 < 5.0f) minval2[i] = 1e20f;
        if (z1 < 2 || z1 > o1 - 2 || x1 < 2 || x1 > n1 - 2 || y1 < 2 || y1 > m1 - 2) {
            minval[i] = 1e20f;
            minval2[i] = 1e20f;
        }
        if (minval[i] < 1e19f) allcount++;
        if (minval2[i] < 1e19f) allcount++;
    }
    // quantile() of src/linearBCV.cpp:36-46 at 0.5*allcount/sz1/2
    const float qf = (float)(0.5 * (double)allcount / (double)(float)sz1 / 2.0);
    auto quantile = [&](const std::vector<float>& v) {
        std::vector<float> c(v);
        const int qi = (int)((float)sz1 * std::min(std::max(qf, 0.01f), 0.99f));
        std::nth_element(c.begin(), c.begin() + qi, c.end());
        return c[qi];
    };
    const float med1 = quantile(minval), med2 = quantile(minval2);
    int valsz = 0;
    for (int i = 0; i < sz1; i++) valsz += (minval[i] < med1) + (minval2[i] < med2);
    std::vector<float> p1(4 * (size_t)valsz), p2(4 * (size_t)valsz);
    int cur = 0;
    for (int i = 0; i < sz1; i++) {
        const int k1 = i / (m1 * n1), j1 = (i - k1 * (m1 * n1)) / m1, i1 = i - j1 * m1 - k1 * m1 * n1;
        const int y1 = i1 * g + stephw, x1 = j1 * g + stephw, z1 = k1 * g + stephw;
        if (minval[i] < med1) {
            const int ind = minind[i];
            p1[cur + 3 * (size_t)valsz] = 1.0f; p2[cur + 3 * (size_t)valsz] = 1.0f;
            p1[cur] = y1; p1[cur + valsz] = x1; p1[cur + 2 * (size_t)valsz] = z1;
            p2[cur] = y1 + ys[ind]; p2[cur + valsz] = x1 + xs[ind]; p2[cur + 2 * (size_t)valsz] = z1 + zs[ind];
            cur++;
        }
        if (minval2[i] < med2) {
            const int ind = minind2[i];
            p1[cur + 3 * (size_t)valsz] = 1.0f; p2[cur + 3 * (size_t)valsz] = 1.0f;
            p2[cur] = y1; p2[cur + valsz] = x1; p2[cur + 2 * (size_t)valsz] = z1;
            p1[cur] = y1 + ys[ind]; p1[cur + valsz] = x1 + xs[ind]; p1[cur + 2 * (size_t)valsz] = z1 + zs[ind];
            cur++;
        }
    }
    if (valsz < 8) return valsz;  // too few points to fit (X not written)
    float X1[16];
    orc_affine_robust(X1, p1.data(), p2.data(), valsz, rigid);
    for (int i = 0; i < 4; i++)  // matmult (src/affineLTS1.h:1-12)
        for (int j = 0; j < 4; j++) {
            float acc = 0.0f;
            for (int k = 0; k < 4; k++) acc += X1[i + k * 4] * Xprev[k + j * 4];
            X[i + j * 4] = acc;
        }
    return valsz;
}

// The linearBCV level loop (src/linearBCV.cpp:163-262) on +1024-shifted images:
// per level both images are warped by the current matrix (moving forwards,
// fixed by its QR inverse), both cost volumes are built with alpha 1 and the
// matrix is re-estimated.  X: 16 floats out.
void orc_linear_register(const float* fixed, const float* moving, int m, int n, int o, int levels, const int* G,
                         const int* Lr, const int* Q, int rigid, float* X) {
    const size_t sz = (size_t)m * n * o;
    float Xprev[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    std::copy(Xprev, Xprev + 16, X);
    const float ident[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    std::vector<float> w1(sz), w2(sz);
    std::vector<uint64_t> mov_mind(sz), fix_mind(sz), warped_mind(sz);
    for (int level = 0; level < levels; level++) {
        const int g = G[level], hw = Lr[level], q = Q[level];
        float Xinv[16];
        lin_qrsolve(Xinv, Xprev, ident, 4, 4);
        orc_lin_warp(w2.data(), fixed, Xinv, m, n, o);
        orc_lin_warp(w1.data(), moving, Xprev, m, n, o);
        const int prev = orc_mind_step(Q[std::max(level - 1, 0)]), curr = orc_mind_step(q);
        if (level == 0 || prev != curr) {
            orc_descriptor(mov_mind.data(), moving, m, n, o, curr);
            orc_descriptor(fix_mind.data(), fixed, m, n, o, curr);
        }
        const int len = 2 * hw + 1, len3 = len * len * len;
        const size_t sz1 = (size_t)(m / g) * (n / g) * (o / g);
        std::vector<float> cost(sz1 * len3), cost2(sz1 * len3);
        orc_descriptor(warped_mind.data(), w1.data(), m, n, o, curr);
        orc_data_cost(fix_mind.data(), warped_mind.data(), cost.data(), m, n, o, g, hw, q, 1.0f);
        orc_descriptor(warped_mind.data(), w2.data(), m, n, o, curr);
        orc_data_cost(mov_mind.data(), warped_mind.data(), cost2.data(), m, n, o, g, hw, q, 1.0f);
        orc_estimate_affine(X, Xprev, fixed, moving, cost.data(), cost2.data(), m, n, o, g, (float)q, hw, rigid);
        std::copy(X, X + 16, Xprev);
    }
}

}  // extern "C"
