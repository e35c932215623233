// Host half of linearBCV (see linear_host.h).  The fit works on at most a few
// ten thousand points, so it stays on the CPU next to the level loop; its
// arithmetic follows the reference's types exactly (compiled without FMA
// contraction): float accumulations, pow(x, 2) of a float evaluated in double
// (exact), the float overload of sqrt, double where a double literal appears.
#include "linear_host.h"

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>

namespace deeds {

namespace {

// Column view of a point set: column c of `len` entries at p + c*len.
struct Cols {
    const float* p;
    int len;
    const float* col(int c) const { return p + (size_t)c * len; }
};

float sq_norm_sqrt(const float* v, int len) {  // norm, src/QRsolve.h:2-8
    float acc = 0.0f;
    for (int i = 0; i < len; i++) acc = (float)((double)acc + (double)v[i] * (double)v[i]);
    return std::sqrt(acc);
}

float dotf(const float* a, const float* b, int len) {  // dotprod, src/QRsolve.h:10-16
    float acc = 0.0f;
    for (int i = 0; i < len; i++) acc += a[i] * b[i];
    return acc;
}

// One-sided Jacobi rotations on the columns of a 3x3 matrix, four sweeps
// (jacobiSVD3, src/QRsolve.h:86-141); U gets the normalised columns, V the
// accumulated rotations.
void jacobi3(const float* A, float* U, float* V) {
    for (int i = 0; i < 9; i++) { U[i] = A[i]; V[i] = 0.0f; }
    V[0] = V[4] = V[8] = 1.0f;
    for (int sweep = 0; sweep < 4; sweep++)
        for (int j = 1; j < 3; j++)
            for (int i = 0; i < j; i++) {
                float* ui = U + 3 * i;
                float* uj = U + 3 * j;
                const float a = dotf(ui, ui, 3), b = dotf(uj, uj, 3), gm = dotf(ui, uj, 3);
                const float zeta = (float)((double)(b - a) / (2.0 * (double)gm));
                const double sgn = zeta > 0 ? 1.0 : -1.0;
                const float t = (float)(sgn / ((double)std::fabs(zeta) + std::sqrt(1.0 + (double)(zeta * zeta))));
                const float c = (float)(1.0 / (double)std::sqrt(1.0f + t * t));
                const float s = c * t;
                float* vi = V + 3 * i;
                float* vj = V + 3 * j;
                for (int k = 0; k < 3; k++) {
                    const float ti = ui[k];
                    ui[k] = c * ti - s * uj[k];
                    uj[k] = s * ti + c * uj[k];
                }
                for (int k = 0; k < 3; k++) {
                    const float ti = vi[k];
                    vi[k] = c * ti - s * vj[k];
                    vj[k] = s * ti + c * vj[k];
                }
            }
    for (int j = 0; j < 3; j++) {
        const float sv = sq_norm_sqrt(U + 3 * j, 3);
        for (int i = 0; i < 3; i++) U[i + 3 * j] /= sv;
    }
}

// findRigid (src/QRsolve.h:143-254): rotation R = sum_k u_k v_k^T from the SVD of
// the cross-covariance, translation through R's QR solve of the second point
// set; RT gets R^T and the translation.
void find_rigid(float* RT, Cols a, Cols b) {
    const int len = a.len;
    std::vector<float> pa(4 * (size_t)len), pb(4 * (size_t)len);  // point-major (x4)
    for (int c = 0; c < 4; c++)
        for (int k = 0; k < len; k++) {
            pa[c + 4 * (size_t)k] = a.col(c)[k];
            pb[c + 4 * (size_t)k] = b.col(c)[k];
        }
    float ma[3] = {0.0f, 0.0f, 0.0f}, mb[3] = {0.0f, 0.0f, 0.0f};
    for (int k = 0; k < len; k++)
        for (int c = 0; c < 3; c++) {
            ma[c] += pa[c + 4 * (size_t)k];
            mb[c] += pb[c + 4 * (size_t)k];
        }
    for (int c = 0; c < 3; c++) {
        ma[c] /= (float)len;
        mb[c] /= (float)len;
    }
    float K[9] = {0.0f}, U[9], V[9], R[16] = {0.0f};
    for (int k = 0; k < len; k++)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) K[i + 3 * j] += (pa[j + 4 * (size_t)k] - ma[j]) * (pb[i + 4 * (size_t)k] - mb[i]);
    jacobi3(K, U, V);
    std::fill(RT, RT + 16, 0.0f);
    R[15] = 1.0f;
    RT[15] = 1.0f;
    for (int k = 0; k < 3; k++)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) R[j + 4 * i] += U[j + 3 * k] * V[i + 3 * k];
    std::vector<float> rb(4 * (size_t)len);
    lin_qrsolve(rb.data(), R, pb.data(), 4, len);
    float t1[3] = {0.0f, 0.0f, 0.0f};
    for (int k = 0; k < len; k++)
        for (int c = 0; c < 3; c++) t1[c] += rb[c + 4 * (size_t)k];
    for (int c = 0; c < 3; c++) t1[c] = t1[c] / (float)len - ma[c];
    float t0[3] = {0.0f, 0.0f, 0.0f};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) t0[i] += R[i + 4 * j] * t1[j];
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) RT[i + 4 * j] += R[j + 4 * i];
        RT[3 + 4 * i] = t0[i];
    }
}

// The k-th smallest of non-negative floats (squared residuals): their bit
// patterns order like the values, so two 16-bit radix passes find it exactly, in
// place of nth_element (whose answer is the same value).
float kth_smallest_nonneg(const std::vector<float>& v, int k, std::vector<uint32_t>& scratch) {
    static thread_local std::vector<uint32_t> hist(65536);
    std::fill(hist.begin(), hist.end(), 0u);
    const size_t n = v.size();
    const uint32_t* bits = reinterpret_cast<const uint32_t*>(v.data());
    for (size_t i = 0; i < n; i++) hist[bits[i] >> 16]++;
    uint32_t hi = 0, below = 0;
    for (;; hi++) {
        if (below + hist[hi] > (uint32_t)k) break;
        below += hist[hi];
    }
    scratch.clear();
    for (size_t i = 0; i < n; i++)
        if ((bits[i] >> 16) == hi) scratch.push_back(bits[i] & 0xffffu);
    std::fill(hist.begin(), hist.end(), 0u);
    for (uint32_t lo : scratch) hist[lo]++;
    const uint32_t want = (uint32_t)k - below;
    uint32_t lo = 0, acc = 0;
    for (;; lo++) {
        if (acc + hist[lo] > want) break;
        acc += hist[lo];
    }
    const uint32_t r = (hi << 16) | lo;
    float out;
    std::memcpy(&out, &r, sizeof(out));
    return out;
}

void fit(float* RT, Cols a, Cols b, bool rigid) {
    if (rigid) find_rigid(RT, a, b);
    else lin_qrsolve(RT, a.p, b.p, a.len, 4);
}

}  // namespace

// The Gram-Schmidt QR with every sum kept in its own sequential accumulator, in
// index order, exactly as the reference evaluates it; what changes is only that
// independent sums (and the vector updates feeding them) share one pass over
// the points, so their dependency chains overlap instead of running one after
// another.  Same bits, several times fewer passes.
void lin_qrsolve(float* X, const float* A, const float* b, int len, int nrhs) {
    std::vector<float> Qv(4 * (size_t)len);
    float* q0 = Qv.data();
    float* q1 = q0 + len;
    float* q2 = q1 + len;
    float* q3 = q2 + len;
    const float* a0 = A;
    const float* a1 = A + len;
    const float* a2 = A + 2 * (size_t)len;
    const float* a3 = A + 3 * (size_t)len;
    auto norm_step = [](float acc, float v) { return (float)((double)acc + (double)v * (double)v); };
    // column 1
    float n0 = 0.0f;
    for (int i = 0; i < len; i++) n0 = norm_step(n0, a0[i]);
    const float r11 = std::sqrt(n0);
    float r12 = 0.0f, r13 = 0.0f, r14 = 0.0f;
    for (int i = 0; i < len; i++) {
        const float q = a0[i] / r11;
        q0[i] = q;
        r12 += q * a1[i];
        r13 += q * a2[i];
        r14 += q * a3[i];
    }
    // column 2 (q2, q3 hold the partially orthogonalised columns 3 and 4)
    float n1 = 0.0f;
    for (int i = 0; i < len; i++) {
        const float v = a1[i] - q0[i] * r12;
        q1[i] = v;
        q2[i] = a2[i] - q0[i] * r13;
        q3[i] = a3[i] - q0[i] * r14;
        n1 = norm_step(n1, v);
    }
    const float r22 = std::sqrt(n1);
    float r23 = 0.0f, r24 = 0.0f;
    for (int i = 0; i < len; i++) {
        const float q = q1[i] / r22;
        q1[i] = q;
        r23 += q * a2[i];
        r24 += q * a3[i];
    }
    // column 3
    float n2 = 0.0f;
    for (int i = 0; i < len; i++) {
        const float v = a2[i] - q0[i] * r13 - q1[i] * r23;
        q2[i] = v;
        q3[i] = a3[i] - q0[i] * r14 - q1[i] * r24;
        n2 = norm_step(n2, v);
    }
    const float r33 = std::sqrt(n2);
    float r34 = 0.0f;
    for (int i = 0; i < len; i++) {
        const float q = q2[i] / r33;
        q2[i] = q;
        r34 += q * a3[i];
    }
    // column 4
    float n3 = 0.0f;
    for (int i = 0; i < len; i++) {
        const float v = a3[i] - q0[i] * r14 - q1[i] * r24 - q2[i] * r34;
        q3[i] = v;
        n3 = norm_step(n3, v);
    }
    const float r44 = std::sqrt(n3);
    for (int i = 0; i < len; i++) q3[i] = q3[i] / r44;
    // right-hand sides: 4 dot products each, up to four right-hand sides per pass
    for (int j0 = 0; j0 < nrhs; j0 += 4) {
        const int nj = std::min(4, nrhs - j0);
        float d[4][4] = {{0.0f}};
        if (nj == 4) {
            const float* b0 = b + (size_t)j0 * len;
            const float* b1 = b0 + len;
            const float* b2 = b1 + len;
            const float* b3 = b2 + len;
            for (int i = 0; i < len; i++) {
                const float qa = q0[i], qb = q1[i], qc = q2[i], qd = q3[i];
                const float bb[4] = {b0[i], b1[i], b2[i], b3[i]};
                for (int j = 0; j < 4; j++) {
                    d[j][0] += qa * bb[j];
                    d[j][1] += qb * bb[j];
                    d[j][2] += qc * bb[j];
                    d[j][3] += qd * bb[j];
                }
            }
        } else {
            for (int j = 0; j < nj; j++) {
                const float* bj = b + (size_t)(j0 + j) * len;
                for (int i = 0; i < len; i++) {
                    d[j][0] += q0[i] * bj[i];
                    d[j][1] += q1[i] * bj[i];
                    d[j][2] += q2[i] * bj[i];
                    d[j][3] += q3[i] * bj[i];
                }
            }
        }
        for (int j = 0; j < nj; j++) {
            const float x4 = d[j][3] / r44;
            const float x3 = (d[j][2] - r34 * x4) / r33;
            const float x2 = (d[j][1] - r23 * x3 - r24 * x4) / r22;
            const float x1 = (d[j][0] - r12 * x2 - r13 * x3 - r14 * x4) / r11;
            float* Xj = X + 4 * (size_t)(j0 + j);
            Xj[0] = x1;
            Xj[1] = x2;
            Xj[2] = x3;
            Xj[3] = x4;
        }
    }
}

void lin_affine_robust(float* RT, const float* p1, const float* p2, int len, bool rigid) {
    if (len < kMinFitPoints) return;  // the trimmed half would be empty (the reference reads outside its arrays)
    const Cols A{p1, len}, B{p2, len};
    fit(RT, A, B, rigid);
    const int half = len / 2;
    std::vector<float> err(len);
    std::vector<uint32_t> scratch;
    scratch.reserve(len);
    std::vector<float> ha(4 * (size_t)half, 1.0f), hb(4 * (size_t)half, 1.0f);  // the kept half; column 3 stays 1
    for (int iter = 0; iter < 15; iter++) {
        for (int l = 0; l < len; l++) {
            float y = 0.0f, x = 0.0f, z = 0.0f;
            for (int c = 0; c < 3; c++) {
                const float v = A.col(c)[l];
                y += v * RT[c];
                x += v * RT[c + 4];
                z += v * RT[c + 8];
            }
            const float h = A.col(3)[l];
            y += h * RT[3];
            x += h * RT[7];
            z += h * RT[11];
            const double ey = (double)(y - B.col(0)[l]), ex = (double)(x - B.col(1)[l]), ez = (double)(z - B.col(2)[l]);
            err[l] = (float)(ey * ey + ex * ex + ez * ez);
        }
        const float median = kth_smallest_nonneg(err, len / 2, scratch);
        // points at or below the median, in order; any beyond the half overwrite the last slot
        int count = 0;
        for (int i = 0; i < len; i++) {
            if (!(err[i] <= median)) continue;
            const int slot = std::min(count, half - 1);
            for (int c = 0; c < 3; c++) {
                ha[slot + (size_t)c * half] = A.col(c)[i];
                hb[slot + (size_t)c * half] = B.col(c)[i];
            }
            count++;
        }
        fit(RT, Cols{ha.data(), half}, Cols{hb.data(), half}, rigid);
    }
}

void lin_matmult(const float* A, const float* B, float* X) {
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            float acc = 0.0f;
            for (int k = 0; k < 4; k++) acc += A[i + 4 * k] * B[k + 4 * j];
            X[i + 4 * j] = acc;
        }
}

int lin_estimate_from_stats(float* X, const float* Xprev, const float* minval, const int* minind, int m1, int n1,
                            int o1, int g, float q, int hw, bool rigid, int* allcount_out, float* quantile_out) {
    const int sz1 = m1 * n1 * o1, len = 2 * hw + 1, stephw = (g - 1) / 2;
    const float* mv[2] = {minval, minval + sz1};
    const int* mi[2] = {minind, minind + sz1};
    int allcount = 0;
    for (int v = 0; v < 2; v++)
        for (int i = 0; i < sz1; i++) allcount += mv[v][i] < 1e19f;
    // quantile() of src/linearBCV.cpp:36-46 at 0.5*allcount/sz1/2 (double, then float)
    const float qf = (float)(0.5 * (double)allcount / (double)(float)sz1 / 2.0);
    const int qi = (int)((float)sz1 * std::min(std::max(qf, 0.01f), 0.99f));
    float med[2];
    std::vector<float> tmp(sz1);
    std::vector<uint32_t> scratch;
    for (int v = 0; v < 2; v++) {  // cost volumes are non-negative, the exclusion value is 1e20
        std::copy(mv[v], mv[v] + sz1, tmp.begin());
        med[v] = kth_smallest_nonneg(tmp, qi, scratch);
    }
    int valsz = 0;
    for (int i = 0; i < sz1; i++) valsz += (mv[0][i] < med[0]) + (mv[1][i] < med[1]);
    if (allcount_out) *allcount_out = allcount;
    if (quantile_out) *quantile_out = qf;
    // ties at the quantile (e.g. a constant image pair) can leave no point strictly
    // below it; the caller reports that instead of fitting
    if (valsz < kMinFitPoints) return valsz;
    std::vector<float> p1(4 * (size_t)valsz), p2(4 * (size_t)valsz);
    float* p1c[4] = {p1.data(), p1.data() + valsz, p1.data() + 2 * (size_t)valsz, p1.data() + 3 * (size_t)valsz};
    float* p2c[4] = {p2.data(), p2.data() + valsz, p2.data() + 2 * (size_t)valsz, p2.data() + 3 * (size_t)valsz};
    int cur = 0;
    for (int i = 0; i < sz1; i++) {
        const int k1 = i / (m1 * n1), j1 = (i - k1 * m1 * n1) / m1, i1 = i - j1 * m1 - k1 * m1 * n1;
        const int cy = i1 * g + stephw, cx = j1 * g + stephw, cz = k1 * g + stephw;
        for (int v = 0; v < 2; v++) {
            if (!(mv[v][i] < med[v])) continue;
            // label l -> displacement ((l%len)-hw, (l/len%len)-hw, (l/len^2)-hw) * q in (y, x, z)
            const int l = mi[v][i];
            const float dy = (l % len - hw) * q, dx = ((l / len) % len - hw) * q, dz = (l / (len * len) - hw) * q;
            // direction 1: node -> node + d; direction 2: node + d -> node
            float** at = v == 0 ? p1c : p2c;
            float** bt = v == 0 ? p2c : p1c;
            at[0][cur] = (float)cy; at[1][cur] = (float)cx; at[2][cur] = (float)cz;
            bt[0][cur] = cy + dy; bt[1][cur] = cx + dx; bt[2][cur] = cz + dz;
            p1c[3][cur] = 1.0f;
            p2c[3][cur] = 1.0f;
            cur++;
        }
    }
    float X1[16];
    lin_affine_robust(X1, p1.data(), p2.data(), valsz, rigid);
    lin_matmult(X1, Xprev, X);
    return valsz;
}

}  // namespace deeds
