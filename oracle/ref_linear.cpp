// TEST INFRASTRUCTURE — not part of the product.
//
// Stage-dump harness around the UNMODIFIED linearBCV reference source.  The
// reference's linearBCV.cpp is compiled into this translation unit with its
// `main` renamed, so its globals (image_m/n/o, RIGID, qc), its quantile() and the
// headers it includes (affineLTS1.h, QRsolve.h, MINDSSCbox.h, dataCostD.h, ...)
// are exactly the reference's; the main below calls one reference function per
// invocation on raw little-endian binary inputs.  Used only to produce golden
// vectors (tests/golden/make_golden.py) that pin the oracle restatement.
//
// usage: ref_linear <stage> <args...>   (see the dispatch table in main)
#define main linearBCV_reference_main
#include "linearBCV.cpp"
#undef main

#include <cstdio>
#include <cstdlib>

template <typename T> static T* load(const char* path, size_t count) {
    T* p = new T[count];
    FILE* f = fopen(path, "rb");
    if (!f) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
    size_t got = fread(p, sizeof(T), count, f);
    fclose(f);
    if (got != count) { fprintf(stderr, "%s: expected %zu items, got %zu\n", path, count, got); exit(2); }
    return p;
}
template <typename T> static void save(const char* path, const T* p, size_t count) {
    FILE* f = fopen(path, "wb");
    if (!f) { fprintf(stderr, "cannot write %s\n", path); exit(2); }
    fwrite(p, sizeof(T), count, f);
    fclose(f);
}

int main(int argc, char** argv) {
    if (argc < 2) { fprintf(stderr, "usage: ref_linear <stage> ...\n"); return 2; }
    string st = argv[1];
    RAND_SAMPLES = 1;  // src/linearBCV.cpp:126
    if (st == "warp") {  // warp in.f32 X.f32(16) m n o out.f32   (affineLTS1.h warpAffine)
        int m = atoi(argv[4]), n = atoi(argv[5]), o = atoi(argv[6]);
        image_m = m; image_n = n; image_o = o;
        size_t s = (size_t)m * n * o;
        float* in = load<float>(argv[2], s);
        float* X = load<float>(argv[3], 16);
        float* out = new float[s];
        warpAffine(out, in, X, m, n, o);
        save(argv[7], out, s);
    } else if (st == "qrinv") {  // qrinv X.f32(16) out.f32(16)   (src/linearBCV.cpp:186-187)
        float* X = load<float>(argv[2], 16);
        float Xinv[16]; float Ident[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
        qrsolve(Xinv, X, Ident, 4, 4);
        save(argv[3], Xinv, 16);
    } else if (st == "estimate") {
        // estimate fixed.f32 moving.f32 cost.f32 cost2.f32 Xprev.f32 m n o g hw q rigid  X.f32 smooth.f32 smooth2.f32
        int m = atoi(argv[7]), n = atoi(argv[8]), o = atoi(argv[9]);
        int g = atoi(argv[10]), hw = atoi(argv[11]);
        float q = atof(argv[12]);
        RIGID = atoi(argv[13]) != 0;
        image_m = m; image_n = n; image_o = o;
        size_t s = (size_t)m * n * o;
        size_t sz1 = (size_t)(m / g) * (n / g) * (o / g);
        int len3 = (int)pow(hw * 2 + 1, 3);
        float* fixed = load<float>(argv[2], s);
        float* moving = load<float>(argv[3], s);
        float* cost = load<float>(argv[4], sz1 * len3);
        float* cost2 = load<float>(argv[5], sz1 * len3);
        float* Xprev = load<float>(argv[6], 16);
        float X[16];
        estimateAffine2(X, Xprev, fixed, moving, cost, cost2, g, q, hw);
        save(argv[14], X, 16);
        save(argv[15], cost, sz1 * len3);  // smoothed in place by estimateAffine2
        save(argv[16], cost2, sz1 * len3);
    } else if (st == "robust") {  // robust pts1.f32 pts2.f32 len rigid out.f32(16)
        int len = atoi(argv[4]);
        RIGID = atoi(argv[5]) != 0;
        float* p1 = load<float>(argv[2], (size_t)len * 4);
        float* p2 = load<float>(argv[3], (size_t)len * 4);
        float RT[16];
        affineRobust(RT, p1, p2, len);
        save(argv[6], RT, 16);
    } else {
        fprintf(stderr, "unknown stage %s\n", st.c_str());
        return 2;
    }
    return 0;
}
