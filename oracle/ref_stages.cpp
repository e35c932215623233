// TEST INFRASTRUCTURE — not part of the product.
//
// Stage-dump harness around the UNMODIFIED deedsBCV reference sources.  It is
// compiled (by oracle/Makefile) against the reference headers where they lie
// and is used only to produce golden vectors that pin the oracle restatement
// (oracle/deeds_oracle.cpp).  It defines the process globals the reference
// headers read (src/deedsBCV0.cpp:24-28, :31-44) and then calls exactly one
// reference function per invocation on raw little-endian binary inputs.
//
// usage: ref_stages <stage> <args...>   (see the dispatch table in main)
#include <iostream>
#include <fstream>
#include <math.h>
#include <sys/time.h>
#include <vector>
#include <algorithm>
#include <numeric>
#include <map>
#include <functional>
#include <string.h>
#include <sstream>
#include <pthread.h>
#include <thread>
#include <cstddef>
#include <cstdint>
#include <climits>
#include <cstdlib>
#include "zlib.h"
#include <sys/stat.h>

using namespace std;

// globals the reference headers expect (defined by src/deedsBCV0.cpp:24-28)
int RAND_SAMPLES;
int image_m; int image_n; int image_o; int image_d = 1;
float SSD0 = 0.0; float SSD1 = 0.0; float SSD2 = 0.0; float distfx_global; float beta = 1;
int qc = 1;
struct mind_data { float* im1; float* d1; uint64_t* mindq; int qs; int ind_d1; };
struct parameters {
    float alpha; int levels; bool segment, affine, rigid;
    vector<int> grid_spacing; vector<int> search_radius; vector<int> quantisation;
    string fixed_file, moving_file, output_stem, moving_seg_file, affine_file, deformed_file;
};

#include "imageIOgzType.h"
#include "transformations.h"
#include "primsMST.h"
#include "regularisation.h"
#include "MINDSSCbox.h"
#include "dataCostD.h"

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
    if (argc < 2) { fprintf(stderr, "usage: ref_stages <stage> ...\n"); return 2; }
    string st = argv[1];
    RAND_SAMPLES = 1;  // src/deedsBCV0.cpp:116
    if (st == "mind") {  // mind in.f32 m n o qs out.u64
        int m = atoi(argv[3]), n = atoi(argv[4]), o = atoi(argv[5]), qs = atoi(argv[6]);
        image_m = m; image_n = n; image_o = o;
        size_t sz = (size_t)m * n * o;
        float* im = load<float>(argv[2], sz);
        uint64_t* q = new uint64_t[sz];
        descriptor(q, im, m, n, o, qs);
        save(argv[7], q, sz);
    } else if (st == "datacost") {  // datacost F.u64 M.u64 m n o g hw q alpha out.f32
        int m = atoi(argv[4]), n = atoi(argv[5]), o = atoi(argv[6]);
        int g = atoi(argv[7]), hw = atoi(argv[8]);
        float q = atof(argv[9]), alpha = atof(argv[10]);
        image_m = m; image_n = n; image_o = o;
        size_t sz = (size_t)m * n * o;
        uint64_t* F = load<uint64_t>(argv[2], sz);
        uint64_t* M = load<uint64_t>(argv[3], sz);
        int len3 = (int)pow(hw * 2 + 1, 3);
        size_t sz1 = (size_t)(m / g) * (n / g) * (o / g);
        float* cost = new float[sz1 * len3];
        dataCostCL((unsigned long*)F, (unsigned long*)M, cost, m, n, o, len3, g, hw, q, alpha, RAND_SAMPLES);
        save(argv[11], cost, sz1 * len3);
    } else if (st == "prims") {  // prims img.f32 m n o g ordered.i32 parents.i32 edgemst.f32
        int m = atoi(argv[3]), n = atoi(argv[4]), o = atoi(argv[5]), g = atoi(argv[6]);
        image_m = m; image_n = n; image_o = o;
        size_t sz = (size_t)m * n * o;
        float* im = load<float>(argv[2], sz);
        size_t sz1 = (size_t)(m / g) * (n / g) * (o / g);
        int* ordered = new int[sz1]; int* parents = new int[sz1]; float* edgemst = new float[sz1];
        primsGraph(im, ordered, parents, edgemst, g, m, n, o);
        save(argv[7], ordered, sz1); save(argv[8], parents, sz1); save(argv[9], edgemst, sz1);
    } else if (st == "reg") {
        // reg cost.f32 u0 v0 w0 ordered parents edgemst m n o g hw q  out_cost.f32 u1 v1 w1
        int m = atoi(argv[9]), n = atoi(argv[10]), o = atoi(argv[11]);
        int g = atoi(argv[12]), hw = atoi(argv[13]); float q = atof(argv[14]);
        image_m = m; image_n = n; image_o = o;
        size_t sz1 = (size_t)(m / g) * (n / g) * (o / g);
        int len3 = (int)pow(hw * 2 + 1, 3);
        float* cost = load<float>(argv[2], sz1 * len3);
        float* u0 = load<float>(argv[3], sz1); float* v0 = load<float>(argv[4], sz1); float* w0 = load<float>(argv[5], sz1);
        int* ordered = load<int>(argv[6], sz1); int* parents = load<int>(argv[7], sz1);
        float* edgemst = load<float>(argv[8], sz1);
        float* u1 = new float[sz1]; float* v1 = new float[sz1]; float* w1 = new float[sz1];
        regularisationCL(cost, u0, v0, w0, u1, v1, w1, hw, g, q, ordered, parents, edgemst);
        save(argv[15], cost, sz1 * len3);
        save(argv[16], u1, sz1); save(argv[17], v1, sz1); save(argv[18], w1, sz1);
    } else if (st == "upsample") {  // upsample u0 v0 w0 m2 n2 o2 m n o  u1 v1 w1
        int m2 = atoi(argv[5]), n2 = atoi(argv[6]), o2 = atoi(argv[7]);
        int m = atoi(argv[8]), n = atoi(argv[9]), o = atoi(argv[10]);
        size_t s2 = (size_t)m2 * n2 * o2, s = (size_t)m * n * o;
        float* u0 = load<float>(argv[2], s2); float* v0 = load<float>(argv[3], s2); float* w0 = load<float>(argv[4], s2);
        float* u1 = new float[s]; float* v1 = new float[s]; float* w1 = new float[s];
        upsampleDeformationsCL(u1, v1, w1, u0, v0, w0, m, n, o, m2, n2, o2);
        save(argv[11], u1, s); save(argv[12], v1, s); save(argv[13], w1, s);
    } else if (st == "warpaffine") {  // warpaffine in.f32 ref.f32 X.f32(16) u v w m n o out.f32
        int m = atoi(argv[8]), n = atoi(argv[9]), o = atoi(argv[10]);
        image_m = m; image_n = n; image_o = o;
        size_t s = (size_t)m * n * o;
        float* in = load<float>(argv[2], s); float* ref = load<float>(argv[3], s);
        float* X = load<float>(argv[4], 16);
        float* u = load<float>(argv[5], s); float* v = load<float>(argv[6], s); float* w = load<float>(argv[7], s);
        float* out = new float[s];
        warpAffine(out, in, ref, X, u, v, w);
        save(argv[11], out, s);
        printf("SSD0 %.9g SSD1 %.9g\n", SSD0, SSD1);
    } else if (st == "warpimage") {  // warpimage in.f32 ref.f32 u v w m n o out.f32
        int m = atoi(argv[7]), n = atoi(argv[8]), o = atoi(argv[9]);
        image_m = m; image_n = n; image_o = o;
        size_t s = (size_t)m * n * o;
        float* in = load<float>(argv[2], s); float* ref = load<float>(argv[3], s);
        float* u = load<float>(argv[4], s); float* v = load<float>(argv[5], s); float* w = load<float>(argv[6], s);
        float* out = new float[s];
        warpImageCL(out, in, ref, u, v, w);
        save(argv[10], out, s);
    } else if (st == "warpseg") {  // warpseg in.i16 X.f32 u v w m n o out.i16
        int m = atoi(argv[7]), n = atoi(argv[8]), o = atoi(argv[9]);
        image_m = m; image_n = n; image_o = o;
        size_t s = (size_t)m * n * o;
        short* in = load<short>(argv[2], s); float* X = load<float>(argv[3], 16);
        float* u = load<float>(argv[4], s); float* v = load<float>(argv[5], s); float* w = load<float>(argv[6], s);
        short* out = new short[s];
        warpAffineS(out, in, X, u, v, w);
        save(argv[10], out, s);
    } else if (st == "consistent") {  // consistent u v w u2 v2 w2 m n o g  (in place -> 6 outputs)
        int m = atoi(argv[8]), n = atoi(argv[9]), o = atoi(argv[10]), g = atoi(argv[11]);
        size_t s = (size_t)m * n * o;
        float* f[6];
        for (int i = 0; i < 6; i++) f[i] = load<float>(argv[2 + i], s);
        consistentMappingCL(f[0], f[1], f[2], f[3], f[4], f[5], m, n, o, g);
        for (int i = 0; i < 6; i++) save(argv[12 + i], f[i], s);
    } else if (st == "jacobian") {  // jacobian u v w m n o g
        int m = atoi(argv[5]), n = atoi(argv[6]), o = atoi(argv[7]), g = atoi(argv[8]);
        size_t s = (size_t)m * n * o;
        float* u = load<float>(argv[2], s); float* v = load<float>(argv[3], s); float* w = load<float>(argv[4], s);
        float j = jacobian(u, v, w, m, n, o, g);
        printf("\nJSTD %.9g\n", j);
    } else {
        fprintf(stderr, "unknown stage %s\n", st.c_str());
        return 2;
    }
    return 0;
}
