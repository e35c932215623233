// linearBCV — command-line driver of the GB300 affine / rigid pre-registration
// (drop-in for the reference's linearBCV, src/linearBCV.cpp:64-325): same flags
// (-F -M -O [-R 1] [-l] [-G] [-L] [-Q] [-S seg]), same output files
// (stem_matrix.txt for deedsBCV -A, stem_deformed_seg.nii.gz).  All registration
// work runs in libdeeds_gpu.
#include <chrono>
#include <cstdio>
#include <string>
#include <vector>

#include "cli_common.h"
#include "deeds_gpu.h"

using namespace deeds_cli;

static void usage() {
    std::printf("=============================================================\n");
    std::printf("Usage (required input arguments):\n");
    std::printf("./linearBCV -F fixed.nii.gz -M moving.nii.gz -O output\n");
    std::printf("optional parameters:\n");
    std::printf(" -R <find rigid instead of affine transform> (default 0)\n");
    std::printf(" -l <number of levels> (default 4)\n");
    std::printf(" -G <grid spacing for each level> (default 7x6x5x4)\n");
    std::printf(" -L <maximum search radius - each level> (default 5x4x3x2)\n");
    std::printf(" -Q <quantisation of search step size> (default 4x3x2x1)\n");
    std::printf("=============================================================\n");
}

static std::string base_name(const std::string& p) {
    const size_t k = p.find_last_of("/\\");
    return k == std::string::npos ? p : p.substr(k + 1);
}

int main(int argc, char** argv) {
    if (argc < 4 || argv[1][1] == 'h') {
        usage();
        return 1;
    }
    Args a;  // linearBCV's defaults (src/linearBCV.cpp:86-89)
    a.levels = 4;
    a.grid = {7, 6, 5, 4};
    a.search = {5, 4, 3, 2};
    a.quant = {4, 3, 2, 1};
    if (!parse_args(argc, argv, a)) {
        for (auto& w : a.warnings) std::printf("%s\n", w.c_str());
        return -1;
    }
    for (auto& w : a.warnings) std::printf("%s\n", w.c_str());
    if (a.required != 3) std::printf("Missing argmuents, use -h for help.\n");
    if (!ends_with_gz(a.fixed_file) || !ends_with_gz(a.moving_file)) {
        std::printf("images must have nii.gz format\n");
        return -1;
    }
    std::printf("Starting linear reg. of %s and %s\n", base_name(a.fixed_file).c_str(),
                base_name(a.moving_file).c_str());
    std::printf("=============================================================\n");
    if (a.rigid) std::printf("Searching only for rigid (6 parameter) transform\n");
    std::string err;
    Volume vf, vm;
    std::vector<float> fixed, moving;
    if (!read_nifti_float(a.fixed_file, vf, fixed, err) || !read_nifti_float(a.moving_file, vm, moving, err)) {
        std::printf("%s\n", err.c_str());
        return -1;
    }
    if (vf.m != vm.m || vf.n != vm.n || vf.o != vm.o) {
        std::printf("Inconsistent image sizes (must have same dimensions)\n");
        return -1;
    }
    const int m = vf.m, n = vf.n, o = vf.o;
    std::string lv[3];
    for (int l = 0; l < a.levels; l++) {
        const char* sep = l ? "x" : "";
        lv[0] += sep + std::to_string(a.grid[l]);
        lv[1] += sep + std::to_string(a.search[l]);
        lv[2] += sep + std::to_string(a.quant[l]);
    }
    std::printf("levels=%d G=%s L=%s Q=%s %s\n", a.levels, lv[0].c_str(), lv[1].c_str(), lv[2].c_str(),
                a.rigid ? "rigid" : "affine");
    deeds_linear_params p;
    deeds_linear_default_params(&p);
    p.levels = a.levels;
    for (int l = 0; l < a.levels; l++) { p.grid[l] = a.grid[l]; p.radius[l] = a.search[l]; p.quant[l] = a.quant[l]; }
    p.rigid = a.rigid != 0;
    p.verbose = 1;
    deeds_ctx* ctx = nullptr;
    if (deeds_create(&ctx, 0) != DEEDS_OK) {
        std::printf("deeds: %s\n", deeds_last_error(nullptr));
        return -1;
    }
    float X[16];
    const auto t0 = std::chrono::steady_clock::now();
    if (deeds_linear_register(ctx, fixed.data(), moving.data(), m, n, o, &p, X) != DEEDS_OK) {
        std::printf("deeds: %s\n", deeds_last_error(ctx));
        deeds_destroy(ctx);
        return -1;
    }
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    // the matrix file: line i holds X[i] X[i+4] X[i+8] X[i+12] (src/linearBCV.cpp:281-294)
    const std::string outfile = a.output_stem + "_matrix.txt";
    FILE* f = std::fopen(outfile.c_str(), "w");
    if (!f) {
        std::printf("cannot write %s\n", outfile.c_str());
        deeds_destroy(ctx);
        return -1;
    }
    for (int i = 0; i < 4; i++) {
        std::fprintf(f, "%g  %g  %g  %g\n", X[i], X[i + 4], X[i + 8], X[i + 12]);
        std::printf("%+4.3f | %+4.3f | %+4.3f | %+4.3f \n", X[i], X[i + 4], X[i + 8], X[i + 12]);
    }
    std::fclose(f);
    if (a.segment) {
        Volume vs;
        std::vector<int16_t> seg;
        if (!read_nifti_short(a.moving_seg_file, vs, seg, err) || vs.m != m || vs.n != n || vs.o != o) {
            std::printf("%s\n", err.empty() ? "segmentation size mismatch" : err.c_str());
            deeds_destroy(ctx);
            return -1;
        }
        std::vector<int16_t> segw((size_t)m * n * o);
        if (deeds_affine_warp_segmentation(ctx, seg.data(), m, n, o, X, segw.data()) != DEEDS_OK) {
            std::printf("deeds: %s\n", deeds_last_error(ctx));
            deeds_destroy(ctx);
            return -1;
        }
        if (!write_nifti_short(a.output_stem + "_deformed_seg.nii.gz", vf, segw.data(), err)) {
            std::printf("%s\n", err.c_str());
            deeds_destroy(ctx);
            return -1;
        }
    }
    std::printf("Finished. Total time: %g sec.\n", secs);
    deeds_destroy(ctx);
    return 0;
}
