// deedsBCV — command-line driver of the GB300 registration (drop-in for the
// reference's deedsBCV, src/deedsBCV0.cpp:55-385): same flags, same output files
// (stem_displacements.dat, stem_deformed.nii.gz, stem_deformed_seg.nii.gz).
// All registration work runs in libdeeds_gpu.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cli_common.h"
#include "deeds_gpu.h"

using namespace deeds_cli;

static void usage() {
    std::printf("=============================================================\n");
    std::printf("Usage (required input arguments):\n");
    std::printf("./deedsBCV -F fixed.nii.gz -M moving.nii.gz -O output\n");
    std::printf("optional parameters:\n");
    std::printf(" -a <regularisation parameter alpha> (default 1.6)\n");
    std::printf(" -l <number of levels> (default 5)\n");
    std::printf(" -G <grid spacing for each level> (default 8x7x6x5x4)\n");
    std::printf(" -L <maximum search radius - each level> (default 8x7x6x5x4)\n");
    std::printf(" -Q <quantisation of search step size> (default 5x4x3x2x1)\n");
    std::printf(" -S <moving_segmentation.nii> (short int)\n");
    std::printf(" -A <affine_matrix.txt> \n");
    std::printf("=============================================================\n");
}

int main(int argc, char** argv) {
    if (argc < 4 || (argv[1][0] == '-' && argv[1][1] == 'h')) {
        usage();
        return 1;
    }
    Args a;
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
    float X[16];
    if (a.affine) {
        if (!read_affine(a.affine_file, X, err)) { std::printf("%s\n", err.c_str()); return -1; }
    } else {
        std::printf("Starting with identity transform.\n");
        identity(X);
    }
    std::string lv[3];
    for (int l = 0; l < a.levels; l++) {
        const char* sep = l ? "x" : "";
        lv[0] += sep + std::to_string(a.grid[l]);
        lv[1] += sep + std::to_string(a.search[l]);
        lv[2] += sep + std::to_string(a.quant[l]);
    }
    std::printf("levels=%d G=%s L=%s Q=%s alpha=%g\n", a.levels, lv[0].c_str(), lv[1].c_str(), lv[2].c_str(),
                a.alpha);
    deeds_params p;
    deeds_default_params(&p);
    p.levels = a.levels;
    for (int l = 0; l < a.levels; l++) { p.grid[l] = a.grid[l]; p.radius[l] = a.search[l]; p.quant[l] = a.quant[l]; }
    p.alpha = a.alpha;
    p.verbose = 1;
    deeds_ctx* ctx = nullptr;
    if (deeds_create(&ctx, 0) != DEEDS_OK) {
        std::printf("deeds: %s\n", deeds_last_error(nullptr));
        return -1;
    }
    const int gl = p.grid[p.levels - 1];
    const size_t sz = (size_t)m * n * o, sz1 = (size_t)(m / gl) * (n / gl) * (o / gl);
    std::vector<float> flow(3 * sz1), warped(sz);
    const auto t0 = std::chrono::steady_clock::now();
    if (deeds_register(ctx, fixed.data(), moving.data(), m, n, o, X, &p, flow.data(), warped.data()) != DEEDS_OK) {
        std::printf("deeds: %s\n", deeds_last_error(ctx));
        deeds_destroy(ctx);
        return -1;
    }
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (!write_raw(a.output_stem + "_displacements.dat", flow.data(), flow.size() * sizeof(float), err) ||
        !write_nifti_float(a.output_stem + "_deformed.nii.gz", vf, warped.data(), err)) {
        std::printf("%s\n", err.c_str());
        deeds_destroy(ctx);
        return -1;
    }
    if (a.segment) {
        Volume vs;
        std::vector<int16_t> seg;
        if (!read_nifti_short(a.moving_seg_file, vs, seg, err) || vs.m != m || vs.n != n || vs.o != o) {
            std::printf("%s\n", err.empty() ? "segmentation size mismatch" : err.c_str());
            deeds_destroy(ctx);
            return -1;
        }
        std::vector<int16_t> segw(sz);
        if (deeds_warp_segmentation(ctx, seg.data(), segw.data()) != DEEDS_OK) {
            std::printf("deeds: %s\n", deeds_last_error(ctx));
            deeds_destroy(ctx);
            return -1;
        }
        const std::string outseg = a.output_stem + "_deformed_seg.nii.gz";
        std::printf("outputseg %s\n", outseg.c_str());
        if (!write_nifti_short(outseg, vf, segw.data(), err)) { std::printf("%s\n", err.c_str()); return -1; }
    }
    std::printf("Finished. Total time: %g sec.\n", secs);
    deeds_destroy(ctx);
    return 0;
}
