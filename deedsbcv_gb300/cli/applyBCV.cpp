// applyBCV / applyBCVfloat — apply a deeds displacement file to a volume
// (drop-in for src/applyBCV.cpp:54-204 and src/applyBCVfloat.cpp): reads
// stem_displacements.dat, infers the grid step from its size, upsamples the
// field and warps -M (int16 labels with nearest neighbour, or with APPLY_FLOAT a
// float image trilinearly) into -D, on the GPU.
#include <cstdio>
#include <string>
#include <vector>

#include "cli_common.h"
#include "deeds_gpu.h"

using namespace deeds_cli;

#ifndef APPLY_FLOAT
#define APPLY_FLOAT 0
#endif

int main(int argc, char** argv) {
    if (argc < 4 || (argv[1][0] == '-' && argv[1][1] == 'h')) {
        std::printf("=============================================================\n");
        std::printf("Usage (required input arguments):\n");
        std::printf(APPLY_FLOAT ? "./applyBCVfloat -M moving.nii.gz -O output -D deformed.nii.gz \n"
                                : "./applyBCV -M moving.nii.gz -O output -D deformed.nii.gz \n");
        std::printf("optional parameters:\n");
        std::printf(" -A <affine_matrix.txt> \n");
        std::printf("=============================================================\n");
        return 1;
    }
    Args a;
    if (!parse_args(argc, argv, a)) {
        for (auto& w : a.warnings) std::printf("%s\n", w.c_str());
        return -1;
    }
    if (!ends_with_gz(a.deformed_file) || !ends_with_gz(a.moving_file)) {
        std::printf("images must have nii.gz format\n");
        return -1;
    }
    std::string err;
    Volume v;
#if APPLY_FLOAT
    std::vector<float> in;
    if (!read_nifti_float(a.moving_file, v, in, err)) { std::printf("%s\n", err.c_str()); return -1; }
#else
    std::vector<int16_t> in;
    if (!read_nifti_short(a.moving_file, v, in, err)) { std::printf("%s\n", err.c_str()); return -1; }
#endif
    float X[16];
    if (a.affine) {
        if (!read_affine(a.affine_file, X, err)) { std::printf("%s\n", err.c_str()); return -1; }
    } else {
        std::printf("Using identity transform.\n");
        identity(X);
    }
    std::vector<float> flow;
    const std::string inputflow = a.output_stem + "_displacements.dat";
    std::printf("Reading displacements from:\n%s\n", inputflow.c_str());
    if (!read_raw_floats(inputflow, flow, err)) { std::printf("%s\n", err.c_str()); return -1; }
    deeds_ctx* ctx = nullptr;
    if (deeds_create(&ctx, 0) != DEEDS_OK) { std::printf("deeds: %s\n", deeds_last_error(nullptr)); return -1; }
    decltype(in) out(in.size());
    const int st = deeds_apply_flow(ctx, flow.data(), flow.size(), 0, X, in.data(), APPLY_FLOAT ? 1 : 0, v.m, v.n, v.o,
                                    out.data());
    if (st != DEEDS_OK) {
        std::printf("deeds: %s\n", deeds_last_error(ctx));
        deeds_destroy(ctx);
        return -1;
    }
#if APPLY_FLOAT
    const bool ok = write_nifti_float(a.deformed_file, v, out.data(), err);
#else
    const bool ok = write_nifti_short(a.deformed_file, v, out.data(), err);
#endif
    deeds_destroy(ctx);
    if (!ok) { std::printf("%s\n", err.c_str()); return -1; }
    return 0;
}
