// Shared pieces of the deedsBCV / applyBCV command-line drivers: argument
// parsing with the reference's semantics (src/parseArguments.h:12-174), NIfTI-1
// (.nii / .nii.gz) IO (src/imageIOgzType.h) and the affine matrix file
// (src/deedsBCV0.cpp:150-174).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace deeds_cli {

struct Args {
    float alpha = 1.6f;
    int levels = 5;
    bool segment = false, affine = false;
    int rigid = 0;
    std::vector<int> grid{8, 7, 6, 5, 4}, search{8, 7, 6, 5, 4}, quant{5, 4, 3, 2, 1};
    std::string fixed_file, moving_file, output_stem, moving_seg_file, affine_file, deformed_file;
    int required = 0;
    std::vector<std::string> warnings;
};

// Parse argv like parseCommandLine(): single-letter flags F M O a l G L Q S A R D,
// level lists "8x7x6x5x4" (up to 10), the level count taken from -G when any of
// -G/-L/-Q is given, defaults 8..2 / 8..1 / 5..1 beyond the given entries.
// Returns false on a malformed command line (missing flag value).
bool parse_args(int argc, char** argv, Args& a);

struct Volume {
    int m = 0, n = 0, o = 0, p = 1;
    std::vector<char> header;  // 352 bytes
};

// Read a NIfTI-1 volume (gz or plain) as float or int16; datatypes 2,4,8,16,64,512.
bool read_nifti_float(const std::string& path, Volume& v, std::vector<float>& data, std::string& err);
bool read_nifti_short(const std::string& path, Volume& v, std::vector<int16_t>& data, std::string& err);
// Write float32 (datatype 16) or int16 (datatype 4) volumes with a correct 352-byte header.
bool write_nifti_float(const std::string& path, const Volume& like, const float* data, std::string& err);
bool write_nifti_short(const std::string& path, const Volume& like, const int16_t* data, std::string& err);

// 4 lines of "a b c d": line i fills X[i], X[i+4], X[i+8], X[i+12].
bool read_affine(const std::string& path, float X[16], std::string& err);
void identity(float X[16]);

bool write_raw(const std::string& path, const void* data, size_t bytes, std::string& err);
bool read_raw_floats(const std::string& path, std::vector<float>& out, std::string& err);

bool ends_with_gz(const std::string& s);

}  // namespace deeds_cli
