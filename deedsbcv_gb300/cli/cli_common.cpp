#include "cli_common.h"

#include "deeds_gpu.h"

#include <zlib.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace deeds_cli {

bool ends_with_gz(const std::string& s) { return s.size() >= 2 && s.compare(s.size() - 2, 2, "gz") == 0; }

static int parse_levels(const char* s, std::vector<int>& dst) {
    // sscanf("%dx%dx...") semantics: leading entries until the first mismatch
    int count = 0;
    const char* p = s;
    while (count < 10) {
        char* end = nullptr;
        long v = std::strtol(p, &end, 10);
        if (end == p) break;
        dst[count++] = (int)v;
        if (*end != 'x') break;
        p = end + 1;
    }
    return count;
}

bool parse_args(int argc, char** argv, Args& a) {
    // defaults beyond the first five levels (src/parseArguments.h:42-44)
    std::vector<int> g{8, 7, 6, 5, 4, 3, 2, 2, 2, 2}, s{8, 7, 6, 5, 4, 3, 2, 1, 1, 0}, q{5, 4, 3, 2, 1, 1, 1, 1, 1, 1};
    int maxlevel = a.levels;
    for (int i = 0; i < maxlevel && i < 10; i++) { g[i] = a.grid[i]; s[i] = a.search[i]; q[i] = a.quant[i]; }
    int num = maxlevel, num2 = maxlevel, num3 = maxlevel;
    bool s_set = false;
    for (int k = 1; k < argc; k++) {
        if (argv[k][0] != '-') continue;
        const char f = argv[k][1];
        const char* known = "FMOalGLQSARD";
        if (f == 0 || !std::strchr(known, f)) {
            a.warnings.push_back(std::string("Invalid option: ") + argv[k] + " use -h for help");
            continue;
        }
        if (k + 1 >= argc) {
            a.warnings.push_back(std::string("Missing value for ") + argv[k]);
            return false;
        }
        const char* v = argv[k + 1];
        switch (f) {
            case 'F': a.fixed_file = v; a.required++; break;
            case 'M': a.moving_file = v; a.required++; break;
            case 'O': a.output_stem = v; a.required++; break;
            case 'a': a.alpha = (float)std::atof(v); break;
            case 'l': maxlevel = std::atoi(v); break;
            case 'G': num = parse_levels(v, g); s_set = true; break;
            case 'L': num2 = parse_levels(v, s); s_set = true; break;
            case 'Q': num3 = parse_levels(v, q); s_set = true; break;
            case 'S': a.moving_seg_file = v; a.segment = true; break;
            case 'A': a.affine_file = v; a.affine = true; break;
            case 'R': a.rigid = std::atoi(v); break;
            case 'D': a.deformed_file = v; a.required++; break;
        }
    }
    if (s_set) maxlevel = num;  // the level count follows -G (src/parseArguments.h:122-124)
    if (num != maxlevel || num2 != maxlevel || num3 != maxlevel) {
        char buf[160];
        std::snprintf(buf, sizeof(buf), "maxlevel=%d, #grid=%d, #search=%d, #quant=%d", maxlevel, num, num2, num3);
        a.warnings.push_back("Max level and number of grid-spacing, search range or quantisation steps are not equal.");
        a.warnings.push_back(buf);
    }
    if (maxlevel < 1) maxlevel = 1;
    if (maxlevel > 10) maxlevel = 10;
    a.levels = maxlevel;
    a.grid.assign(g.begin(), g.begin() + maxlevel);
    a.search.assign(s.begin(), s.begin() + maxlevel);
    a.quant.assign(q.begin(), q.begin() + maxlevel);
    return true;
}

namespace {

// Worker threads for gzip IO: DEEDS_GZ_THREADS, else every core.
int gz_threads() {
    const char* e = std::getenv("DEEDS_GZ_THREADS");
    return e ? std::atoi(e) : 0;
}

// The whole decompressed file (gzip or plain) through the library's parallel
// reader; the buffer is sized from the gzip ISIZE trailer, so a single-member
// file is inflated once.
bool slurp(const std::string& path, std::vector<char>& raw, std::string& err) {
    size_t hint = 0;
    if (FILE* f = std::fopen(path.c_str(), "rb")) {
        unsigned char mag[2] = {0, 0}, tr[4] = {0, 0, 0, 0};
        std::fseek(f, 0, SEEK_END);
        const long n = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        const bool gz = std::fread(mag, 1, 2, f) == 2 && mag[0] == 0x1f && mag[1] == 0x8b;
        if (gz && n >= 4 && std::fseek(f, n - 4, SEEK_SET) == 0 && std::fread(tr, 1, 4, f) == 4)
            hint = (size_t)tr[0] | ((size_t)tr[1] << 8) | ((size_t)tr[2] << 16) | ((size_t)tr[3] << 24);
        if (!gz || hint > (size_t)n * 64 + (1u << 20)) hint = (size_t)std::max<long>(n, 0) * (gz ? 4 : 1);
        std::fclose(f);
    } else {
        err = "gzopen of '" + path + "' failed.";
        return false;
    }
    raw.resize(std::max<size_t>(hint, 352));
    size_t total = 0;
    deeds_status st = deeds_gz_read(path.c_str(), raw.data(), raw.size(), &total, gz_threads());
    if (st != DEEDS_OK && total > raw.size()) {  // more than the trailer said (several members)
        raw.resize(total);
        st = deeds_gz_read(path.c_str(), raw.data(), raw.size(), &total, gz_threads());
    }
    if (st != DEEDS_OK) {
        err = path + ": " + deeds_gz_last_error();
        return false;
    }
    raw.resize(total);
    return true;
}

bool parse_header(const std::vector<char>& raw, const std::string& path, Volume& v, short& dtype, size_t& data_off,
                  std::string& err) {
    if (raw.size() < 352) { err = path + ": truncated header"; return false; }
    v.header.assign(raw.begin(), raw.begin() + 352);
    short dims[8];
    std::memcpy(dims, v.header.data() + 40, sizeof(dims));
    std::memcpy(&dtype, v.header.data() + 70, 2);
    v.m = dims[1]; v.n = dims[2]; v.o = dims[3]; v.p = dims[4] > 0 ? dims[4] : 1;
    if (v.m < 1 || v.n < 1 || v.o < 1) { err = path + ": bad dimensions"; return false; }
    float vox_offset = 352.0f;
    std::memcpy(&vox_offset, v.header.data() + 108, 4);
    data_off = std::max<size_t>(352, (size_t)vox_offset);
    return true;
}

template <class T>
bool read_nifti(const std::string& path, Volume& v, std::vector<T>& out, std::string& err) {
    std::vector<char> raw;
    if (!slurp(path, raw, err)) return false;
    short dtype = 0;
    size_t off = 0;
    if (!parse_header(raw, path, v, dtype, off, err)) return false;
    const size_t count = (size_t)v.m * v.n * v.o * v.p;
    size_t esz;
    switch (dtype) {
        case 2: esz = 1; break;
        case 4: case 512: esz = 2; break;
        case 8: case 16: esz = 4; break;
        case 64: esz = 8; break;
        default: err = "Datatype " + std::to_string(dtype) + " not supported."; return false;
    }
    if (raw.size() < off + count * esz) { err = path + ": truncated data"; return false; }
    out.resize(count);
    for (size_t i = 0; i < count; i++) {
        const char* p = raw.data() + off + i * esz;
        switch (dtype) {
            case 2: out[i] = (T)(*(const uint8_t*)p); break;
            case 4: { int16_t x; std::memcpy(&x, p, 2); out[i] = (T)x; } break;
            case 512: { uint16_t x; std::memcpy(&x, p, 2); out[i] = (T)x; } break;
            case 8: { int32_t x; std::memcpy(&x, p, 4); out[i] = (T)x; } break;
            case 16: { float x; std::memcpy(&x, p, 4); out[i] = (T)x; } break;
            case 64: { double x; std::memcpy(&x, p, 8); out[i] = (T)x; } break;
        }
    }
    return true;
}

bool write_nifti(const std::string& path, const Volume& like, const void* data, size_t bytes, short dtype,
                 short bitpix, std::string& err) {
    std::vector<char> h(like.header);
    h.resize(352, 0);
    const int32_t hsz = 348;
    std::memcpy(h.data(), &hsz, 4);
    short dims[8] = {(short)(like.o > 1 ? 3 : 2), (short)like.m, (short)like.n, (short)like.o, 1, 1, 1, 1};
    std::memcpy(h.data() + 40, dims, sizeof(dims));
    std::memcpy(h.data() + 70, &dtype, 2);
    std::memcpy(h.data() + 72, &bitpix, 2);
    const float off = 352.0f;
    std::memcpy(h.data() + 108, &off, 4);
    if (ends_with_gz(path)) {
        if (deeds_gz_write(path.c_str(), h.data(), 352, data, bytes, Z_DEFAULT_COMPRESSION, gz_threads()) != DEEDS_OK) {
            err = "File error. Could not write " + path + ": " + deeds_gz_last_error();
            return false;
        }
        return true;
    }
    std::ofstream f(path, std::ios::binary);
    if (!f) { err = "File error. Could not write " + path; return false; }
    f.write(h.data(), 352);
    f.write(static_cast<const char*>(data), (std::streamsize)bytes);
    return (bool)f;
}

}  // namespace

bool read_nifti_float(const std::string& path, Volume& v, std::vector<float>& data, std::string& err) {
    return read_nifti(path, v, data, err);
}
bool read_nifti_short(const std::string& path, Volume& v, std::vector<int16_t>& data, std::string& err) {
    return read_nifti(path, v, data, err);
}
bool write_nifti_float(const std::string& path, const Volume& like, const float* data, std::string& err) {
    return write_nifti(path, like, data, sizeof(float) * like.m * like.n * like.o, 16, 32, err);
}
bool write_nifti_short(const std::string& path, const Volume& like, const int16_t* data, std::string& err) {
    return write_nifti(path, like, data, sizeof(int16_t) * like.m * like.n * like.o, 4, 16, err);
}

void identity(float X[16]) {
    for (int i = 0; i < 16; i++) X[i] = 0.0f;
    X[0] = X[5] = X[10] = X[15] = 1.0f;
}

bool read_affine(const std::string& path, float X[16], std::string& err) {
    std::ifstream f(path);
    if (!f) { err = "cannot open affine matrix " + path; return false; }
    for (int i = 0; i < 4; i++) {
        std::string line;
        if (!std::getline(f, line)) { err = "affine matrix " + path + " has fewer than 4 lines"; return false; }
        if (std::sscanf(line.c_str(), "%f  %f  %f  %f", &X[i], &X[i + 4], &X[i + 8], &X[i + 12]) != 4) {
            err = "affine matrix " + path + ": bad line " + std::to_string(i + 1);
            return false;
        }
    }
    return true;
}

bool write_raw(const std::string& path, const void* data, size_t bytes, std::string& err) {
    std::ofstream f(path, std::ios::binary);
    if (!f) { err = "cannot write " + path; return false; }
    f.write(static_cast<const char*>(data), (std::streamsize)bytes);
    return (bool)f;
}

bool read_raw_floats(const std::string& path, std::vector<float>& out, std::string& err) {
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    if (!f) { err = "readFile error. Did not find " + path; return false; }
    const std::streamsize len = f.tellg();
    f.seekg(0);
    out.resize((size_t)len / sizeof(float));
    f.read(reinterpret_cast<char*>(out.data()), (std::streamsize)(out.size() * sizeof(float)));
    return (bool)f;
}

}  // namespace deeds_cli
