// Parallel gzip IO for the NIfTI volumes of the command-line drivers (the
// reference reads and writes them with single-threaded zlib,
// src/imageIOgzType.h:14-26, 212-218).
//
// Writing: the stream is cut into chunks that worker threads deflate
// independently; each chunk becomes one complete gzip member (RFC 1952), and
// concatenated members are a valid gzip file that zlib's gzread, gzip(1) and
// Python's gzip module read as one stream.  Each member's header carries an
// extra subfield 'D','G' holding the member's total length, so a reader can
// find every member without inflating (readers that do not know the subfield
// skip it, as RFC 1952 requires).
//
// Reading: files whose members all carry the subfield are inflated in parallel
// into their final offsets (each member's uncompressed size is its ISIZE
// trailer); any other gzip file goes through zlib's sequential gzread.
#include <zlib.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/deeds_gpu.h"

namespace {

constexpr size_t kChunk = 4u << 20;  // uncompressed bytes per member
constexpr int kHeaderLen = 10 + 2 + 8;  // fixed header, XLEN, one 8-byte subfield

void put32(unsigned char* p, uint32_t v) {
    p[0] = (unsigned char)v; p[1] = (unsigned char)(v >> 8); p[2] = (unsigned char)(v >> 16); p[3] = (unsigned char)(v >> 24);
}
uint32_t get32(const unsigned char* p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

int worker_count(int threads, size_t jobs) {
    int t = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
    if (t < 1) t = 1;
    return (int)std::min<size_t>((size_t)t, std::max<size_t>(jobs, 1));
}

// Run fn(i) for i in [0, n) on `workers` threads.
template <class Fn>
void parallel_for(size_t n, int workers, Fn fn) {
    std::atomic<size_t> next{0};
    auto body = [&]() {
        for (size_t i = next++; i < n; i = next++) fn(i);
    };
    std::vector<std::thread> pool;
    for (int w = 1; w < workers; w++) pool.emplace_back(body);
    body();
    for (auto& t : pool) t.join();
}

// One member: header with the 'DG' length subfield, raw deflate data, CRC32, ISIZE.
bool deflate_member(const unsigned char* src, size_t n, int level, std::vector<unsigned char>& out) {
    z_stream zs;
    std::memset(&zs, 0, sizeof(zs));
    if (deflateInit2(&zs, level, Z_DEFLATED, -15, 8, Z_DEFAULT_STRATEGY) != Z_OK) return false;
    const size_t bound = deflateBound(&zs, (uLong)n);
    out.resize(kHeaderLen + bound + 8);
    zs.next_in = const_cast<unsigned char*>(src);
    zs.avail_in = (uInt)n;
    zs.next_out = out.data() + kHeaderLen;
    zs.avail_out = (uInt)bound;
    const int rc = deflate(&zs, Z_FINISH);
    const size_t clen = zs.total_out;
    deflateEnd(&zs);
    if (rc != Z_STREAM_END) return false;
    unsigned char* h = out.data();
    h[0] = 0x1f; h[1] = 0x8b; h[2] = 8; h[3] = 4;  // deflate, FEXTRA
    put32(h + 4, 0);                                 // no modification time
    h[8] = 0; h[9] = 255;                            // OS unknown
    h[10] = 8; h[11] = 0;                            // XLEN
    h[12] = 'D'; h[13] = 'G'; h[14] = 4; h[15] = 0;  // subfield id, length
    const size_t total = kHeaderLen + clen + 8;
    put32(h + 16, (uint32_t)total);
    unsigned char* t = out.data() + kHeaderLen + clen;
    put32(t, (uint32_t)crc32(crc32(0L, Z_NULL, 0), src, (uInt)n));
    put32(t + 4, (uint32_t)n);
    out.resize(total);
    return true;
}

struct Member {
    size_t off, len;       // in the compressed file
    size_t out_off, out_len;
};

// Walk the members of an in-memory file; false unless every member carries the
// 'DG' subfield with a consistent length.
bool index_members(const std::vector<unsigned char>& f, std::vector<Member>& ms) {
    size_t pos = 0, out = 0;
    while (pos < f.size()) {
        if (f.size() - pos < (size_t)kHeaderLen + 8) return false;
        const unsigned char* h = f.data() + pos;
        if (h[0] != 0x1f || h[1] != 0x8b || h[2] != 8 || h[3] != 4) return false;
        if (h[10] != 8 || h[11] != 0 || h[12] != 'D' || h[13] != 'G' || h[14] != 4 || h[15] != 0) return false;
        const size_t len = get32(h + 16);
        if (len < (size_t)kHeaderLen + 8 || len > f.size() - pos) return false;
        const size_t isize = get32(h + len - 4);
        ms.push_back(Member{pos, len, out, isize});
        out += isize;
        pos += len;
    }
    return !ms.empty();
}

bool read_file(const char* path, std::vector<unsigned char>& f) {
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return false;
    std::fseek(fp, 0, SEEK_END);
    const long n = std::ftell(fp);
    std::fseek(fp, 0, SEEK_SET);
    if (n < 0) { std::fclose(fp); return false; }
    f.resize((size_t)n);
    const size_t got = n ? std::fread(f.data(), 1, (size_t)n, fp) : 0;
    std::fclose(fp);
    return got == (size_t)n;
}

bool inflate_member(const unsigned char* m, size_t len, unsigned char* dst, size_t isize) {
    z_stream zs;
    std::memset(&zs, 0, sizeof(zs));
    if (inflateInit2(&zs, -15) != Z_OK) return false;
    zs.next_in = const_cast<unsigned char*>(m + kHeaderLen);
    zs.avail_in = (uInt)(len - kHeaderLen - 8);
    zs.next_out = dst;
    zs.avail_out = (uInt)isize;
    const int rc = inflate(&zs, Z_FINISH);
    const bool ok = rc == Z_STREAM_END && zs.total_out == isize;
    inflateEnd(&zs);
    return ok && (uint32_t)crc32(crc32(0L, Z_NULL, 0), dst, (uInt)isize) == get32(m + len - 8);
}

thread_local std::string g_gz_err;

}  // namespace

extern "C" {

deeds_status deeds_gz_write(const char* path, const void* head, size_t head_bytes, const void* data,
                            size_t data_bytes, int level, int threads) {
    if (!path || (head_bytes && !head) || (data_bytes && !data)) return DEEDS_ERR_INVALID;
    // logical stream = head ++ data, cut into chunks
    const size_t total = head_bytes + data_bytes;
    const size_t nchunk = std::max<size_t>(1, (total + kChunk - 1) / kChunk);
    std::vector<std::vector<unsigned char>> outs(nchunk);
    std::vector<unsigned char> first;  // the chunk that straddles head and data, assembled
    std::atomic<bool> ok{true};
    auto chunk_ptr = [&](size_t c, size_t& n) -> const unsigned char* {
        const size_t lo = c * kChunk, hi = std::min(total, lo + kChunk);
        n = hi - lo;
        if (lo >= head_bytes) return static_cast<const unsigned char*>(data) + (lo - head_bytes);
        return nullptr;  // overlaps the head: assembled below
    };
    if (head_bytes) {  // chunks that overlap the head are small and few: copy them into one buffer
        const size_t hi = std::min(total, ((head_bytes + kChunk - 1) / kChunk) * kChunk);
        first.resize(hi);
        std::memcpy(first.data(), head, head_bytes);
        if (hi > head_bytes) std::memcpy(first.data() + head_bytes, data, hi - head_bytes);
    }
    parallel_for(nchunk, worker_count(threads, nchunk), [&](size_t c) {
        size_t n = 0;
        const unsigned char* p = chunk_ptr(c, n);
        if (!p) p = first.data() + c * kChunk;
        if (!deflate_member(p, n, level, outs[c])) ok = false;
    });
    if (!ok) { g_gz_err = "deflate failed"; return DEEDS_ERR_INTERNAL; }
    FILE* fp = std::fopen(path, "wb");
    if (!fp) { g_gz_err = std::string("cannot write ") + path; return DEEDS_ERR_INVALID; }
    bool wok = true;
    for (auto& o : outs) wok = wok && std::fwrite(o.data(), 1, o.size(), fp) == o.size();
    wok = (std::fclose(fp) == 0) && wok;
    if (!wok) { g_gz_err = std::string("write error on ") + path; return DEEDS_ERR_INTERNAL; }
    return DEEDS_OK;
}

deeds_status deeds_gz_read(const char* path, void* out, size_t cap, size_t* total, int threads) {
    if (!path || !total) return DEEDS_ERR_INVALID;
    std::vector<unsigned char> f;
    if (!read_file(path, f)) { g_gz_err = std::string("cannot read ") + path; return DEEDS_ERR_INVALID; }
    std::vector<Member> ms;
    if (index_members(f, ms)) {
        const size_t n = ms.back().out_off + ms.back().out_len;
        *total = n;
        if (!out) return DEEDS_OK;
        if (cap < n) return DEEDS_ERR_INVALID;
        std::atomic<bool> ok{true};
        unsigned char* dst = static_cast<unsigned char*>(out);
        parallel_for(ms.size(), worker_count(threads, ms.size()), [&](size_t i) {
            if (!inflate_member(f.data() + ms[i].off, ms[i].len, dst + ms[i].out_off, ms[i].out_len)) ok = false;
        });
        if (!ok) { g_gz_err = std::string("corrupt gzip member in ") + path; return DEEDS_ERR_INTERNAL; }
        return DEEDS_OK;
    }
    // any other gzip (or plain) file: zlib's sequential reader, twice if the size is asked first
    gzFile g = gzopen(path, "rb");
    if (!g) { g_gz_err = std::string("gzopen of ") + path + " failed"; return DEEDS_ERR_INVALID; }
    size_t n = 0;
    bool overflow = false;
    unsigned char* dst = static_cast<unsigned char*>(out);
    for (;;) {
        unsigned char tmp[1 << 16];
        unsigned char* w = (dst && !overflow && cap - std::min(cap, n) >= sizeof(tmp)) ? dst + n : tmp;
        const int rd = gzread(g, w, sizeof(tmp));
        if (rd < 0) { gzclose(g); g_gz_err = std::string("gzread error on ") + path; return DEEDS_ERR_INTERNAL; }
        if (rd == 0) break;
        if (dst && w == tmp) {
            if (n + (size_t)rd > cap) overflow = true;  // keep counting: *total reports the full size
            else std::memcpy(dst + n, tmp, (size_t)rd);
        }
        n += (size_t)rd;
    }
    gzclose(g);
    *total = n;
    if (overflow) { g_gz_err = std::string("buffer too small for ") + path; return DEEDS_ERR_INVALID; }
    return DEEDS_OK;
}

const char* deeds_gz_last_error(void) { return g_gz_err.c_str(); }

}  // extern "C"
