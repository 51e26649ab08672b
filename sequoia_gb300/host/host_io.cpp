// host_io.cpp -- the OBJ loader and BMP writer of the drop-in (sequoia_host.h).
//
// OBJ: the reference reads the file with fgets() into a 256-byte buffer and
// splits each line with gstrtok (src/main.cpp:88-179).  The parse here keeps
// those semantics token for token (see sequoia_host.h) but splits the file
// into chunks at newline boundaries -- a newline always ends an fgets() line,
// so chunk starts are line starts -- and parses the chunks in parallel.  The
// only cross-chunk state is the vertex count that negative indices are
// relative to; each chunk resolves them against its local count and adds its
// vertex base afterwards (index arithmetic is modulo 2^32 in both, as the
// reference's int/unsigned mix is).
//
// BMP: the reference writes through stb_image_write with vertical flip on
// (src/main.cpp:335-336).  The file written here is the plain Windows BMP
// format for that case: 14-byte file header, 40-byte info header, 24 bits per
// pixel, B G R order, each row padded to a multiple of 4 bytes.  BMP rows run
// bottom-up; with the flip, rgb row 0 is the first row in the file.
#include "sequoia_host.h"

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

namespace {

thread_local std::string g_error;

sq_status host_fail(sq_status s, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_error = buf;
    return s;
}

// fgets(line, 256, fp) reads at most 255 characters and stops after '\n'.
constexpr size_t kLineMax = 255;

struct Token {
    const char* p = nullptr;
    size_t len = 0;
    bool ok = false;
};

// gstrtok (src/main.cpp:88-106): the token runs from *s to the first
// delimiter, which is consumed; no delimiter before the end of the line means
// no token (and *s is left at the end).
inline Token next_token(const char*& s, const char* e, bool first)
{
    const char* b = s;
    for (; s < e; ++s) {
        const char c = *s;
        if (c == ' ' || c == '\t' || c == '\n' || (first && c == '\r')) {
            Token t;
            t.p = b;
            t.len = (size_t)(s - b);
            t.ok = true;
            ++s;
            return t;
        }
    }
    return Token();
}

// atof / atoi on a NUL-terminated copy of the token, as the reference calls
// them on gstrtok's static buffer
inline float token_float_libc(const Token& t)
{
    char buf[kLineMax + 1];
    memcpy(buf, t.p, t.len);
    buf[t.len] = '\0';
    return (float)strtod(buf, nullptr);
}

inline int token_int_libc(const Token& t)
{
    char buf[kLineMax + 1];
    memcpy(buf, t.p, t.len);
    buf[t.len] = '\0';
    return (int)strtol(buf, nullptr, 10);
}

// Exact powers of ten in double (10^0 .. 10^22 are all representable).
constexpr double kPow10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                               1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};

// (float)atof(token) without the library call for plain decimals, by
// Clinger's fast path (W. D. Clinger, "How to read floating point numbers
// accurately", PLDI 1990): when the decimal significand m < 2^53 and the
// decimal exponent |e| <= 22, both m and 10^|e| are exact doubles, so the one
// IEEE multiply or divide m * 10^e is the correctly rounded double -- the
// value strtod returns.  The float is then that double rounded to float, as
// the reference's (float)atof does.  Only a token that is exactly
// [+-]digits[.digits][(e|E)[+-]digits] (optionally followed by '\r', where
// strtod stops too) takes the fast path; everything else (leading
// whitespace, hex, inf/nan, trailing text, long significands, large
// exponents) goes to strtod itself.
inline float token_float(const Token& t)
{
    const char* p = t.p;
    const char* e = t.p + t.len;
    if (e > p && e[-1] == '\r') --e;
    if (p == e) return token_float_libc(t);
    bool neg = false;
    if (*p == '+' || *p == '-') neg = *p++ == '-';
    uint64_t m = 0;
    int digits = 0, frac = 0;
    bool any = false;
    while (p < e && *p >= '0' && *p <= '9') {
        if (m || *p != '0') ++digits;
        m = m * 10 + (uint64_t)(*p++ - '0');
        any = true;
        if (digits > 18) return token_float_libc(t);
    }
    if (p < e && *p == '.') {
        ++p;
        while (p < e && *p >= '0' && *p <= '9') {
            if (m || *p != '0') ++digits;
            m = m * 10 + (uint64_t)(*p++ - '0');
            ++frac;
            any = true;
            if (digits > 18) return token_float_libc(t);
        }
    }
    if (!any) return token_float_libc(t);
    int ex = 0;
    if (p < e && (*p == 'e' || *p == 'E')) {
        ++p;
        bool eneg = false;
        if (p < e && (*p == '+' || *p == '-')) eneg = *p++ == '-';
        if (p == e) return token_float_libc(t);
        while (p < e && *p >= '0' && *p <= '9') {
            ex = ex * 10 + (*p++ - '0');
            if (ex > 1000) return token_float_libc(t);
        }
        if (eneg) ex = -ex;
    }
    if (p != e) return token_float_libc(t);
    ex -= frac;
    if (m > (1ull << 53) || ex < -22 || ex > 22) return token_float_libc(t);
    double v = (double)m;
    v = ex < 0 ? v / kPow10[-ex] : v * kPow10[ex];
    return (float)(neg ? -v : v);
}

// atoi(token) = (int)strtol(token, NULL, 10); the fast path takes
// [+-]digits with at most 9 digits (no overflow), stopping at the first
// non-digit as strtol does ("7/2/9" reads 7).
inline int token_int(const Token& t)
{
    const char* p = t.p;
    const char* e = t.p + t.len;
    bool neg = false;
    if (p < e && (*p == '+' || *p == '-')) neg = *p++ == '-';
    int v = 0, n = 0;
    while (p < e && *p >= '0' && *p <= '9') {
        if (++n > 9) return token_int_libc(t);
        v = v * 10 + (*p++ - '0');
    }
    if (n == 0) return token_int_libc(t);
    return neg ? -v : v;
}

struct Chunk {
    const char* begin = nullptr;
    const char* end = nullptr;
    std::vector<float> verts;       // 3 per vertex
    std::vector<uint32_t> index;    // 3 per face, local resolution
    std::vector<uint8_t> relative;  // per index: 1 = negative (add the vertex base)
    std::vector<uint32_t> face_line;
    uint32_t lines = 0;
    uint32_t vbase = 0, fbase = 0, lbase = 0;
    bool failed = false;
    uint32_t fail_line = 0;
    char fail_msg[96] = {0};
};

inline bool is_word(const Token& t, char c) { return t.ok && t.len == 1 && t.p[0] == c; }

void parse_chunk(Chunk& ck)
{
    const char* p = ck.begin;
    while (p < ck.end) {
        // one fgets() line: up to 255 characters, through the first '\n'
        const char* lim = std::min(ck.end, p + kLineMax);
        const char* nl = static_cast<const char*>(memchr(p, '\n', (size_t)(lim - p)));
        const char* next = nl ? nl + 1 : lim;
        // the C string ends at an embedded NUL
        const char* nul = static_cast<const char*>(memchr(p, '\0', (size_t)(next - p)));
        const char* e = nul ? nul : next;
        const uint32_t line = ck.lines++;
        const char* s = p;
        p = next;

        const Token cmd = next_token(s, e, true);
        if (is_word(cmd, 'v')) {
            float f[3];
            for (int i = 0; i < 3; ++i) {
                const Token t = next_token(s, e, false);
                if (!t.ok) {
                    ck.failed = true;
                    ck.fail_line = line;
                    snprintf(ck.fail_msg, sizeof(ck.fail_msg), "vertex record has fewer than 3 delimited values");
                    return;
                }
                f[i] = token_float(t);
            }
            ck.verts.insert(ck.verts.end(), f, f + 3);
        } else if (is_word(cmd, 'f')) {
            const uint32_t vcount = (uint32_t)(ck.verts.size() / 3);
            uint32_t idx[3];
            uint8_t rel[3];
            for (int i = 0; i < 3; ++i) {
                const Token t = next_token(s, e, false);
                if (!t.ok) {
                    ck.failed = true;
                    ck.fail_line = line;
                    snprintf(ck.fail_msg, sizeof(ck.fail_msg), "face record has fewer than 3 delimited indices");
                    return;
                }
                const int v = token_int(t);
                rel[i] = v < 0;
                idx[i] = (uint32_t)v + (v < 0 ? vcount : 0xFFFFFFFFu);
            }
            ck.index.insert(ck.index.end(), idx, idx + 3);
            ck.relative.insert(ck.relative.end(), rel, rel + 3);
            ck.face_line.push_back(line);
            const Token t4 = next_token(s, e, false);
            if (t4.ok) {
                const int v = token_int(t4);
                const uint32_t i3 = (uint32_t)v + (v < 0 ? vcount : 0xFFFFFFFFu);
                const uint32_t q[3] = {idx[0], idx[2], i3};
                const uint8_t r[3] = {rel[0], rel[2], (uint8_t)(v < 0)};
                ck.index.insert(ck.index.end(), q, q + 3);
                ck.relative.insert(ck.relative.end(), r, r + 3);
                ck.face_line.push_back(line);
            }
        }
    }
}

template <class F>
void parallel_for(uint32_t n, uint32_t threads, F&& f)
{
    if (threads <= 1 || n <= 1) {
        for (uint32_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::vector<std::thread> pool;
    std::atomic_uint next{0};
    const uint32_t t = std::min(threads, n);
    pool.reserve(t);
    for (uint32_t k = 0; k < t; ++k) {
        pool.emplace_back([&] {
            for (uint32_t i; (i = next.fetch_add(1)) < n;) f(i);
        });
    }
    for (auto& th : pool) th.join();
}

uint32_t pick_threads(uint32_t threads)
{
    if (threads == 0) {
        const unsigned h = std::thread::hardware_concurrency();
        threads = h ? h : 1;
    }
    return std::min<uint32_t>(threads, 256);
}

}  // namespace

extern "C" {

const char* sq_host_last_error(void) { return g_error.c_str(); }

void sq_obj_free(sq_triangle* tris) { free(tris); }

sq_status sq_obj_parse(const char* text, uint64_t len, uint32_t threads, sq_triangle** tris, uint32_t* tri_count,
                       sq_obj_info* info)
{
    if (!tris || !tri_count || (!text && len)) return host_fail(SQ_ERR_INVALID, "null argument");
    *tris = nullptr;
    *tri_count = 0;
    threads = pick_threads(threads);
    // chunks of at least 1 MB, a few per thread, each starting after a '\n'
    const uint64_t min_chunk = 1u << 20;
    uint64_t want = std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)threads * 4, len / min_chunk));
    std::vector<Chunk> chunks;
    chunks.reserve(want);
    const char* end = text + len;
    const char* cur = text;
    for (uint64_t k = 1; k <= want && cur < end; ++k) {
        const char* cut = (k == want) ? end : text + (len * k) / want;
        if (cut < cur) cut = cur;
        if (cut < end) {
            const char* nl = static_cast<const char*>(memchr(cut, '\n', (size_t)(end - cut)));
            cut = nl ? nl + 1 : end;
        }
        if (cut > cur) {
            chunks.emplace_back();
            chunks.back().begin = cur;
            chunks.back().end = cut;
            cur = cut;
        }
    }
    parallel_for((uint32_t)chunks.size(), threads, [&](uint32_t i) { parse_chunk(chunks[i]); });

    uint64_t nv = 0, nf = 0, nl = 0;
    for (Chunk& ck : chunks) {
        if (ck.failed)
            return host_fail(SQ_ERR_INVALID, "OBJ line %llu: %s", (unsigned long long)(nl + ck.fail_line + 1),
                             ck.fail_msg);
        ck.vbase = (uint32_t)nv;
        ck.fbase = (uint32_t)nf;
        ck.lbase = (uint32_t)nl;
        nv += ck.verts.size() / 3;
        nf += ck.face_line.size();
        nl += ck.lines;
    }
    if (nv > 0xFFFFFFFFull || nf > 0xFFFFFFFFull / 2)
        return host_fail(SQ_ERR_TOO_LARGE, "OBJ has %llu vertices and %llu faces", (unsigned long long)nv,
                         (unsigned long long)nf);
    std::vector<float> verts((size_t)nv * 3);
    parallel_for((uint32_t)chunks.size(), threads, [&](uint32_t i) {
        const Chunk& ck = chunks[i];
        if (!ck.verts.empty()) memcpy(verts.data() + 3ull * ck.vbase, ck.verts.data(), ck.verts.size() * 4);
    });
    sq_triangle* out = nullptr;
    if (nf) {
        out = static_cast<sq_triangle*>(malloc(sizeof(sq_triangle) * nf));
        if (!out) return host_fail(SQ_ERR_OOM, "cannot allocate %llu triangles", (unsigned long long)nf);
    }
    std::vector<uint64_t> bad(chunks.size(), ~0ull);
    parallel_for((uint32_t)chunks.size(), threads, [&](uint32_t i) {
        Chunk& ck = chunks[i];
        const size_t faces = ck.face_line.size();
        for (size_t f = 0; f < faces; ++f) {
            sq_triangle& t = out[ck.fbase + f];
            float* dst[3] = {t.v0, t.v1, t.v2};
            for (int k = 0; k < 3; ++k) {
                const uint32_t g = ck.index[3 * f + k] + (ck.relative[3 * f + k] ? ck.vbase : 0u);
                if ((uint64_t)g >= nv) {
                    bad[i] = ((uint64_t)ck.face_line[f] << 32) | g;
                    return;
                }
                memcpy(dst[k], verts.data() + 3ull * g, 12);
            }
        }
    });
    for (size_t i = 0; i < chunks.size(); ++i) {
        if (bad[i] != ~0ull) {
            free(out);
            return host_fail(SQ_ERR_INVALID, "OBJ line %llu: face index %lld outside the %llu vertices",
                             (unsigned long long)(chunks[i].lbase + (bad[i] >> 32) + 1),
                             (long long)(int32_t)(uint32_t)bad[i] + 1, (unsigned long long)nv);
        }
    }
    *tris = out;
    *tri_count = (uint32_t)nf;
    if (info) {
        info->faces = (uint32_t)nf;
        info->vertices = (uint32_t)nv;
        info->lines = (uint32_t)nl;
        info->threads = threads;
    }
    return SQ_OK;
}

sq_status sq_obj_load(const char* path, uint32_t threads, sq_triangle** tris, uint32_t* tri_count, sq_obj_info* info)
{
    if (!path) return host_fail(SQ_ERR_INVALID, "null path");
    const int fd = open(path, O_RDONLY);
    if (fd < 0) return host_fail(SQ_ERR_INVALID, "Can't open OBJ file %s: %s", path, strerror(errno));
    struct stat st;
    if (fstat(fd, &st) == 0 && S_ISREG(st.st_mode) && st.st_size > 0) {
        // a regular file is mapped, so the parse threads fault its pages in
        // parallel instead of waiting for one sequential read
        void* m = mmap(nullptr, (size_t)st.st_size, PROT_READ, MAP_PRIVATE, fd, 0);
        if (m != MAP_FAILED) {
            close(fd);
            const sq_status s = sq_obj_parse(static_cast<const char*>(m), (uint64_t)st.st_size, threads, tris,
                                             tri_count, info);
            munmap(m, (size_t)st.st_size);
            return s;
        }
    }
    std::vector<char> buf;
    char tmp[1 << 16];
    for (;;) {
        const ssize_t got = read(fd, tmp, sizeof(tmp));
        if (got < 0 && errno == EINTR) continue;
        if (got < 0) {
            close(fd);
            return host_fail(SQ_ERR_INVALID, "read error on OBJ file %s: %s", path, strerror(errno));
        }
        if (got == 0) break;
        buf.insert(buf.end(), tmp, tmp + got);
    }
    close(fd);
    return sq_obj_parse(buf.data(), buf.size(), threads, tris, tri_count, info);
}

uint64_t sq_bmp_size(uint32_t w, uint32_t h)
{
    const uint64_t row = (3ull * w + 3) & ~3ull;
    return 54 + row * h;
}

sq_status sq_bmp_encode(uint32_t w, uint32_t h, const uint8_t* rgb, uint8_t* out)
{
    if (!out || (!rgb && w && h)) return host_fail(SQ_ERR_INVALID, "null argument");
    if (w > 0x7FFFFFFFu || h > 0x7FFFFFFFu || sq_bmp_size(w, h) > 0xFFFFFFFFull)
        return host_fail(SQ_ERR_TOO_LARGE, "BMP of %ux%u does not fit the format", w, h);
    const uint64_t row = (3ull * w + 3) & ~3ull;
    auto put16 = [](uint8_t* p, uint32_t v) { p[0] = (uint8_t)v; p[1] = (uint8_t)(v >> 8); };
    auto put32 = [](uint8_t* p, uint32_t v) {
        p[0] = (uint8_t)v; p[1] = (uint8_t)(v >> 8); p[2] = (uint8_t)(v >> 16); p[3] = (uint8_t)(v >> 24);
    };
    memset(out, 0, 54);
    out[0] = 'B';
    out[1] = 'M';
    put32(out + 2, (uint32_t)sq_bmp_size(w, h));  // file size
    put32(out + 10, 54);                          // pixel data offset
    put32(out + 14, 40);                          // info header size
    put32(out + 18, w);
    put32(out + 22, h);                           // positive: bottom-up rows
    put16(out + 26, 1);                           // planes
    put16(out + 28, 24);                          // bits per pixel
    // compression 0, image size 0, resolution 0, palette 0: already zero
    uint8_t* px = out + 54;
    for (uint32_t y = 0; y < h; ++y) {
        const uint8_t* src = rgb + 3ull * w * y;  // vertically flipped: rgb row 0 is stored first
        uint8_t* dst = px + row * y;
        for (uint32_t x = 0; x < w; ++x) {
            dst[3 * x + 0] = src[3 * x + 2];
            dst[3 * x + 1] = src[3 * x + 1];
            dst[3 * x + 2] = src[3 * x + 0];
        }
        for (uint64_t k = 3ull * w; k < row; ++k) dst[k] = 0;
    }
    return SQ_OK;
}

sq_status sq_bmp_write(const char* path, uint32_t w, uint32_t h, const uint8_t* rgb)
{
    if (!path) return host_fail(SQ_ERR_INVALID, "null path");
    if (sq_bmp_size(w, h) > 0xFFFFFFFFull) return host_fail(SQ_ERR_TOO_LARGE, "BMP of %ux%u does not fit", w, h);
    std::vector<uint8_t> img(sq_bmp_size(w, h));
    const sq_status s = sq_bmp_encode(w, h, rgb, img.data());
    if (s != SQ_OK) return s;
    FILE* fp = fopen(path, "wb");
    if (!fp) return host_fail(SQ_ERR_INVALID, "cannot open %s for writing: %s", path, strerror(errno));
    const size_t put = fwrite(img.data(), 1, img.size(), fp);
    const int rc = fclose(fp);
    if (put != img.size() || rc != 0) return host_fail(SQ_ERR_INVALID, "write error on %s", path);
    return SQ_OK;
}

}  // extern "C"
