// colo_ingest.cu -- the point CSV parsed on the device.
//
// populateData (Codes/colocationFinder.cpp:139-254) reads the file serially.
// Here the text after the count line is copied to the device once; one pass
// finds the line ends, and one thread per line parses "fid,x,y" with the
// host reader's rules (std::stoi / std::stof prefix parsing, boost's
// tokenizer).  The parsed coordinates stay on the device as the dataset's
// resident copy.
//
// Exactness: a coordinate is converted on the device only when the decimal
// has at most 19 significant digits and the value is m * 10^e with
// m < 2^53 and |e| <= 22.  Then m and 10^|e| are exact doubles and one IEEE
// multiply or divide gives the correctly rounded double of the decimal
// (Clinger's fast path, "How to read floating point numbers accurately",
// PLDI 1990).  Rounding that double to float is the correctly rounded float
// unless the double lies exactly on a float rounding midpoint, which is
// detected.  Every other line -- a midpoint, more digits, a larger exponent,
// a float outside the normal range, "inf"/"nan"/hex/'+', quotes or escapes --
// is flagged and parsed on the host by the same reader the CPU path uses, so
// results are bit-identical to it.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include "colo_batch.h"
#include "colo_device.cuh"
#include "colo_host.h"

namespace colo {

// Host reader pieces (colo_io.cpp).
bool csv_parse_line(const char* b, const char* e, int32_t* id, float* x, float* y, bool* minus_one,
                    std::string* token);
bool csv_parse_count(const char* b, const char* e, long* n);
bool csv_parse_bounds(const char* b, const char* e, float bounds[4]);

namespace {

enum : uint8_t { L_OK = 0, L_EMPTY = 1, L_HOST = 2, L_BAD = 3, L_MINUS1 = 4 };

constexpr uint32_t kNlBytes = 64;   // bytes per thread when finding line ends

__device__ __forceinline__ uint32_t count_nl_word(uint32_t w) {
    // bytes equal to '\n' (0x0A) in a 32-bit word
    const uint32_t x = w ^ 0x0A0A0A0Au;
    const uint32_t t = ((x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | x;   // high bit set in bytes that are non-zero
    return __popc(~t & 0x80808080u);
}

__global__ void k_count_lines(const uint8_t* __restrict__ buf, uint64_t n, uint32_t* __restrict__ cnt) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t b = t * kNlBytes;
    if (b >= n) return;
    uint32_t c = 0;
    if (b + kNlBytes <= n) {
        const uint4* p = reinterpret_cast<const uint4*>(buf + b);
#pragma unroll
        for (int i = 0; i < (int)(kNlBytes / 16); ++i) {
            const uint4 v = p[i];
            c += count_nl_word(v.x) + count_nl_word(v.y) + count_nl_word(v.z) + count_nl_word(v.w);
        }
    } else {
        for (uint64_t i = b; i < n; ++i) c += buf[i] == '\n';
    }
    cnt[t] = c;
}

__global__ void k_line_ends(const uint8_t* __restrict__ buf, uint64_t n, const uint64_t* __restrict__ off,
                            uint64_t* __restrict__ nl) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t b = t * kNlBytes;
    if (b >= n) return;
    uint64_t o = off[t];
    const uint64_t e = b + kNlBytes < n ? b + kNlBytes : n;
    for (uint64_t i = b; i < e; ++i)
        if (buf[i] == '\n') nl[o++] = i;
}

__device__ __forceinline__ bool is_space(uint8_t c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}

// std::stoi on [b, e): 0 ok, 1 malformed.
__device__ int parse_int_dev(const uint8_t* b, const uint8_t* e, int32_t* v) {
    const uint8_t* p = b;
    while (p < e && is_space(*p)) ++p;
    bool neg = false;
    if (p < e && (*p == '+' || *p == '-')) neg = *p++ == '-';
    const uint8_t* d = p;
    int64_t r = 0;
    for (; p < e && *p >= '0' && *p <= '9'; ++p)
        if (r <= (int64_t)INT32_MAX + 1) r = r * 10 + (*p - '0');
    if (p == d) return 1;
    if (neg) r = -r;
    if (r < INT32_MIN || r > INT32_MAX) return 1;
    *v = (int32_t)r;
    return 0;
}

// std::stof on [b, e) as the host reader does it: 0 converted exactly here,
// 1 left to the host, 2 malformed (no number at the start).
__device__ int parse_float_dev(const uint8_t* b, const uint8_t* e, float* v) {
    const uint8_t* p = b;
    while (p < e && is_space(*p)) ++p;
    for (const uint8_t* q = p; q < e; ++q)
        if (*q == 'x' || *q == 'X') return 1;   // hexadecimal forms: the host
    if (p < e && (*p == '+' || *p == 'i' || *p == 'I' || *p == 'n' || *p == 'N')) return 1;
    bool neg = false;
    if (p < e && *p == '-') {
        neg = true;
        ++p;
        if (p < e && (*p == 'i' || *p == 'I' || *p == 'n' || *p == 'N')) return 1;
    }
    uint64_t m = 0;
    int sig = 0, frac = 0, dropped = 0;
    bool any = false;
    for (; p < e && *p >= '0' && *p <= '9'; ++p) {
        any = true;
        if (m == 0 && *p == '0') continue;
        if (sig < 19) {
            m = m * 10 + (*p - '0');
            ++sig;
        } else {
            ++dropped;
        }
    }
    if (p < e && *p == '.') {
        ++p;
        for (; p < e && *p >= '0' && *p <= '9'; ++p) {
            any = true;
            if (m == 0 && *p == '0') {
                ++frac;
                continue;
            }
            if (sig < 19) {
                m = m * 10 + (*p - '0');
                ++sig;
                ++frac;
            } else {
                ++dropped;   // digits past 19 after the point: the value is not m * 10^e exactly
            }
        }
    }
    if (!any) return 2;
    if (dropped) return 1;
    int ex = 0;
    if (p < e && (*p == 'e' || *p == 'E')) {
        const uint8_t* q = p + 1;
        bool eneg = false;
        if (q < e && (*q == '+' || *q == '-')) eneg = *q++ == '-';
        if (q < e && *q >= '0' && *q <= '9') {   // otherwise the 'e' is not part of the number
            int x = 0;
            for (; q < e && *q >= '0' && *q <= '9'; ++q)
                if (x < 100000) x = x * 10 + (*q - '0');
            ex = eneg ? -x : x;
        }
    }
    if (m == 0) {
        *v = neg ? -0.0f : 0.0f;
        return 0;
    }
    const int e10 = ex - frac;
    if (m >= (1ull << 53) || e10 < -22 || e10 > 22) return 1;
    const double p10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                            1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
    const double dm = (double)m;   // exact: m < 2^53
    const double d = e10 >= 0 ? __dmul_rn(dm, p10[e10]) : __ddiv_rn(dm, p10[-e10]);
    // float normal range only (no subnormal or overflow handling here)
    if (!(d >= 1.1754943508222875e-38) || d > 3.4028234663852886e38) return 1;
    // a float rounding midpoint: the 29 low mantissa bits are exactly 1000...0
    const unsigned long long bits = (unsigned long long)__double_as_longlong(d);
    if ((bits & ((1ull << 29) - 1)) == (1ull << 28)) return 1;
    const float f = __double2float_rn(d);
    *v = neg ? -f : f;
    return 0;
}

__device__ __forceinline__ void to_host(uint64_t i, uint8_t* st, unsigned long long* marks, uint64_t* host_list,
                                        uint64_t host_cap) {
    st[i] = L_HOST;
    const unsigned long long q = atomicAdd(&marks[2], 1ull);
    if (q < host_cap) host_list[q] = i;
}

__device__ __forceinline__ void failed(uint64_t i, uint8_t code, uint8_t* st, unsigned long long* marks) {
    st[i] = code;
    atomicMin(&marks[1], (unsigned long long)i);
}

// One thread per line of the body: lines 0 .. L-1 end at nl[i]; line L (if
// the text does not end with a newline) ends at n.
__global__ void k_parse_lines(const uint8_t* __restrict__ buf, uint64_t n, const uint64_t* __restrict__ nl,
                              uint64_t L, uint64_t lines, float* __restrict__ x, float* __restrict__ y,
                              int32_t* __restrict__ raw, uint8_t* __restrict__ st,
                              unsigned long long* __restrict__ marks, uint64_t* __restrict__ host_list,
                              uint64_t host_cap) {
    // marks[0]: first empty line, marks[1]: first malformed / id -1 line,
    // marks[2]: lines left to the host (their indices in host_list, unordered)
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= lines) return;
    const uint64_t b = i == 0 ? 0 : nl[i - 1] + 1;
    uint64_t e = i < L ? nl[i] : n;
    if (e > b && buf[e - 1] == '\r') --e;
    if (e == b) {
        st[i] = L_EMPTY;
        atomicMin(&marks[0], (unsigned long long)i);
        return;
    }
    const uint8_t* p = buf + b;
    const uint8_t* pe = buf + e;
    const uint8_t *c1 = nullptr, *c2 = nullptr, *c3 = nullptr;
    for (const uint8_t* q = p; q < pe; ++q) {
        const uint8_t ch = *q;
        if (ch == '"' || ch == '\\') {   // the tokenizer's quotes and escapes: the host
            to_host(i, st, marks, host_list, host_cap);
            return;
        }
        if (ch == ',') {
            if (!c1) c1 = q;
            else if (!c2) c2 = q;
            else if (!c3) c3 = q;
        }
    }
    int32_t id = 0;
    float xv = 0.f, yv = 0.f;
    if (!c2 || parse_int_dev(p, c1, &id) != 0) {
        failed(i, L_BAD, st, marks);
        return;
    }
    const int fx = parse_float_dev(c1 + 1, c2, &xv);
    const int fy = parse_float_dev(c2 + 1, c3 ? c3 : pe, &yv);
    if (fx == 2 || fy == 2) {
        failed(i, L_BAD, st, marks);
        return;
    }
    if (fx == 1 || fy == 1) {   // the host decides (a float it rejects makes the line malformed)
        to_host(i, st, marks, host_list, host_cap);
        return;
    }
    if (id == -1) {
        failed(i, L_MINUS1, st, marks);
        return;
    }
    x[i] = xv;
    y[i] = yv;
    raw[i] = id;
    st[i] = L_OK;
}

// Group starts (the first point of every run of equal ids) with the byte
// range of their id field, for the feature names.
__global__ void k_group_starts(const int32_t* __restrict__ raw, uint64_t np, const uint64_t* __restrict__ nl,
                               unsigned long long* __restrict__ cnt, uint64_t* __restrict__ out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    if (i > 0 && raw[i] == raw[i - 1]) return;
    const unsigned long long k = atomicAdd(cnt, 1ull);
    out[2 * k] = i;
    out[2 * k + 1] = i == 0 ? 0 : nl[i - 1] + 1;
}

// Byte ranges [b, e) of the listed lines (a trailing '\r' kept; the host drops it).
__global__ void k_line_bounds(const uint64_t* __restrict__ idx, uint64_t m, const uint64_t* __restrict__ nl,
                              uint64_t L, uint64_t n, uint64_t* __restrict__ out) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m) return;
    const uint64_t i = idx[q];
    out[2 * q] = i == 0 ? 0 : nl[i - 1] + 1;
    out[2 * q + 1] = i < L ? nl[i] : n;
}

// Values of the lines parsed on the host, into the point arrays.
__global__ void k_scatter_points(const uint64_t* __restrict__ idx, const float* __restrict__ xs,
                                 const float* __restrict__ ys, const int32_t* __restrict__ ids, uint64_t m,
                                 float* __restrict__ x, float* __restrict__ y, int32_t* __restrict__ raw) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m) return;
    x[idx[q]] = xs[q];
    y[idx[q]] = ys[q];
    raw[idx[q]] = ids[q];
}

}  // namespace

colo_status parse_points_csv_device(cudaStream_t s, const char* path, HostPoints& hp, DevBuf<float>& dx,
                                    DevBuf<float>& dy, std::string& err) {
    // the file mapped (pages populated up front) and copied to the device from there
    struct Mapped {
        const char* p = nullptr;
        size_t n = 0;
        void* map = nullptr;
        bool ok = false;
        explicit Mapped(const char* path) {
            const int fd = ::open(path, O_RDONLY);
            if (fd < 0) return;
            struct stat st;
            if (::fstat(fd, &st) == 0) {
                n = (size_t)st.st_size;
                if (n == 0) {
                    ok = true;
                } else {
                    map = ::mmap(nullptr, n, PROT_READ, MAP_PRIVATE | MAP_POPULATE, fd, 0);
                    if (map != MAP_FAILED) {
                        p = static_cast<const char*>(map);
                        ok = true;
                    } else {
                        map = nullptr;
                    }
                }
            }
            ::close(fd);
        }
        ~Mapped() {
            if (map) ::munmap(map, n);
        }
    } file(path);
    if (!file.ok) {
        err = std::string("cannot read dataset: ") + path;
        return COLO_ERR_IO;
    }
    const char* beg = file.p;
    const char* end = beg + file.n;
    // the count line, on the host
    const char* nl0 = file.n == 0 ? nullptr : (const char*)std::memchr(beg, '\n', file.n);
    const char* le0 = nl0 ? nl0 : end;
    if (le0 > beg && le0[-1] == '\r') --le0;
    long N = 0;
    if (file.n == 0 || !csv_parse_count(beg, le0, &N)) {
        err = "dataset: first line must hold the point count";
        return COLO_ERR_PARSE;
    }
    const char* body = nl0 ? nl0 + 1 : end;
    const uint64_t nb = (uint64_t)(end - body);
    hp.clear();
    // the text on the device, and its line ends
    DevBuf<uint8_t> dbuf;
    dbuf.alloc(nb ? nb : 16, s);
    if (nb) COLO_CUDA(cudaMemcpyAsync(dbuf.get(), body, nb, cudaMemcpyHostToDevice, s));
    const uint64_t nthreads = (nb + kNlBytes - 1) / kNlBytes;
    DevBuf<uint32_t> cnt;
    DevBuf<uint64_t> off;
    uint64_t L = 0;
    if (nthreads) {
        cnt.alloc(nthreads, s);
        off.alloc(nthreads, s);
        {
            KScope ks("csv_lines");
            k_count_lines<<<(unsigned)((nthreads + 255) / 256), 256, 0, s>>>(dbuf.get(), nb, cnt.get());
            COLO_LAUNCH_CHECK();
            count_launch();
        }
        scan_u32_to_u64(cnt.get(), off.get(), nthreads, s, &L);
    }
    DevBuf<uint64_t> dnl;
    dnl.alloc(L ? L : 1, s);
    uint64_t last_nl = 0;
    if (L) {
        {
            KScope ks("csv_lines");
            k_line_ends<<<(unsigned)((nthreads + 255) / 256), 256, 0, s>>>(dbuf.get(), nb, off.get(), dnl.get());
            COLO_LAUNCH_CHECK();
            count_launch();
        }
        COLO_CUDA(cudaMemcpyAsync(&last_nl, dnl.get() + L - 1, 8, cudaMemcpyDeviceToHost, s));
        COLO_CUDA(cudaStreamSynchronize(s));
    }
    // a last line without its newline counts too (std::getline)
    const uint64_t lines = L + ((L == 0 ? nb > 0 : last_nl + 1 < nb) ? 1 : 0);
    // every line parsed on the device
    DevBuf<float> px, py;
    DevBuf<int32_t> praw;
    DevBuf<uint8_t> pst;
    DevBuf<unsigned long long> marks;
    DevBuf<uint64_t> hlist;
    const uint64_t host_cap = std::max<uint64_t>(1024, lines / 64);
    marks.alloc(3, s);
    hlist.alloc(host_cap, s);
    {
        const unsigned long long init[3] = {~0ull, ~0ull, 0ull};
        COLO_CUDA(cudaMemcpyAsync(marks.get(), init, sizeof(init), cudaMemcpyHostToDevice, s));
    }
    px.alloc(lines ? lines : 1, s);
    py.alloc(lines ? lines : 1, s);
    praw.alloc(lines ? lines : 1, s);
    pst.alloc(lines ? lines : 1, s);
    if (lines) {
        KScope ks("csv_parse");
        k_parse_lines<<<(unsigned)((lines + 255) / 256), 256, 0, s>>>(dbuf.get(), nb, dnl.get(), L, lines, px.get(),
                                                                     py.get(), praw.get(), pst.get(), marks.get(),
                                                                     hlist.get(), host_cap);
        COLO_LAUNCH_CHECK();
        count_launch();
    }
    unsigned long long hm[3] = {~0ull, ~0ull, 0ull};
    COLO_CUDA(cudaMemcpyAsync(hm, marks.get(), sizeof(hm), cudaMemcpyDeviceToHost, s));
    COLO_CUDA(cudaStreamSynchronize(s));
    const unsigned long long first_empty = hm[0];
    const uint64_t np = first_empty < lines ? first_empty : lines;   // point lines before the empty line
    // the first failing device line before the empty line, and its kind
    const uint64_t first_bad = hm[1] < np ? hm[1] : np;
    uint8_t bad_kind = L_BAD;
    if (first_bad < np) COLO_CUDA(cudaMemcpy(&bad_kind, pst.get() + first_bad, 1, cudaMemcpyDeviceToHost));
    // lines the host reads: the listed ones before the first device failure, and the bounds line
    std::vector<uint64_t> want;
    if (hm[2] > host_cap) {   // more than the list holds: find them from the statuses
        std::vector<uint8_t> hst(np);
        if (np) COLO_CUDA(cudaMemcpy(hst.data(), pst.get(), np, cudaMemcpyDeviceToHost));
        for (uint64_t i = 0; i < first_bad; ++i)
            if (hst[i] == L_HOST) want.push_back(i);
    } else if (hm[2]) {
        std::vector<uint64_t> hl(hm[2]);
        COLO_CUDA(cudaMemcpy(hl.data(), hlist.get(), hm[2] * 8, cudaMemcpyDeviceToHost));
        for (uint64_t i : hl)
            if (i < first_bad) want.push_back(i);
        std::sort(want.begin(), want.end());
    }
    const bool has_bounds = first_empty < lines && first_empty + 1 < lines;
    if (has_bounds) want.push_back(first_empty + 1);
    std::vector<uint64_t> rng(2 * want.size());
    if (!want.empty()) {
        DevBuf<uint64_t> didx, drng;
        didx.alloc(want.size(), s);
        drng.alloc(2 * want.size(), s);
        COLO_CUDA(cudaMemcpyAsync(didx.get(), want.data(), want.size() * 8, cudaMemcpyHostToDevice, s));
        k_line_bounds<<<(unsigned)((want.size() + 255) / 256), 256, 0, s>>>(didx.get(), want.size(), dnl.get(), L,
                                                                           nb, drng.get());
        COLO_LAUNCH_CHECK();
        count_launch();
        COLO_CUDA(cudaMemcpyAsync(rng.data(), drng.get(), rng.size() * 8, cudaMemcpyDeviceToHost, s));
        COLO_CUDA(cudaStreamSynchronize(s));
    }
    auto line_at = [&](size_t q, const char** lb, const char** lend) {
        *lb = body + rng[2 * q];
        *lend = body + rng[2 * q + 1];
        if (*lend > *lb && (*lend)[-1] == '\r') --*lend;
    };
    // host lines in order: the first failing line, device or host, is the one the serial reader names
    const size_t nhost = has_bounds ? want.size() - 1 : want.size();
    std::vector<std::pair<uint64_t, std::string>> host_tokens;
    std::vector<uint64_t> hidx;
    std::vector<float> hxv, hyv;
    std::vector<int32_t> hrv;
    for (size_t q = 0; q < nhost; ++q) {
        const uint64_t i = want[q];
        const char *lb, *lend;
        line_at(q, &lb, &lend);
        int32_t id;
        float xv, yv;
        bool m1 = false;
        std::string tok;
        if (!csv_parse_line(lb, lend, &id, &xv, &yv, &m1, &tok)) {
            err = m1 ? "dataset: feature id -1 is the reference's 'no feature yet' marker (line " +
                           std::to_string(i + 2) + ")"
                     : "dataset: malformed point line " + std::to_string(i + 2);
            return COLO_ERR_PARSE;
        }
        hidx.push_back(i);
        hxv.push_back(xv);
        hyv.push_back(yv);
        hrv.push_back(id);
        host_tokens.emplace_back(i, std::move(tok));
    }
    if (first_bad < np) {
        err = bad_kind == L_MINUS1 ? "dataset: feature id -1 is the reference's 'no feature yet' marker (line " +
                                               std::to_string(first_bad + 2) + ")"
                                         : "dataset: malformed point line " + std::to_string(first_bad + 2);
        return COLO_ERR_PARSE;
    }
    if ((long)np != N) {
        err = "dataset: count line says " + std::to_string(N) + " points, found " + std::to_string(np);
        return COLO_ERR_PARSE;
    }
    if (!has_bounds) {
        err = "dataset: bounds line missing";
        return COLO_ERR_PARSE;
    }
    {
        const char *lb, *lend;
        line_at(want.size() - 1, &lb, &lend);
        if (!csv_parse_bounds(lb, lend, hp.bounds)) {
            err = "dataset: bounds line must be minX,minY,maxX,maxY";
            return COLO_ERR_PARSE;
        }
    }
    // the host's values into the device arrays
    if (!hidx.empty()) {
        const uint64_t m = hidx.size();
        DevBuf<uint64_t> di;
        DevBuf<float> dxs, dys;
        DevBuf<int32_t> dis;
        di.alloc(m, s);
        dxs.alloc(m, s);
        dys.alloc(m, s);
        dis.alloc(m, s);
        COLO_CUDA(cudaMemcpyAsync(di.get(), hidx.data(), m * 8, cudaMemcpyHostToDevice, s));
        COLO_CUDA(cudaMemcpyAsync(dxs.get(), hxv.data(), m * 4, cudaMemcpyHostToDevice, s));
        COLO_CUDA(cudaMemcpyAsync(dys.get(), hyv.data(), m * 4, cudaMemcpyHostToDevice, s));
        COLO_CUDA(cudaMemcpyAsync(dis.get(), hrv.data(), m * 4, cudaMemcpyHostToDevice, s));
        k_scatter_points<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(di.get(), dxs.get(), dys.get(), dis.get(), m,
                                                                    px.get(), py.get(), praw.get());
        COLO_LAUNCH_CHECK();
        count_launch();
        COLO_CUDA(cudaStreamSynchronize(s));   // the host vectors above are about to go
    }
    // group starts and the line start of each (feature names)
    DevBuf<unsigned long long> gcnt;
    DevBuf<uint64_t> gout;
    gcnt.alloc(1, s);
    gcnt.zero(s);
    gout.alloc(2 * (np ? np : 1), s);
    if (np) {
        KScope ks("csv_groups");
        k_group_starts<<<(unsigned)((np + 255) / 256), 256, 0, s>>>(praw.get(), np, dnl.get(), gcnt.get(), gout.get());
        COLO_LAUNCH_CHECK();
        count_launch();
    }
    unsigned long long G = 0;
    COLO_CUDA(cudaMemcpyAsync(&G, gcnt.get(), 8, cudaMemcpyDeviceToHost, s));
    hp.x.resize(np);
    hp.y.resize(np);
    hp.raw.resize(np);
    if (np) {
        COLO_CUDA(cudaMemcpyAsync(hp.x.data(), px.get(), np * 4, cudaMemcpyDeviceToHost, s));
        COLO_CUDA(cudaMemcpyAsync(hp.y.data(), py.get(), np * 4, cudaMemcpyDeviceToHost, s));
        COLO_CUDA(cudaMemcpyAsync(hp.raw.data(), praw.get(), np * 4, cudaMemcpyDeviceToHost, s));
    }
    COLO_CUDA(cudaStreamSynchronize(s));
    std::vector<uint64_t> g(2 * G);
    if (G) {
        COLO_CUDA(cudaMemcpyAsync(g.data(), gout.get(), 2 * G * 8, cudaMemcpyDeviceToHost, s));
        COLO_CUDA(cudaStreamSynchronize(s));
    }
    std::vector<std::pair<uint64_t, uint64_t>> starts(G);
    for (uint64_t q = 0; q < G; ++q) starts[q] = {g[2 * q], g[2 * q + 1]};
    std::sort(starts.begin(), starts.end());
    size_t hq = 0;
    hp.tokens.reserve(G);
    for (const auto& st : starts) {
        const uint64_t i = st.first;
        while (hq < host_tokens.size() && host_tokens[hq].first < i) ++hq;
        if (hq < host_tokens.size() && host_tokens[hq].first == i) {
            hp.tokens.emplace_back(i, host_tokens[hq].second);   // the tokenizer's unescaped field
            continue;
        }
        const char* lb = body + st.second;   // a device-parsed line: plain text up to the first comma
        const char* c1 = (const char*)std::memchr(lb, ',', (size_t)(end - lb));
        hp.tokens.emplace_back(i, std::string(lb, c1 ? c1 : lb));
    }
    hp.tokens_complete = true;
    dx = std::move(px);
    dy = std::move(py);
    return COLO_OK;
}

}  // namespace colo
