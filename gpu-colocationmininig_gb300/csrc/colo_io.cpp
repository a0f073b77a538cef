// colo_io.cpp -- input formats of the reference: config file, parameter
// file and the point CSV; output: ColocationDegree_<k>.txt pattern files.
// Also the binary point file (.colo), which has no counterpart in the
// reference: the parsed CSV, loaded without parsing.
#include <algorithm>
#include <cerrno>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <thread>
#include <vector>

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include "colo_host.h"

namespace colo {

namespace {

// Split one CSV line the way boost::escaped_list_separator<char> does with
// its defaults (separator ',', quote '"', escape '\\'), which is the
// tokenizer populateData uses (colocationFinder.cpp:156).
void split_fields(const char* b, const char* e, std::vector<std::string>& out) {
    out.clear();
    bool simple = true;
    for (const char* p = b; p < e; ++p)
        if (*p == '"' || *p == '\\') {
            simple = false;
            break;
        }
    if (simple) {
        const char* s = b;
        for (const char* p = b; p <= e; ++p)
            if (p == e || *p == ',') {
                out.emplace_back(s, p);
                s = p + 1;
            }
        return;
    }
    std::string cur;
    bool inq = false;
    for (const char* p = b; p < e; ++p) {
        char ch = *p;
        if (ch == '\\' && p + 1 < e) {
            char nx = *++p;
            cur.push_back(nx == 'n' ? '\n' : nx);
        } else if (ch == '"') {
            inq = !inq;
        } else if (ch == ',' && !inq) {
            out.push_back(cur);
            cur.clear();
        } else {
            cur.push_back(ch);
        }
    }
    out.push_back(cur);
}

inline bool is_space(char c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}

// std::stof on the characters [b, e): leading whitespace skipped, longest
// numeric prefix, at least one character consumed.
bool parse_float(const char* b, const char* e, float* v) {
    const char* p = b;
    while (p < e && is_space(*p)) ++p;
    bool slow = (p < e && *p == '+');
    for (const char* q = p; q < e && !slow; ++q)
        if (*q == 'x' || *q == 'X') slow = true;
    if (!slow) {
        auto r = std::from_chars(p, e, *v, std::chars_format::general);
        if (r.ec == std::errc()) return true;
        if (r.ec == std::errc::result_out_of_range) slow = true;
        else return false;
    }
    const std::string s(b, e);
    char* endp = nullptr;
    errno = 0;
    *v = std::strtof(s.c_str(), &endp);
    return endp != s.c_str() && errno != ERANGE;
}
bool parse_float(const std::string& s, float* v) { return parse_float(s.data(), s.data() + s.size(), v); }

// std::stoi on the characters [b, e) (strtol base 10, then the int range).
bool parse_int(const char* b, const char* e, long* v) {
    const char* p = b;
    while (p < e && is_space(*p)) ++p;
    bool neg = false;
    if (p < e && (*p == '+' || *p == '-')) neg = *p++ == '-';
    const char* d = p;
    int64_t r = 0;
    for (; p < e && *p >= '0' && *p <= '9'; ++p)
        if (r <= (int64_t)INT32_MAX + 1) r = r * 10 + (*p - '0');
    if (p == d) return false;
    if (neg) r = -r;
    if (r < INT32_MIN || r > INT32_MAX) return false;
    *v = (long)r;
    return true;
}
bool parse_int(const std::string& s, long* v) { return parse_int(s.data(), s.data() + s.size(), v); }

}  // namespace

colo_status read_params_file(const char* path, colo_params* p, std::string& err) {
    std::ifstream ifs(path);
    if (!ifs.is_open()) {
        err = std::string("parameter file missing: ") + path;
        return COLO_ERR_IO;
    }
    float R = 0, thr = 0;
    unsigned flag = 0;
    ifs >> R;
    ifs >> thr;
    ifs >> flag;
    if (!(R > 0) || !std::isfinite(R) || !std::isfinite(thr)) {
        err = "parameter file: distance must be a positive number followed by the PI threshold";
        return COLO_ERR_PARSE;
    }
    p->distance = R;
    p->pi_threshold = thr;
    p->filter_flag = flag;
    return COLO_OK;
}

colo_status read_config_file(const char* path, std::string out[5], std::string& err) {
    std::ifstream in(path);
    if (!in.is_open()) {
        err = std::string("configuration file missing: ") + path;
        return COLO_ERR_IO;
    }
    for (int i = 0; i < 5; ++i) {
        std::string line;
        std::getline(in, line);
        if (!line.empty() && line.back() == '\r') line.pop_back();
        out[i] = line;
    }
    return COLO_OK;
}

namespace {

// Read-only view of a whole file: mapped when it can be, else read.
struct FileView {
    const char* p = nullptr;
    size_t n = 0;
    bool ok = false;
    void* map = nullptr;
    std::vector<char> buf;
    explicit FileView(const char* path) {
        int fd = ::open(path, O_RDONLY);
        if (fd < 0) return;
        struct stat st;
        if (::fstat(fd, &st) != 0) {
            ::close(fd);
            return;
        }
        n = (size_t)st.st_size;
        if (n > 0) {
            map = ::mmap(nullptr, n, PROT_READ, MAP_PRIVATE | MAP_POPULATE, fd, 0);
            if (map == MAP_FAILED) {
                map = nullptr;
                buf.resize(n);
                size_t got = 0;
                while (got < n) {
                    ssize_t r = ::read(fd, buf.data() + got, n - got);
                    if (r <= 0) break;
                    got += (size_t)r;
                }
                if (got != n) {
                    ::close(fd);
                    return;
                }
                p = buf.data();
            } else {
                ::madvise(map, n, MADV_SEQUENTIAL);
                p = (const char*)map;
            }
        }
        ::close(fd);
        ok = true;
    }
    ~FileView() {
        if (map) ::munmap(map, n);
    }
    FileView(const FileView&) = delete;
    FileView& operator=(const FileView&) = delete;
};

// One line of [p, end) as std::getline gives it (a trailing '\r' dropped);
// returns the start of the next line.
inline const char* line_at(const char* p, const char* end, const char** le) {
    const char* nl = (const char*)std::memchr(p, '\n', (size_t)(end - p));
    const char* e = nl ? nl : end;
    *le = (e > p && e[-1] == '\r') ? e - 1 : e;
    return nl ? nl + 1 : end;
}

// Points of a run of whole lines, parsed by one thread.
struct CsvChunk {
    const char* b = nullptr;
    const char* e = nullptr;
    std::vector<float> x, y;
    std::vector<int32_t> raw;
    std::vector<std::pair<uint64_t, std::string>> tokens;   // chunk-local index
    bool stopped = false;           // met the empty line that ends the points
    const char* after = nullptr;    // the line after it
    bool failed = false;
    bool minus_one = false;         // the failure is an id of -1
    uint64_t fail_line = 0;         // 1-based within the chunk
};

void parse_chunk(CsvChunk& c) {
    std::vector<std::string> f;
    uint64_t line = 0;
    const size_t guess = (size_t)(c.e - c.b) / 24 + 16;
    c.x.reserve(guess);
    c.y.reserve(guess);
    c.raw.reserve(guess);
    for (const char* p = c.b; p < c.e;) {
        const char* le;
        const char* next = line_at(p, c.e, &le);
        ++line;
        if (le == p) {
            c.stopped = true;
            c.after = next;
            return;
        }
        long id;
        float xv, yv;
        const char *t0 = p, *t1 = nullptr;
        bool ok;
        const bool simple = !std::memchr(p, '"', (size_t)(le - p)) && !std::memchr(p, '\\', (size_t)(le - p));
        if (simple) {
            const char* c1 = (const char*)std::memchr(p, ',', (size_t)(le - p));
            const char* c2 = c1 ? (const char*)std::memchr(c1 + 1, ',', (size_t)(le - c1 - 1)) : nullptr;
            const char* c3 = c2 ? (const char*)std::memchr(c2 + 1, ',', (size_t)(le - c2 - 1)) : nullptr;
            t1 = c1;
            ok = c2 && parse_int(p, c1, &id) && parse_float(c1 + 1, c2, &xv) && parse_float(c2 + 1, c3 ? c3 : le, &yv);
        } else {
            split_fields(p, le, f);
            ok = f.size() >= 3 && parse_int(f[0], &id) && parse_float(f[1], &xv) && parse_float(f[2], &yv);
        }
        if (ok && id == -1) {
            ok = false;
            c.minus_one = true;
        }
        if (!ok) {
            c.failed = true;
            c.fail_line = line;
            return;
        }
        if (c.raw.empty() || c.raw.back() != (int32_t)id)
            c.tokens.emplace_back(c.raw.size(), simple ? std::string(t0, t1) : f[0]);
        c.raw.push_back((int32_t)id);
        c.x.push_back(xv);
        c.y.push_back(yv);
        p = next;
    }
}

unsigned csv_threads(unsigned requested, size_t bytes) {
    if (requested) return requested;
    unsigned hw = std::thread::hardware_concurrency();
    if (hw == 0) hw = 1;
    const size_t per = (size_t)4 << 20;       // a thread per 4 MB of text
    return (unsigned)std::max<size_t>(1, std::min<size_t>(std::min<unsigned>(hw, 64), bytes / per));
}

template <class Fn>
void run_threads(unsigned T, Fn&& fn) {
    if (T == 1) {
        fn(0u);
        return;
    }
    std::vector<std::thread> th;
    th.reserve(T - 1);
    for (unsigned t = 1; t < T; ++t) th.emplace_back([&fn, t] { fn(t); });
    fn(0u);
    for (auto& t : th) t.join();
}

}  // namespace

// One point line, one count line and the bounds line with the reader's rules
// (for the device reader's host-side lines).
bool csv_parse_line(const char* b, const char* e, int32_t* id, float* x, float* y, bool* minus_one,
                    std::string* token) {
    *minus_one = false;
    std::vector<std::string> f;
    split_fields(b, e, f);
    long v;
    if (f.size() < 3 || !parse_int(f[0], &v) || !parse_float(f[1], x) || !parse_float(f[2], y)) return false;
    if (v == -1) {
        *minus_one = true;
        return false;
    }
    *id = (int32_t)v;
    if (token) *token = f[0];
    return true;
}

bool csv_parse_count(const char* b, const char* e, long* n) { return parse_int(b, e, n) && *n >= 0; }

bool csv_parse_bounds(const char* b, const char* e, float bounds[4]) {
    std::vector<std::string> f;
    split_fields(b, e, f);
    if (f.size() < 4) return false;
    for (int i = 0; i < 4; ++i)
        if (!parse_float(f[i], &bounds[i])) return false;
    return true;
}

// populateData (colocationFinder.cpp:139-254), parsed in parallel: the point
// lines are cut into runs of whole lines, one per thread; each run is parsed
// until its end or an empty line, and the runs are joined in order up to the
// first empty line.  Errors name the same line the serial reading would stop
// at: the first failing line before the first empty line.
colo_status parse_points_csv(const char* path, HostPoints& hp, std::string& err, unsigned threads) {
    FileView fv(path);
    if (!fv.ok) {
        err = std::string("cannot read dataset: ") + path;
        return COLO_ERR_IO;
    }
    const char* end = fv.p + fv.n;
    long N = 0;
    const char* body = fv.p;
    bool counted = false;
    if (fv.n > 0) {
        const char* le;
        body = line_at(fv.p, end, &le);
        counted = parse_int(fv.p, le, &N) && N >= 0;
    }
    if (!counted) {
        err = "dataset: first line must hold the point count";
        return COLO_ERR_PARSE;
    }
    const unsigned T = csv_threads(threads, (size_t)(end - body));
    std::vector<CsvChunk> ch(T);
    const char* cut = body;
    for (unsigned t = 0; t < T; ++t) {
        ch[t].b = cut;
        if (t + 1 == T) {
            cut = end;
        } else {
            const char* target = body + (size_t)((double)(end - body) * (t + 1) / T);
            if (target < cut) target = cut;
            const char* nl = target < end ? (const char*)std::memchr(target, '\n', (size_t)(end - target)) : nullptr;
            cut = nl ? nl + 1 : end;
        }
        ch[t].e = cut;
    }
    run_threads(T, [&](unsigned t) { parse_chunk(ch[t]); });

    uint64_t n = 0, line_no = 1;
    unsigned last = T;           // the chunk that holds the empty line (T: none)
    for (unsigned t = 0; t < T; ++t) {
        const CsvChunk& c = ch[t];
        if (c.failed) {
            line_no += c.fail_line;
            if (c.minus_one)
                err = "dataset: feature id -1 is the reference's 'no feature yet' marker (line " +
                      std::to_string(line_no) + ")";
            else
                err = "dataset: malformed point line " + std::to_string(line_no);
            return COLO_ERR_PARSE;
        }
        n += c.raw.size();
        line_no += c.raw.size();
        if (c.stopped) {
            last = t;
            break;
        }
    }
    if ((long)n != N) {
        err = "dataset: count line says " + std::to_string(N) + " points, found " + std::to_string(n);
        return COLO_ERR_PARSE;
    }
    hp.clear();
    hp.x.resize(n);
    hp.y.resize(n);
    hp.raw.resize(n);
    const unsigned used = last < T ? last + 1 : T;
    std::vector<uint64_t> off(used + 1, 0);
    bool have_prev = false;      // a run's first point starts a feature unless the id continues
    int32_t prev_raw = 0;
    for (unsigned t = 0; t < used; ++t) {
        CsvChunk& c = ch[t];
        off[t + 1] = off[t] + c.raw.size();
        for (auto& tk : c.tokens)
            if (tk.first > 0 || !have_prev || prev_raw != c.raw[0])
                hp.tokens.emplace_back(off[t] + tk.first, std::move(tk.second));
        if (!c.raw.empty()) {
            have_prev = true;
            prev_raw = c.raw.back();
        }
    }
    run_threads(used, [&](unsigned t) {
        const CsvChunk& c = ch[t];
        if (c.raw.empty()) return;
        std::memcpy(hp.x.data() + off[t], c.x.data(), c.x.size() * sizeof(float));
        std::memcpy(hp.y.data() + off[t], c.y.data(), c.y.size() * sizeof(float));
        std::memcpy(hp.raw.data() + off[t], c.raw.data(), c.raw.size() * sizeof(int32_t));
    });
    hp.tokens_complete = true;
    const char* b = last < T ? ch[last].after : end;
    if (b >= end) {
        err = "dataset: bounds line missing";
        return COLO_ERR_PARSE;
    }
    const char* le;
    line_at(b, end, &le);
    std::vector<std::string> f;
    split_fields(b, le, f);
    if (f.size() < 4) {
        err = "dataset: bounds line must be minX,minY,maxX,maxY";
        return COLO_ERR_PARSE;
    }
    for (int i = 0; i < 4; ++i)
        if (!parse_float(f[i], &hp.bounds[i])) {
            err = "dataset: bounds line must be minX,minY,maxX,maxY";
            return COLO_ERR_PARSE;
        }
    return COLO_OK;
}

colo_status write_points_csv(const HostPoints& hp, const std::vector<std::string>& names,
                             const std::vector<uint32_t>& fstart, const std::vector<uint32_t>& fcount, const char* path,
                             std::string& err) {
    FILE* fo = std::fopen(path, "wb");
    if (!fo) {
        err = std::string("cannot write ") + path;
        return COLO_ERR_IO;
    }
    std::fprintf(fo, "%zu\n", hp.x.size());
    for (size_t f = 0; f < names.size(); ++f)
        for (uint64_t i = fstart[f]; i < (uint64_t)fstart[f] + fcount[f]; ++i)
            std::fprintf(fo, "%s,%.9g,%.9g\n", names[f].c_str(), (double)hp.x[i], (double)hp.y[i]);
    std::fprintf(fo, "\n%.9g,%.9g,%.9g,%.9g", (double)hp.bounds[0], (double)hp.bounds[1],
                 (double)hp.bounds[2], (double)hp.bounds[3]);
    std::fclose(fo);
    return COLO_OK;
}

std::vector<uint64_t> group_starts(const int32_t* raw, uint64_t n, bool* minus_one) {
    *minus_one = false;
    std::vector<uint64_t> out;
    if (n == 0) return out;
    unsigned T = std::thread::hardware_concurrency();
    if (T == 0) T = 1;
    T = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(std::min<unsigned>(T, 64), n >> 20));
    std::vector<std::vector<uint64_t>> part(T);
    std::vector<char> bad(T, 0);
    run_threads(T, [&](unsigned t) {
        const uint64_t a = n * t / T, b = n * (t + 1) / T;
        for (uint64_t i = a; i < b; ++i) {
            if (raw[i] == -1) bad[t] = 1;
            if (i == 0 || raw[i] != raw[i - 1]) part[t].push_back(i);
        }
    });
    for (unsigned t = 0; t < T; ++t) {
        *minus_one |= bad[t] != 0;
        out.insert(out.end(), part[t].begin(), part[t].end());
    }
    return out;
}

// ---------------------------------------------------------------------------
// Binary point file (.colo).  Little-endian, 64-byte header, then
//   x[n] f32, y[n] f32, raw[n] i32   (the CSV's columns, in file order)
//   name_len[nfeat] u32, names        (each feature's id token, concatenated)
// Features are the runs of equal consecutive ids, as in the CSV, so the file
// carries the same grouping and names.
// ---------------------------------------------------------------------------
namespace {

static_assert(__BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__, "the binary point file is little-endian");

struct BinHeader {
    char magic[8];
    uint32_t version;
    uint32_t header_bytes;
    uint64_t n;
    uint64_t nfeat;
    uint64_t name_bytes;
    float bounds[4];
    uint64_t reserved;
};
static_assert(sizeof(BinHeader) == 64, "header layout");
constexpr char kBinMagic[8] = {'C', 'O', 'L', 'O', 'P', 'T', 'S', '1'};

bool write_all(FILE* f, const void* p, size_t bytes) { return bytes == 0 || std::fwrite(p, 1, bytes, f) == bytes; }

}  // namespace

colo_status write_points_binary(const HostPoints& hp, const std::vector<std::string>& names, const char* path,
                                std::string& err) {
    BinHeader h{};
    std::memcpy(h.magic, kBinMagic, 8);
    h.version = 1;
    h.header_bytes = sizeof(BinHeader);
    h.n = hp.x.size();
    h.nfeat = names.size();
    std::vector<uint32_t> len(names.size());
    for (size_t i = 0; i < names.size(); ++i) {
        len[i] = (uint32_t)names[i].size();
        h.name_bytes += names[i].size();
    }
    std::memcpy(h.bounds, hp.bounds, sizeof(h.bounds));
    FILE* fo = std::fopen(path, "wb");
    if (!fo) {
        err = std::string("cannot write ") + path;
        return COLO_ERR_IO;
    }
    bool ok = write_all(fo, &h, sizeof(h)) && write_all(fo, hp.x.data(), hp.x.size() * 4) &&
              write_all(fo, hp.y.data(), hp.y.size() * 4) && write_all(fo, hp.raw.data(), hp.raw.size() * 4) &&
              write_all(fo, len.data(), len.size() * 4);
    for (size_t i = 0; ok && i < names.size(); ++i) ok = write_all(fo, names[i].data(), names[i].size());
    ok = (std::fclose(fo) == 0) && ok;
    if (!ok) {
        err = std::string("cannot write ") + path;
        return COLO_ERR_IO;
    }
    return COLO_OK;
}

colo_status read_points_binary(const char* path, HostPoints& hp, std::string& err) {
    const int fd = ::open(path, O_RDONLY);
    if (fd < 0) {
        err = std::string("cannot read dataset: ") + path;
        return COLO_ERR_IO;
    }
    struct Closer {
        int fd;
        ~Closer() { ::close(fd); }
    } closer{fd};
    struct stat st;
    if (::fstat(fd, &st) != 0) {
        err = std::string("cannot read dataset: ") + path;
        return COLO_ERR_IO;
    }
    const uint64_t fsize = (uint64_t)st.st_size;
    // whole read of [off, off + bytes) into dst
    auto pread_all = [fd](void* dst, uint64_t bytes, uint64_t off) {
        char* p = static_cast<char*>(dst);
        while (bytes) {
            const ssize_t r = ::pread(fd, p, bytes, (off_t)off);
            if (r <= 0) return false;
            p += r;
            off += (uint64_t)r;
            bytes -= (uint64_t)r;
        }
        return true;
    };
    BinHeader h;
    if (fsize < sizeof(h) || !pread_all(&h, sizeof(h), 0)) {
        err = "binary points: file shorter than its header";
        return COLO_ERR_PARSE;
    }
    if (std::memcmp(h.magic, kBinMagic, 8) != 0 || h.version != 1 || h.header_bytes != sizeof(h)) {
        err = "binary points: not a version-1 point file";
        return COLO_ERR_PARSE;
    }
    const uint64_t body = fsize - sizeof(h);
    if (h.n > body / 12 || h.nfeat > (body - 12 * h.n) / 4 || h.name_bytes != body - 12 * h.n - 4 * h.nfeat) {
        err = "binary points: sizes in the header do not match the file (truncated or corrupt)";
        return COLO_ERR_PARSE;
    }
    const uint64_t n = h.n;
    hp.clear();
    hp.x.resize(n);
    hp.y.resize(n);
    hp.raw.resize(n);
    // the three columns read in parallel, each straight into its array
    void* dst[3] = {hp.x.data(), hp.y.data(), hp.raw.data()};
    bool ok3[3] = {true, true, true};
    run_threads(n >= (1u << 20) ? 3u : 1u, [&](unsigned t) {
        for (unsigned i = t; i < 3; i += (n >= (1u << 20) ? 3u : 1u))
            if (n) ok3[i] = pread_all(dst[i], n * 4, sizeof(h) + 4 * n * i);
    });
    std::vector<uint32_t> len(h.nfeat);
    std::string names(h.name_bytes, '\0');
    if (!ok3[0] || !ok3[1] || !ok3[2] || (h.nfeat && !pread_all(len.data(), h.nfeat * 4, sizeof(h) + 12 * n)) ||
        (h.name_bytes && !pread_all(&names[0], h.name_bytes, sizeof(h) + 12 * n + 4 * h.nfeat))) {
        err = std::string("cannot read dataset: ") + path;
        return COLO_ERR_IO;
    }
    std::memcpy(hp.bounds, h.bounds, sizeof(hp.bounds));
    bool minus_one = false;
    const std::vector<uint64_t> starts = group_starts(hp.raw.data(), n, &minus_one);
    if (minus_one) {
        err = "binary points: feature id -1 is the reference's 'no feature yet' marker";
        return COLO_ERR_PARSE;
    }
    if (starts.size() != h.nfeat) {
        err = "binary points: the ids form " + std::to_string(starts.size()) + " features, the file names " +
              std::to_string(h.nfeat);
        return COLO_ERR_PARSE;
    }
    uint64_t used = 0;
    hp.tokens.reserve(starts.size());
    for (uint64_t g = 0; g < starts.size(); ++g) {
        if (len[g] > h.name_bytes - used) {
            err = "binary points: name lengths exceed the name table";
            return COLO_ERR_PARSE;
        }
        hp.tokens.emplace_back(starts[g], names.substr(used, len[g]));
        used += len[g];
    }
    if (used != h.name_bytes) {
        err = "binary points: name lengths do not cover the name table";
        return COLO_ERR_PARSE;
    }
    hp.tokens_complete = true;
    return COLO_OK;
}

// savetoFileGen format (colocationFinder.cpp:979-997).
colo_status write_patterns(const MineResult& r, const std::vector<std::string>& names, const char* location,
                           std::string& err) {
    for (const LevelTrace& L : r.levels) {
        std::string fn = std::string(location) + "ColocationDegree_" + std::to_string(L.k) + ".txt";
        FILE* fo = std::fopen(fn.c_str(), "wb");
        if (!fo) {
            err = "cannot write " + fn;
            return COLO_ERR_IO;
        }
        size_t C = L.prevalent.size();
        for (size_t c = 0; c < C; ++c) {
            if (!L.prevalent[c]) continue;
            std::fputs("( ", fo);
            for (uint32_t j = 0; j < L.k; ++j) {
                std::fputs(names[L.cand[c * L.k + j] - L.f0].c_str(), fo);
                std::fputs(" ", fo);
                std::fputs(j != L.k - 1 ? "| " : ")\n", fo);
            }
        }
        std::fclose(fo);
    }
    return COLO_OK;
}

}  // namespace colo
