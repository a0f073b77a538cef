// colo_io.cpp -- input formats of the reference: config file, parameter
// file and the point CSV; output: ColocationDegree_<k>.txt pattern files.
#include <cerrno>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

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

// std::stof: leading whitespace skipped, longest numeric prefix, at least one
// character consumed.
bool parse_float(const std::string& s, float* v) {
    const char* p = s.c_str();
    const char* e = p + s.size();
    while (p < e && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\v' || *p == '\f' || *p == '\r')) ++p;
    bool slow = (p < e && *p == '+');
    for (const char* q = p; q < e && !slow; ++q)
        if (*q == 'x' || *q == 'X') slow = true;
    if (!slow) {
        auto r = std::from_chars(p, e, *v, std::chars_format::general);
        if (r.ec == std::errc()) return true;
        if (r.ec == std::errc::result_out_of_range) slow = true;
        else return false;
    }
    char* endp = nullptr;
    errno = 0;
    *v = std::strtof(s.c_str(), &endp);
    return endp != s.c_str() && errno != ERANGE;
}

// std::stoi
bool parse_int(const std::string& s, long* v) {
    const char* b = s.c_str();
    char* e = nullptr;
    errno = 0;
    long r = std::strtol(b, &e, 10);
    if (e == b || errno == ERANGE || r < INT32_MIN || r > INT32_MAX) return false;
    *v = r;
    return true;
}

struct LineReader {
    std::vector<char> buf;
    size_t pos = 0;
    bool ok = false;
    explicit LineReader(const char* path) {
        FILE* f = std::fopen(path, "rb");
        if (!f) return;
        std::fseek(f, 0, SEEK_END);
        long sz = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        buf.resize(sz > 0 ? (size_t)sz : 0);
        if (sz > 0 && std::fread(buf.data(), 1, (size_t)sz, f) != (size_t)sz) {
            std::fclose(f);
            return;
        }
        std::fclose(f);
        ok = true;
    }
    // std::getline; a trailing '\r' is dropped.  Returns false at end of data.
    bool next(const char** b, const char** e) {
        if (pos >= buf.size()) {
            *b = *e = nullptr;
            return false;
        }
        const char* s = buf.data() + pos;
        const char* end = buf.data() + buf.size();
        const char* nl = (const char*)std::memchr(s, '\n', end - s);
        const char* le = nl ? nl : end;
        pos = (size_t)(le - buf.data()) + (nl ? 1 : 0);
        if (le > s && le[-1] == '\r') --le;
        *b = s;
        *e = le;
        return true;
    }
};

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

colo_status parse_points_csv(const char* path, HostPoints& hp, std::string& err) {
    LineReader rd(path);
    if (!rd.ok) {
        err = std::string("cannot read dataset: ") + path;
        return COLO_ERR_IO;
    }
    const char *b, *e;
    std::vector<std::string> f;
    rd.next(&b, &e);
    long N = 0;
    if (!parse_int(std::string(b ? b : "", b ? e - b : 0), &N) || N < 0) {
        err = "dataset: first line must hold the point count";
        return COLO_ERR_PARSE;
    }
    hp.clear();
    hp.x.reserve(N);
    hp.y.reserve(N);
    hp.raw.reserve(N);
    uint64_t line_no = 1;
    while (rd.next(&b, &e) && e > b) {
        ++line_no;
        split_fields(b, e, f);
        long id;
        float xv, yv;
        if (f.size() < 3 || !parse_int(f[0], &id) || !parse_float(f[1], &xv) || !parse_float(f[2], &yv)) {
            err = "dataset: malformed point line " + std::to_string(line_no);
            return COLO_ERR_PARSE;
        }
        if (id == -1) {
            err = "dataset: feature id -1 is the reference's 'no feature yet' marker (line " +
                  std::to_string(line_no) + ")";
            return COLO_ERR_PARSE;
        }
        hp.raw.push_back((int32_t)id);
        hp.first_token.push_back(f[0]);
        hp.x.push_back(xv);
        hp.y.push_back(yv);
    }
    if ((long)hp.x.size() != N) {
        err = "dataset: count line says " + std::to_string(N) + " points, found " + std::to_string(hp.x.size());
        return COLO_ERR_PARSE;
    }
    if (!rd.next(&b, &e)) {
        err = "dataset: bounds line missing";
        return COLO_ERR_PARSE;
    }
    split_fields(b, e, f);
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
                             const std::vector<uint32_t>& feat, const char* path, std::string& err) {
    FILE* fo = std::fopen(path, "wb");
    if (!fo) {
        err = std::string("cannot write ") + path;
        return COLO_ERR_IO;
    }
    std::fprintf(fo, "%zu\n", hp.x.size());
    for (size_t i = 0; i < hp.x.size(); ++i)
        std::fprintf(fo, "%s,%.9g,%.9g\n", names[feat[i]].c_str(), (double)hp.x[i], (double)hp.y[i]);
    std::fprintf(fo, "\n%.9g,%.9g,%.9g,%.9g", (double)hp.bounds[0], (double)hp.bounds[1],
                 (double)hp.bounds[2], (double)hp.bounds[3]);
    std::fclose(fo);
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
