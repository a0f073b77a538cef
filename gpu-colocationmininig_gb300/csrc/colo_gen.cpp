// colo_gen.cpp -- seeded synthetic point sets with planted colocations.
//
// There is no public dataset for this benchmark: the workloads are synthetic
// by definition.  Each feature's instances are either planted (one instance
// of every member of a planted pattern around a shared seed centre,
// isotropic Gaussian offset), clustered in Gaussian hotspots that belong to
// that feature, or uniform.  Points are emitted grouped by feature (feature
// ids 0..F-1), the layout the reference's reader requires.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

struct Rng {
    uint64_t s[4];
    static uint64_t splitmix(uint64_t& z) {
        z += 0x9e3779b97f4a7c15ull;
        uint64_t r = z;
        r = (r ^ (r >> 30)) * 0xbf58476d1ce4e5b9ull;
        r = (r ^ (r >> 27)) * 0x94d049bb133111ebull;
        return r ^ (r >> 31);
    }
    explicit Rng(uint64_t seed) {
        uint64_t z = seed;
        for (auto& v : s) v = splitmix(z);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {   // xoshiro256**
        uint64_t r = rotl(s[1] * 5, 7) * 9;
        uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    double u01() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    uint64_t below(uint64_t n) { return n ? next() % n : 0; }
    // Irwin-Hall(12) - 6: mean 0, variance 1, only additions (platform-stable).
    double gauss() {
        double t = 0;
        for (int i = 0; i < 12; ++i) t += u01();
        return t - 6.0;
    }
};

// Logarithm and exponential from IEEE-754 basic operations only (this file is
// compiled with -ffp-contract=off), so the generated points are the same bits
// on every platform; libm's log/exp/pow may differ in the last place between
// architectures.  log: x = m * 2^e with m in [sqrt(1/2), sqrt(2)), then
// log m = 2 atanh(t), t = (m - 1) / (m + 1), by its odd power series
// (|t| <= 0.172, 24 terms).  exp: x = k ln2 + r with |r| <= ln2 / 2, then
// the Taylor series of e^r (28 terms) scaled by 2^k.
constexpr double kLn2 = 0.69314718055994530942;

double det_log(double x) {
    int e = 0;
    double m = std::frexp(x, &e);
    if (m < 0.70710678118654752440) {
        m *= 2.0;
        e -= 1;
    }
    const double t = (m - 1.0) / (m + 1.0), t2 = t * t;
    double s = 0.0, p = t;
    for (int i = 0; i < 24; ++i) {
        s += p / (double)(2 * i + 1);
        p *= t2;
    }
    return 2.0 * s + (double)e * kLn2;
}

double det_exp(double x) {
    const double k = std::floor(x / kLn2 + 0.5);
    const double r = x - k * kLn2;
    double s = 1.0, term = 1.0;
    for (int i = 1; i < 28; ++i) {
        term *= r / (double)i;
        s += term;
    }
    return std::ldexp(s, (int)k);
}

}  // namespace

extern "C" {

typedef struct {
    uint64_t n;              // total points
    uint32_t nfeat;
    double zipf_s;           // 0 = equal sizes
    double width;            // domain [0, width)^2
    double hot_frac;         // fraction of non-planted points in hotspots
    uint32_t nhot;
    double hot_sig_lo, hot_sig_hi;   // hotspot sigma, log-uniform
    double dense_frac;       // extra fraction of each feature in dense hotspots
    uint32_t ndense;
    double dense_sigma;
    uint32_t npat;
    uint32_t pat_min, pat_max;
    double pat_sigma;        // planted offset sigma
    double seed_frac;        // seeds per pattern = seed_frac * min member count / share
    uint64_t seed;
    int32_t config0;         // 1: the fixed three patterns of the small plain config
    int32_t pad;
} colo_gen_spec;

// Fills x[n], y[n], fid[n] (grouped by feature) and bounds; returns the
// number of planted patterns written to pat_members (npat * pat_max entries,
// unused slots = -1) when non-NULL.
int colo_gen_points(const colo_gen_spec* sp, float* x, float* y, int32_t* fid, float* bounds,
                    int32_t* pat_members) {
    const uint64_t N = sp->n;
    const uint32_t F = sp->nfeat;
    if (F == 0 || N < F) return -1;
    Rng rng(sp->seed);
    // ---- feature sizes ----
    std::vector<uint64_t> cnt(F, 0);
    if (sp->zipf_s <= 0) {
        for (uint32_t f = 0; f < F; ++f) cnt[f] = N / F + (f < N % F ? 1 : 0);
    } else {
        std::vector<double> w(F);
        double H = 0;
        for (uint32_t f = 0; f < F; ++f) H += (w[f] = det_exp(-sp->zipf_s * det_log((double)(f + 1))));
        uint64_t tot = 0;
        for (uint32_t f = 0; f < F; ++f) {
            cnt[f] = std::max<uint64_t>(1, (uint64_t)std::floor((double)N * w[f] / H));
            tot += cnt[f];
        }
        for (uint32_t f = 0; tot < N; f = (f + 1) % F, ++tot) cnt[f]++;
        for (uint32_t f = 0; tot > N; f = (f + 1) % F)
            if (cnt[f] > 1) {
                cnt[f]--;
                --tot;
            }
    }
    // ---- planted patterns ----
    std::vector<std::vector<uint32_t>> pats;
    if (sp->config0) {
        pats = {{0, 1}, {2, 3, 4}, {5, 6, 7, 8}};
    } else {
        // PI is the smallest member participation ratio, so a planted pattern
        // is prevalent only when its members have similar counts: members are
        // a window of consecutive size ranks, away from the Zipf head where
        // neighbouring ranks differ most.
        for (uint32_t p = 0; p < sp->npat; ++p) {
            uint32_t sz = sp->pat_min + (uint32_t)rng.below(sp->pat_max - sp->pat_min + 1);
            if (sz > F) sz = F;
            uint32_t lo = std::min<uint32_t>(2 * sp->pat_max, F - sz);
            uint32_t start = lo + (uint32_t)rng.below(F - sz - lo + 1);
            std::vector<uint32_t> m;
            for (uint32_t t = 0; t < sz; ++t) m.push_back(start + t);
            pats.push_back(m);
        }
    }
    std::vector<uint32_t> share(F, 0);
    for (auto& p : pats)
        for (uint32_t f : p) share[f]++;
    std::vector<uint64_t> seeds(pats.size());
    for (size_t p = 0; p < pats.size(); ++p) {
        double mn = 1e300;
        for (uint32_t f : pats[p]) mn = std::min(mn, (double)cnt[f] / share[f]);
        seeds[p] = sp->config0 ? 1200 : (uint64_t)std::floor(sp->seed_frac * mn);
    }
    // ---- hotspots (each belongs to one feature, chosen by size) ----
    struct Hot { double cx, cy, sig; };
    std::vector<std::vector<Hot>> hot(F);
    std::vector<Hot> dense;   // shared by all features: every feature sends dense_frac of its points there
    auto pick_feature = [&]() {
        uint64_t r = rng.below(N);
        for (uint32_t f = 0; f < F; ++f) {
            if (r < cnt[f]) return f;
            r -= cnt[f];
        }
        return F - 1;
    };
    const double W = sp->width;
    for (uint32_t h = 0; h < sp->nhot; ++h) {
        uint32_t f = pick_feature();
        double lo = det_log(sp->hot_sig_lo), hi = det_log(sp->hot_sig_hi);
        hot[f].push_back({rng.u01() * W, rng.u01() * W, det_exp(lo + rng.u01() * (hi - lo))});
    }
    for (uint32_t h = 0; h < sp->ndense; ++h) dense.push_back({rng.u01() * W, rng.u01() * W, sp->dense_sigma});
    auto clampw = [&](double v) {
        if (v < 0) v = 0;
        if (v >= W) v = std::nextafter(W, 0.0);
        float fv = (float)v;
        if ((double)fv >= W) fv = std::nextafter((float)W, 0.0f);
        return fv;
    };
    auto place = [&](double cx, double cy, double sig, float* ox, float* oy) {
        double px = 0, py = 0;
        for (int t = 0; t < 8; ++t) {
            px = cx + sig * rng.gauss();
            py = cy + sig * rng.gauss();
            if (px >= 0 && px < W && py >= 0 && py < W) break;
        }
        *ox = clampw(px);
        *oy = clampw(py);
    };
    // ---- emit, grouped by feature ----
    std::vector<uint64_t> start(F + 1, 0);
    for (uint32_t f = 0; f < F; ++f) start[f + 1] = start[f] + cnt[f];
    std::vector<uint64_t> cur(start.begin(), start.end() - 1);
    for (size_t p = 0; p < pats.size(); ++p)
        for (uint64_t s = 0; s < seeds[p]; ++s) {
            double cx = rng.u01() * W, cy = rng.u01() * W;
            for (uint32_t f : pats[p]) {
                if (cur[f] >= start[f + 1]) continue;
                uint64_t i = cur[f]++;
                place(cx, cy, sp->pat_sigma, &x[i], &y[i]);
            }
        }
    for (uint32_t f = 0; f < F; ++f) {
        uint64_t left = start[f + 1] - cur[f];
        uint64_t nd = dense.empty() ? 0 : (uint64_t)std::floor(sp->dense_frac * (double)cnt[f]);
        if (nd > left) nd = left;
        for (uint64_t t = 0; t < nd; ++t) {
            const Hot& h = dense[rng.below(dense.size())];
            uint64_t i = cur[f]++;
            place(h.cx, h.cy, h.sig, &x[i], &y[i]);
        }
        while (cur[f] < start[f + 1]) {
            uint64_t i = cur[f]++;
            if (!hot[f].empty() && rng.u01() < sp->hot_frac) {
                const Hot& h = hot[f][rng.below(hot[f].size())];
                place(h.cx, h.cy, h.sig, &x[i], &y[i]);
            } else {
                x[i] = clampw(rng.u01() * W);
                y[i] = clampw(rng.u01() * W);
            }
        }
        for (uint64_t i = start[f]; i < start[f + 1]; ++i) fid[i] = (int32_t)f;
    }
    bounds[0] = 0.0f;
    bounds[1] = 0.0f;
    bounds[2] = (float)W;
    bounds[3] = (float)W;
    if (pat_members) {
        uint32_t mx = std::max<uint32_t>(sp->pat_max, 4);
        for (size_t p = 0; p < pats.size(); ++p)
            for (uint32_t t = 0; t < mx; ++t) pat_members[p * mx + t] = t < pats[p].size() ? (int32_t)pats[p][t] : -1;
    }
    return (int)pats.size();
}

}  // extern "C"
