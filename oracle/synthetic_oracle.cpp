// Test infrastructure (oracle only): the seeded synthetic workloads, generated
// on the CPU without the product library, so that the CPU arm of the benchmark
// (the oracle's LM solve) runs with nothing of the product loaded. Same random
// stream and draw order as the product's generator, so the two produce
// bit-identical problems (a CPU test checks this):
//   xoshiro256** seeded by splitmix64, normal deviates by Box-Muller (cosine
//   first, sine kept as the spare); cameras (angle-axis N(0,0.1), t N(0,1),
//   f U(400,600), k1 N(0,1e-2), k2 N(0,1e-4)); points x,y U(-3,3), z U(-10,-3);
//   discrete power-law track lengths by inverse CDF; distinct cameras drawn
//   until the point is in front (camera z < -1) and inside |u|,|v| <= 1.5;
//   observation = projection (BAL camera model, reference
//   src/bal_reader.cpp:100-128) + N(0,1) px (outliers N(0,sigma)); stable sort
//   camera-major; initial estimate = truth + N(0,0.01) per camera parameter and
//   N(0,0.05) per point coordinate.
// Built with -ffp-contract=off.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

struct Stream {
    uint64_t s[4];
    bool spare_ok = false;
    double spare = 0.0;

    explicit Stream(uint64_t seed) {
        uint64_t z = seed;
        for (uint64_t& w : s) {
            z += 0x9e3779b97f4a7c15ull;
            uint64_t x = z;
            x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
            x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
            w = x ^ (x >> 31);
        }
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t bits() {
        const uint64_t out = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return out;
    }
    double unit() { return (bits() >> 11) * (1.0 / 9007199254740992.0); }
    double range(double a, double b) { return a + (b - a) * unit(); }
    double gauss() {
        if (spare_ok) {
            spare_ok = false;
            return spare;
        }
        double u1 = unit();
        while (u1 <= 0.0) u1 = unit();
        const double u2 = unit();
        const double rad = std::sqrt(-2.0 * std::log(u1));
        const double ang = 6.283185307179586 * u2;
        spare = rad * std::sin(ang);
        spare_ok = true;
        return rad * std::cos(ang);
    }
    double gauss(double sigma) { return sigma * gauss(); }
    int pick(int n) { return static_cast<int>(unit() * n); }
};

// Rotate by the angle-axis vector and translate (BAL camera, reference src/bal_reader.cpp:100-121).
void camera_point(const double* cam, const double* X, double* P) {
    const double th = std::sqrt(cam[0] * cam[0] + cam[1] * cam[1] + cam[2] * cam[2]);
    if (th > 1e-12) {
        const double w0 = cam[0] / th, w1 = cam[1] / th, w2 = cam[2] / th;
        const double c = std::cos(th), s = std::sin(th);
        const double wX = w0 * X[0] + w1 * X[1] + w2 * X[2];
        const double k = wX * (1.0 - c);
        P[0] = X[0] * c + (w1 * X[2] - w2 * X[1]) * s + w0 * k + cam[3];
        P[1] = X[1] * c + (w2 * X[0] - w0 * X[2]) * s + w1 * k + cam[4];
        P[2] = X[2] * c + (w0 * X[1] - w1 * X[0]) * s + w2 * k + cam[5];
    } else {
        P[0] = X[0] + cam[3];
        P[1] = X[1] + cam[4];
        P[2] = X[2] + cam[5];
    }
}

// Projection (reference src/bal_reader.cpp:122-128).
void project(const double* cam, const double* X, double* px) {
    double P[3];
    camera_point(cam, X, P);
    const double u = -P[0] / P[2], v = -P[1] / P[2];
    const double r2 = u * u + v * v;
    const double d = 1.0 + cam[7] * r2 + cam[8] * r2 * r2;
    px[0] = cam[6] * d * u - 0.0;  // the residual against a zero observation
    px[1] = cam[6] * d * v - 0.0;
}

struct Shape {
    int C, P, kmin, kmax;
    double alpha, out_frac, out_sigma;
};

bool shape_of(int id, Shape* s) {
    switch (id) {
        case 1: *s = {16, 22000, 2, 8, 1.29, 0.0, 0.0}; return true;
        case 2: *s = {257, 65000, 2, 12, 2.23, 0.0, 0.0}; return true;
        case 3: *s = {1000, 200000, 2, 16, 2.05, 0.0, 0.0}; return true;
        case 4: *s = {1000, 200000, 2, 16, 2.05, 0.0, 0.0}; return true;
        case 5: *s = {5000, 1500000, 2, 200, 2.2, 0.05, 20.0}; return true;
        default: return false;
    }
}

struct Obs {
    int c, p;
    double x, y;
};

struct Generated {
    std::vector<double> cams, pts, px;
    std::vector<int> oc, op;
};

Generated generate(const Shape& sh, uint64_t seed) {
    Stream rng(seed);
    const int C = sh.C, P = sh.P;
    std::vector<double> tc(9ull * C), tp(3ull * P);
    for (int c = 0; c < C; ++c) {
        double* cam = &tc[9ull * c];
        for (int i = 0; i < 3; ++i) cam[i] = rng.gauss(0.1);
        for (int i = 3; i < 6; ++i) cam[i] = rng.gauss(1.0);
        cam[6] = rng.range(400.0, 600.0);
        cam[7] = rng.gauss(1e-2);
        cam[8] = rng.gauss(1e-4);
    }
    for (int p = 0; p < P; ++p) {
        double* X = &tp[3ull * p];
        X[0] = rng.range(-3.0, 3.0);
        X[1] = rng.range(-3.0, 3.0);
        X[2] = rng.range(-10.0, -3.0);
    }
    const int kmax = std::min(sh.kmax, C);
    std::vector<double> cdf;
    double tot = 0.0;
    for (int k = sh.kmin; k <= kmax; ++k) tot += std::pow(static_cast<double>(k), -sh.alpha);
    double acc = 0.0;
    for (int k = sh.kmin; k <= kmax; ++k) {
        acc += std::pow(static_cast<double>(k), -sh.alpha) / tot;
        cdf.push_back(acc);
    }
    cdf.back() = 1.0;
    std::vector<Obs> obs;
    obs.reserve(static_cast<size_t>(P) * 6);
    std::vector<int> seen;
    std::vector<char> taken(C, 0);
    for (int p = 0; p < P; ++p) {
        const double u = rng.unit();
        const int want = sh.kmin + static_cast<int>(std::lower_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
        seen.clear();
        const double* X = &tp[3ull * p];
        for (int attempt = 0; attempt < 64 * C && static_cast<int>(seen.size()) < want; ++attempt) {
            const int c = rng.pick(C);
            if (taken[c]) continue;
            double Pc[3];
            camera_point(&tc[9ull * c], X, Pc);
            if (!(Pc[2] < -1.0)) continue;
            const double uu = -Pc[0] / Pc[2], vv = -Pc[1] / Pc[2];
            if (std::fabs(uu) > 1.5 || std::fabs(vv) > 1.5) continue;
            taken[c] = 1;
            seen.push_back(c);
        }
        for (int c : seen) taken[c] = 0;
        for (int c : seen) {
            double pred[2];
            project(&tc[9ull * c], X, pred);
            const bool outlier = sh.out_frac > 0.0 && rng.unit() < sh.out_frac;
            const double sigma = outlier ? sh.out_sigma : 1.0;
            const double nx = rng.gauss(sigma), ny = rng.gauss(sigma);
            obs.push_back({c, p, pred[0] + nx, pred[1] + ny});
        }
    }
    std::stable_sort(obs.begin(), obs.end(), [](const Obs& a, const Obs& b) { return a.c < b.c; });
    Generated g;
    g.oc.resize(obs.size());
    g.op.resize(obs.size());
    g.px.resize(2 * obs.size());
    for (size_t i = 0; i < obs.size(); ++i) {
        g.oc[i] = obs[i].c;
        g.op[i] = obs[i].p;
        g.px[2 * i] = obs[i].x;
        g.px[2 * i + 1] = obs[i].y;
    }
    g.cams = tc;
    for (double& v : g.cams) v += rng.gauss(0.01);
    g.pts = tp;
    for (double& v : g.pts) v += rng.gauss(0.05);
    return g;
}

Generated g_last;

}  // namespace

extern "C" {

// Generates workload `id` (1..5) with `seed` into an internal buffer; returns
// 0 and the sizes, or 1 for an unknown id. oracle_synthetic_copy copies it out.
int oracle_synthetic(int id, unsigned long long seed, int* C, int* P, int* E) {
    Shape sh;
    if (!shape_of(id, &sh)) return 1;
    g_last = generate(sh, seed);
    *C = sh.C;
    *P = sh.P;
    *E = static_cast<int>(g_last.oc.size());
    return 0;
}

void oracle_synthetic_copy(double* cams, double* pts, int* oc, int* op, double* px) {
    std::memcpy(cams, g_last.cams.data(), g_last.cams.size() * sizeof(double));
    std::memcpy(pts, g_last.pts.data(), g_last.pts.size() * sizeof(double));
    std::memcpy(oc, g_last.oc.data(), g_last.oc.size() * sizeof(int));
    std::memcpy(op, g_last.op.data(), g_last.op.size() * sizeof(int));
    std::memcpy(px, g_last.px.data(), g_last.px.size() * sizeof(double));
    g_last = Generated();
}

}  // extern "C"
