// Seeded synthetic problem generator (host). Own xoshiro256** stream; normal
// deviates by the Box-Muller transform. Built with -ffp-contract=off.

#include "synthetic.hpp"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <random>
#include <stdexcept>
#include <vector>

namespace gba {
namespace {

class Rng {
public:
    explicit Rng(uint64_t seed) {
        uint64_t z = seed;
        for (auto& w : s_) {
            z += 0x9e3779b97f4a7c15ull;
            uint64_t x = z;
            x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
            x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
            w = x ^ (x >> 31);
        }
    }
    uint64_t next() {
        const uint64_t r = rotl(s_[1] * 5, 7) * 9;
        const uint64_t t = s_[1] << 17;
        s_[2] ^= s_[0];
        s_[3] ^= s_[1];
        s_[1] ^= s_[2];
        s_[0] ^= s_[3];
        s_[2] ^= t;
        s_[3] = rotl(s_[3], 45);
        return r;
    }
    double uniform() { return (next() >> 11) * (1.0 / 9007199254740992.0); }  // [0, 1)
    double uniform(double a, double b) { return a + (b - a) * uniform(); }
    double normal() {
        if (have_spare_) {
            have_spare_ = false;
            return spare_;
        }
        double u1 = uniform();
        while (u1 <= 0.0) u1 = uniform();
        const double u2 = uniform();
        const double r = std::sqrt(-2.0 * std::log(u1));
        const double th = 6.283185307179586 * u2;
        spare_ = r * std::sin(th);
        have_spare_ = true;
        return r * std::cos(th);
    }
    double normal(double sigma) { return sigma * normal(); }
    int below(int n) { return static_cast<int>(uniform() * n); }

private:
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t s_[4];
    bool have_spare_ = false;
    double spare_ = 0.0;
};

// Camera-frame point of X for camera cam (Rodrigues + translation).
void to_camera(const double* cam, const double* X, double* P) {
    const double th = std::sqrt(cam[0] * cam[0] + cam[1] * cam[1] + cam[2] * cam[2]);
    if (th > 1e-12) {
        const double w0 = cam[0] / th, w1 = cam[1] / th, w2 = cam[2] / th;
        const double c = std::cos(th), s = std::sin(th);
        const double wX = w0 * X[0] + w1 * X[1] + w2 * X[2];
        P[0] = X[0] * c + (w1 * X[2] - w2 * X[1]) * s + w0 * wX * (1.0 - c) + cam[3];
        P[1] = X[1] * c + (w2 * X[0] - w0 * X[2]) * s + w1 * wX * (1.0 - c) + cam[4];
        P[2] = X[2] * c + (w0 * X[1] - w1 * X[0]) * s + w2 * wX * (1.0 - c) + cam[5];
    } else {
        for (int i = 0; i < 3; ++i) P[i] = X[i] + cam[3 + i];
    }
}

}  // namespace

SyntheticConfig synthetic_config(int id) {
    switch (id) {
        case 1: return {16, 22000, 2, 8, 1.29, 0.0, 0.0};
        case 2: return {257, 65000, 2, 12, 2.23, 0.0, 0.0};
        case 3: return {1000, 200000, 2, 16, 2.05, 0.0, 0.0};
        case 4: return {1000, 200000, 2, 16, 2.05, 0.0, 0.0};
        case 5: return {5000, 1500000, 2, 200, 2.2, 0.05, 20.0};
        default: throw std::invalid_argument("synthetic workload id must be 1..5");
    }
}

BALProblem make_synthetic(const SyntheticConfig& cfg, uint64_t seed, BALProblem* truth_out) {
    const int C = cfg.num_cameras, P = cfg.num_points;
    if (C < 2 || P < 1 || cfg.track_min < 1 || cfg.track_max < cfg.track_min)
        throw std::invalid_argument("bad synthetic config");
    Rng rng(seed);

    BALProblem truth;
    truth.num_cameras = C;
    truth.num_points = P;
    truth.cameras.resize(9ull * C);
    const bool local = cfg.window > 0;
    constexpr double kSpacing = 0.5;  // local mode: distance between consecutive camera centres
    std::vector<double> centres(local ? 3ull * C : 0);
    for (int c = 0; c < C; ++c) {
        double* cam = truth.camera(c);
        for (int i = 0; i < 3; ++i) cam[i] = rng.normal(0.1);
        if (local) {
            // centre (0.5 c, ~0, ~0), t = -R centre
            const double ctr[3] = {kSpacing * c, rng.normal(0.1), rng.normal(0.1)};
            const double rot[9] = {cam[0], cam[1], cam[2], 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
            double rc[3];
            to_camera(rot, ctr, rc);  // R centre (the record's translation is zero)
            for (int i = 0; i < 3; ++i) {
                cam[3 + i] = -rc[i];
                centres[3ull * c + i] = ctr[i];
            }
        } else {
            for (int i = 3; i < 6; ++i) cam[i] = rng.normal(1.0);
        }
        cam[6] = rng.uniform(400.0, 600.0);
        cam[7] = rng.normal(1e-2);
        cam[8] = rng.normal(1e-4);
    }
    truth.points.resize(3ull * P);
    for (int p = 0; p < P; ++p) {
        double* X = truth.point(p);
        X[0] = local ? rng.uniform(-1.0, kSpacing * (C - 1) + 1.0) : rng.uniform(-3.0, 3.0);
        X[1] = rng.uniform(-3.0, 3.0);
        X[2] = rng.uniform(-10.0, -3.0);
    }

    // discrete power-law track lengths, inverse CDF over [min, max]
    const int kmax = std::min(cfg.track_max, local ? std::min(C, 2 * cfg.window + 1) : C);
    std::vector<double> cdf;
    double tot = 0.0;
    for (int k = cfg.track_min; k <= kmax; ++k) tot += std::pow(static_cast<double>(k), -cfg.track_alpha);
    double acc = 0.0;
    for (int k = cfg.track_min; k <= kmax; ++k) {
        acc += std::pow(static_cast<double>(k), -cfg.track_alpha) / tot;
        cdf.push_back(acc);
    }
    cdf.back() = 1.0;

    struct Obs {
        int c, p;
        double x, y;
    };
    std::vector<Obs> obs;
    obs.reserve(static_cast<size_t>(P) * 6);
    std::vector<int> chosen;
    std::vector<char> used(C, 0);
    for (int p = 0; p < P; ++p) {
        const double u = rng.uniform();
        const int want = cfg.track_min + static_cast<int>(std::lower_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
        chosen.clear();
        const double* X = truth.point(p);
        const int c_near = local ? std::min(C - 1, std::max(0, static_cast<int>(std::lround(X[0] / kSpacing)))) : 0;
        for (int attempt = 0; attempt < 64 * C && static_cast<int>(chosen.size()) < want; ++attempt) {
            const int c = local ? c_near - cfg.window + rng.below(2 * cfg.window + 1) : rng.below(C);
            if (c < 0 || c >= C) continue;
            if (used[c]) continue;
            double Pc[3];
            to_camera(truth.camera(c), X, Pc);
            if (!(Pc[2] < -1.0)) continue;  // in front of the camera, depth > 1
            const double uu = -Pc[0] / Pc[2], vv = -Pc[1] / Pc[2];
            if (std::fabs(uu) > 1.5 || std::fabs(vv) > 1.5) continue;  // inside the field of view
            used[c] = 1;
            chosen.push_back(c);
        }
        for (int c : chosen) used[c] = 0;
        for (int c : chosen) {
            const double zero[2] = {0.0, 0.0};
            double pred[2];
            snavely_residual(truth.camera(c), X, zero, pred);
            const bool outlier = cfg.outlier_fraction > 0.0 && rng.uniform() < cfg.outlier_fraction;
            const double sigma = outlier ? cfg.outlier_sigma : 1.0;
            const double nx = rng.normal(sigma), ny = rng.normal(sigma);
            obs.push_back({c, p, pred[0] + nx, pred[1] + ny});
        }
    }
    std::stable_sort(obs.begin(), obs.end(), [](const Obs& a, const Obs& b) { return a.c < b.c; });

    BALProblem prob;
    prob.num_cameras = C;
    prob.num_points = P;
    prob.num_observations = static_cast<int>(obs.size());
    prob.obs_camera.resize(obs.size());
    prob.obs_point.resize(obs.size());
    prob.obs_pixel.resize(2 * obs.size());
    for (size_t i = 0; i < obs.size(); ++i) {
        prob.obs_camera[i] = obs[i].c;
        prob.obs_point[i] = obs[i].p;
        prob.obs_pixel[2 * i] = obs[i].x;
        prob.obs_pixel[2 * i + 1] = obs[i].y;
    }
    prob.cameras = truth.cameras;
    if (local) {
        // the centre (not the translation, which grows with the distance from
        // the origin) and the rotation are perturbed, so every camera moves by
        // the same amount whatever its place on the path
        for (int c = 0; c < C; ++c) {
            double* cam = prob.camera(c);
            double n[9];
            for (double& v : n) v = rng.normal(0.01);
            for (int i = 0; i < 3; ++i) cam[i] += n[i];
            const double ctr[3] = {centres[3ull * c] + n[3], centres[3ull * c + 1] + n[4], centres[3ull * c + 2] + n[5]};
            const double rot[9] = {cam[0], cam[1], cam[2], 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
            double rc[3];
            to_camera(rot, ctr, rc);
            for (int i = 0; i < 3; ++i) cam[3 + i] = -rc[i];
            for (int i = 6; i < 9; ++i) cam[i] += n[i];
        }
    } else {
        for (double& v : prob.cameras) v += rng.normal(0.01);
    }
    prob.points = truth.points;
    for (double& v : prob.points) v += rng.normal(0.05);
    if (truth_out) {
        truth.num_observations = prob.num_observations;
        truth.obs_camera = prob.obs_camera;
        truth.obs_point = prob.obs_point;
        truth.obs_pixel = prob.obs_pixel;
        *truth_out = std::move(truth);
    }
    return prob;
}

BALProblem make_launch_bounds_problem(int num_points) {
    // Same generator steps as the reference regression test so the inputs are
    // identical: libstdc++ mt19937_64(7) with uniform_real_distribution draws
    // in the same order (x, y, z per point; then 3 perturbations per point).
    const int C = 8, P = num_points;
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> xy(-3.0, 3.0), zz(4.0, 12.0), pert(-0.05, 0.05);
    BALProblem truth, prob;
    truth.num_cameras = prob.num_cameras = C;
    truth.num_points = prob.num_points = P;
    truth.num_observations = prob.num_observations = 2 * P;
    truth.cameras.resize(9 * C);
    for (int i = 0; i < C; ++i) {
        double* c = truth.camera(i);
        const double fi = i;
        c[0] = 0.02 * (fi + 1.0);
        c[1] = -0.01 * fi;
        c[2] = 0.03;
        c[3] = 0.3 * fi;
        c[4] = -0.1 * fi;
        c[5] = 0.05 * fi;
        c[6] = 500.0 + 10.0 * fi;
        c[7] = -0.05;
        c[8] = 0.001;
    }
    truth.points.resize(3ull * P);
    for (int k = 0; k < P; ++k) {
        const double x = xy(rng);
        const double y = xy(rng);
        const double z = zz(rng);
        truth.points[3ull * k] = x;
        truth.points[3ull * k + 1] = y;
        truth.points[3ull * k + 2] = z;
    }
    prob.cameras = truth.cameras;
    prob.points = truth.points;
    for (int k = 0; k < P; ++k)
        for (int j = 0; j < 3; ++j) prob.points[3ull * k + j] += pert(rng);
    prob.obs_camera.resize(2ull * P);
    prob.obs_point.resize(2ull * P);
    prob.obs_pixel.assign(4ull * P, 0.0);
    for (int k = 0; k < P; ++k) {
        const int cams[2] = {k % C, (k + 1) % C};
        for (int m = 0; m < 2; ++m) {
            const size_t e = 2ull * k + m;
            prob.obs_camera[e] = cams[m];
            prob.obs_point[e] = k;
            const double zero[2] = {0.0, 0.0};
            double pred[2];
            snavely_residual(truth.camera(cams[m]), truth.point(k), zero, pred);
            prob.obs_pixel[2 * e] = pred[0];
            prob.obs_pixel[2 * e + 1] = pred[1];
        }
    }
    return prob;
}

}  // namespace gba
