#pragma once
// Seeded synthetic BAL-shaped problems (the BAL datasets are not available
// offline; these stand in for them with the same shapes).

#include <cstdint>

#include "gba/bal_problem.hpp"

namespace gba {

struct SyntheticConfig {
    int num_cameras;
    int num_points;
    int track_min, track_max;  // track length range (observations per point)
    double track_alpha;        // discrete power law P(k) ~ k^-alpha on [min, max]
    double outlier_fraction;   // share of observations with outlier noise
    double outlier_sigma;      // px
    // > 0: spatially local covisibility, as along a camera path: camera c's
    // centre lies at x = 0.5 c on the x axis, points spread along the path, and
    // a point's track takes cameras within +-window of the camera nearest to it
    // (the camera graph is then a band); 0: cameras anywhere, tracks drawn from all
    int window = 0;
};

// Workloads 1..5:
//   1: 16 cameras / 22,000 points, tracks 2-8   (alpha 1.29, ~84k observations)
//   2: 257 / 65,000, tracks 2-12                (alpha 2.23, ~225k)
//   3: 1,000 / 200,000, tracks 2-16             (alpha 2.05, ~800k)
//   4: the workload-3 shape (use a different seed)
//   5: 5,000 / 1,500,000, tracks 2-200          (alpha 2.2, ~8.8M), 5% outliers N(0, 20 px)
SyntheticConfig synthetic_config(int id);

// Generates a problem: truth cameras (angle-axis ~N(0,0.1), t ~N(0,1),
// f ~U(400,600), k1 ~N(0,1e-2), k2 ~N(0,1e-4)), truth points uniform in
// x,y in [-3,3], z in [-10,-3] (in front of the rig: camera-frame z < -1),
// each point observed by k distinct random cameras that see it in front,
// observations = projection + N(0,1) px (outliers N(0, sigma)), then the
// initial estimate perturbs every camera parameter by N(0,0.01) and every
// point coordinate by N(0,0.05). Observations are emitted camera-major like the
// BAL files. If truth is non-null it receives the unperturbed parameters.
BALProblem make_synthetic(const SyntheticConfig& cfg, uint64_t seed, BALProblem* truth = nullptr);

// The reference's launch-bounds regression problem (tests/test_launch_bounds.cpp:
// 28-80): 8 cameras on a fixed formula, 400,000 points from std::mt19937_64(7),
// two noise-free observations per point, points perturbed by U(-0.05, 0.05).
BALProblem make_launch_bounds_problem(int num_points = 400000);

}  // namespace gba
