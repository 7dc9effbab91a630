#pragma once
// Drop-in problem container and CPU camera model of the gba API.
//
// Interface kept identical to the reference (include/gba/bal_problem.hpp:15-50):
// same struct name, member names, member order and free functions, so reference
// callers compile unchanged. The implementation (gpu-bundle-adjustment_gb300/csrc/bal_io.cpp)
// is this project's own.

#include <string>
#include <vector>

namespace gba {

// Bundle-adjustment problem in the BAL structure-of-arrays layout.
//   cameras: 9 doubles per camera = Rodrigues rotation[3], translation[3],
//            focal length, k1, k2.
//   points:  3 doubles per point.
//   obs_camera / obs_point: camera and point index of each observation.
//   obs_pixel: 2 doubles per observation (x, y interleaved).
struct BALProblem {
    int num_cameras = 0;
    int num_points = 0;
    int num_observations = 0;

    std::vector<double> cameras;   // 9 * num_cameras
    std::vector<double> points;    // 3 * num_points

    std::vector<int> obs_camera;    // num_observations
    std::vector<int> obs_point;     // num_observations
    std::vector<double> obs_pixel;  // 2 * num_observations

    const double* camera(int i) const { return cameras.data() + 9 * i; }
    double* camera(int i) { return cameras.data() + 9 * i; }
    const double* point(int i) const { return points.data() + 3 * i; }
    double* point(int i) { return points.data() + 3 * i; }
};

// Reads a BAL text file (or a .bz2 file, decompressed through `bzcat`).
// Throws std::runtime_error on a malformed header, an index out of range,
// trailing data or a read failure (reference: src/bal_reader.cpp:66-98).
BALProblem load_bal(const std::string& path);

// Writes a BAL text file that load_bal reads back bit-exactly (%.17g).
// Additive: the reference has no writer in its library.
void write_bal(const std::string& path, const BALProblem& p);

// Snavely reprojection residual of one observation, on the CPU:
//   P = R(rodrigues) X + t,  p = -P / P.z,  d = 1 + k1 |p|^2 + k2 |p|^4,
//   residual = f d p - observed.
// Rotation applied with the Rodrigues formula when |rodrigues| > 1e-12,
// else P = X + t (reference: src/bal_reader.cpp:100-128).
void snavely_residual(const double* camera9, const double* point3,
                      const double* observed2, double* out2);

// Sum of squared residuals over all observations (reference:
// src/bal_reader.cpp:130-139). Cost = total_squared_error / 2.
double total_squared_error(const BALProblem& p);

}  // namespace gba
