// Test infrastructure: extern "C" wrappers over the reference's own BAL reader
// and CPU residual (reference src/bal_reader.cpp, compiled from its source by
// build_oracle.py against the reference's include/gba/bal_problem.hpp).

#include <cstring>
#include <exception>
#include <string>

#include "gba/bal_problem.hpp"

extern "C" {

int ref_snavely_residual(const double* cam, const double* pt, const double* obs, double* out2) {
    gba::snavely_residual(cam, pt, obs, out2);
    return 0;
}

double ref_total_squared_error(int C, int P, int E, const double* cams, const double* pts, const int* oc,
                               const int* op, const double* px) {
    gba::BALProblem p;
    p.num_cameras = C;
    p.num_points = P;
    p.num_observations = E;
    p.cameras.assign(cams, cams + 9ll * C);
    p.points.assign(pts, pts + 3ll * P);
    p.obs_camera.assign(oc, oc + E);
    p.obs_point.assign(op, op + E);
    p.obs_pixel.assign(px, px + 2ll * E);
    return gba::total_squared_error(p);
}

// Returns 0 and the dimensions, or 1 if load_bal threw.
int ref_load_bal_dims(const char* path, int* C, int* P, int* E) {
    try {
        const gba::BALProblem p = gba::load_bal(path);
        *C = p.num_cameras;
        *P = p.num_points;
        *E = p.num_observations;
        return 0;
    } catch (const std::exception&) {
        return 1;
    }
}

int ref_load_bal(const char* path, double* cams, double* pts, int* oc, int* op, double* px) {
    try {
        const gba::BALProblem p = gba::load_bal(path);
        std::memcpy(cams, p.cameras.data(), p.cameras.size() * sizeof(double));
        std::memcpy(pts, p.points.data(), p.points.size() * sizeof(double));
        std::memcpy(oc, p.obs_camera.data(), p.obs_camera.size() * sizeof(int));
        std::memcpy(op, p.obs_point.data(), p.obs_point.size() * sizeof(int));
        std::memcpy(px, p.obs_pixel.data(), p.obs_pixel.size() * sizeof(double));
        return 0;
    } catch (const std::exception&) {
        return 1;
    }
}

}  // extern "C"
