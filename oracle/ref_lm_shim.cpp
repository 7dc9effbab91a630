// Test infrastructure (oracle only): extern "C" entry to the reference's own
// LM driver, gba::solve_bal_gpu (reference include/gba/lm.hpp:34,
// src/lm.cu:371-724), compiled unmodified from the reference checkout by
// build_oracle.py and linked against ref_host_runtime.cpp (the CPU stand-in
// for the CUDA runtime). Parameters are updated in place, as the reference
// does.

#include <cstring>
#include <exception>
#include <string>

#include "gba/bal_problem.hpp"
#include "gba/lm.hpp"

extern "C" {

// termination: 0 CONVERGENCE, 1 MAX_ITERATIONS, 2 FAILURE, -1 other.
// Returns 0, or 1 if the solver threw (message in err, up to err_len bytes).
int gba_ref_solve_bal(int C, int P, int E, double* cams, double* pts, const int* oc, const int* op,
                      const double* px, int max_iterations, double initial_lambda, double rel_decrease_tol,
                      int max_inner_trials, int verbose, double* initial_cost, double* final_cost, int* iterations,
                      int* termination, unsigned long long* anomalies, double* total_time_s, char* err,
                      int err_len) {
    try {
        gba::BALProblem p;
        p.num_cameras = C;
        p.num_points = P;
        p.num_observations = E;
        p.cameras.assign(cams, cams + 9ll * C);
        p.points.assign(pts, pts + 3ll * P);
        p.obs_camera.assign(oc, oc + E);
        p.obs_point.assign(op, op + E);
        p.obs_pixel.assign(px, px + 2ll * E);
        gba::LMOptions o;
        o.max_iterations = max_iterations;
        o.initial_lambda = initial_lambda;
        o.rel_decrease_tol = rel_decrease_tol;
        o.max_inner_trials = max_inner_trials;
        o.verbose = verbose != 0;
        const gba::LMResult r = gba::solve_bal_gpu(p, o);
        std::memcpy(cams, p.cameras.data(), p.cameras.size() * sizeof(double));
        std::memcpy(pts, p.points.data(), p.points.size() * sizeof(double));
        *initial_cost = r.initial_cost;
        *final_cost = r.final_cost;
        *iterations = r.iterations;
        *termination = r.termination == "CONVERGENCE" ? 0
                       : r.termination == "MAX_ITERATIONS" ? 1
                       : r.termination == "FAILURE"        ? 2
                                                           : -1;
        *anomalies = r.anomalies;
        *total_time_s = r.total_time_s;
        return 0;
    } catch (const std::exception& e) {
        if (err && err_len > 0) {
            std::strncpy(err, e.what(), static_cast<size_t>(err_len - 1));
            err[err_len - 1] = '\0';
        }
        return 1;
    }
}

}  // extern "C"
