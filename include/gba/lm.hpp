#pragma once
// Drop-in public interface of the GB300 Levenberg-Marquardt solver.
//
// The reference declarations (include/gba/lm.hpp:13-42) are kept: LMOptions with
// the same five fields and defaults, LMResult with the same six fields, the same
// solve_bal_gpu and edge_residual_jacobian_host signatures. Everything after the
// "additive" markers is new, defaulted, and ignorable by reference callers.
//
// Parameters live in the caller's BALProblem (host, FP64) and are updated in place.

#include <string>
#include <vector>

#include "gba/bal_problem.hpp"

namespace gba {

// How the reduced camera system S dc = rhs is solved each trial.
enum class SolverForm {
    // All FP64: FP64 residuals/Jacobians, dense S assembled on the device and
    // factored by the blocked FP64 tensor-core (DMMA) Cholesky. The drop-in.
    Plain = 0,
    // FP32 residuals/Jacobians with FP64 accumulation; S never formed: FP32
    // implicit matvecs inside block-Jacobi PCG (FP32 vectors, FP64 scalars),
    // wrapped in iterative refinement to LMOptions::refine_tol. Where the
    // plain form is FP64 the cost evaluation (accept / reject), the
    // refinement residual, the right-hand side, the back-substitution and the
    // 3x3 point inverses V'^-1 run in float-float arithmetic (unevaluated sums
    // of two FP32 numbers, ~48-bit significands, on GB300's FP32 pipe) with
    // FP64 sums: the cost agrees with the FP64 cost
    // to ~1e-12 relative and a cost term whose residual leaves FP32's range is
    // recomputed in FP64 (tests/test_gpu_mixed.py). With refine_tol >= 1e-3
    // (inexact Newton steps) the right-hand side and back-substitution are FP32.
    Mixed = 1,
    // Mixed, with block-Jacobi corrected by the learned coarse space: a per-camera
    // MLP (weights from LMOptions::model_path) predicts the camera's rows of a
    // basis of the slow modes (the similarity gauge and soft modes), used in a
    // two-level PCG preconditioner; block-Jacobi judges it on the first inner
    // solve (iterations and S-norm step error) and is its fallback.
    MixedLearned = 2,
};

// Robust loss applied to each observation's squared residual s = |r|^2
// (the reference GPU solver has none; its Ceres baseline offers Huber,
// benchmarks/bench_ceres.cpp:120-142). Huber: rho(s) = s for s <= delta^2,
// 2 delta sqrt(s) - delta^2 above; the normal equations use the weights
// rho'(s) = min(1, delta / sqrt(s)).
enum class Loss { None = 0, Huber = 1 };

struct LMOptions {
    int max_iterations = 50;
    double initial_lambda = 1e-3;    // Marquardt diagonal damping
    double rel_decrease_tol = 1e-6;  // convergence: relative cost decrease
    int max_inner_trials = 16;       // lambda escalations per outer iteration
    bool verbose = false;            // per-trial log to stderr

    // ---- additive ----
    SolverForm form = SolverForm::Plain;
    double refine_tol = 1e-8;     // mixed: FP64 refinement stops at ||rhs - S dc|| <= tol ||rhs||
    int refine_max_steps = 12;    // mixed: FP64 refinement steps per trial (most take 2-4)
    double pcg_tol = 1e-4;        // mixed: relative residual target of each inner FP32 PCG solve
    int pcg_max_iters = 200;      // mixed: PCG iteration cap per inner solve
    std::string model_path;       // learned form: MLP weights file (gba_mlp binary)
    double target_cost = 0.0;     // if > 0: record the wall time at which cost first <= target
    bool stop_at_target = false;  // end the solve ("TARGET_COST") once cost <= target_cost
    Loss loss = Loss::None;       // robust loss; cost = sum rho(|r|^2) / 2
    double huber_delta = 1.0;     // Huber threshold (px)
    // plain form: storage of S (0 auto, 1 dense, 2 band of the cameras in reverse
    // Cuthill-McKee order; auto takes the band when it is at most a third of the
    // dense matrix)
    int schur_layout = 0;
    // mixed forms: 1 = the ordered two-pass FP32 PCG product (bit-identical
    // reruns); 0 = the one-pass product (atomic adds: reruns agree to rounding)
    int deterministic = 0;
};

struct LMResult {
    double initial_cost = 0.0;
    double final_cost = 0.0;
    int iterations = 0;               // accepted outer iterations
    std::string termination;          // "CONVERGENCE" | "MAX_ITERATIONS" | "FAILURE"
                                      // (+ "TARGET_COST" with LMOptions::stop_at_target)
    unsigned long long anomalies = 0; // cumulative non-finite edge / trial-residual count
    double total_time_s = 0.0;        // wall time of the solve, device setup included

    // ---- additive ----
    std::vector<double> trajectory;        // cost at start and after every accepted iteration
    std::vector<double> trajectory_time_s; // wall time (from solve start) of each trajectory entry
    int trials = 0;                        // inner trials evaluated (accepted + rejected)
    long long pcg_iterations = 0;          // mixed: total inner PCG iterations
    int refine_steps = 0;                  // mixed: total FP64 refinement steps
    // mixed: largest relative residual ||rhs - S dc|| / ||rhs|| of a refined
    // Schur step over the solve's trials (float-float residual of the system
    // the refinement solves), 0 for the plain form
    double max_refine_residual = 0.0;
    int schur_band_rows = 0;  // plain form: rows of the band S was stored in (0: dense)
    double time_to_target_s = -1.0;        // first time cost <= LMOptions::target_cost, or -1
    // Learned form: which preconditioner won the judged first inner solve
    // (1 = learned, 2 = block-Jacobi, 0 = not judged) and its inner PCG
    // iterations with block-Jacobi (stopped at 5/4 of the learned count, past
    // which it cannot win) and with the learned coarse correction.
    int learned_choice = 0;
    long long judge_iters_block_jacobi = 0, judge_iters_learned = 0;
    // Phase wall times (device-synchronised): setup, accumulate, damp+V^-1,
    // Schur solve (assembly+factor or PCG), back-substitution, trial cost.
    double t_setup = 0, t_accumulate = 0, t_damp = 0, t_schur = 0, t_backsub = 0, t_cost = 0;
};

// Runs LM on the current CUDA device. Modifies prob's cameras and points to the
// solution. Throws std::runtime_error on CUDA failure or invalid input
// (reference: include/gba/lm.hpp:34, src/lm.cu:371-724).
LMResult solve_bal_gpu(BALProblem& prob, const LMOptions& opts = {});

// Host entry point to the same residual + analytic Jacobian that the FP64 edge
// kernel evaluates (one __host__ __device__ template). Jc is 2x9 row-major
// (rodrigues[3], t[3], f, k1, k2), Jp is 2x3 row-major
// (reference: include/gba/lm.hpp:40-42, src/lm.cu:365-369).
void edge_residual_jacobian_host(const double* camera9, const double* point3,
                                 const double* observed2, double* out_residual2,
                                 double* out_Jc, double* out_Jp);

}  // namespace gba
