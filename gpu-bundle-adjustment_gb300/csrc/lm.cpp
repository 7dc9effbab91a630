// Host LM driver: Marquardt damping with Nielsen accept/reject, every numeric
// stage on the device (Solver). Only scalars cross to the host per trial: the
// SSE, the non-SPD count, the factorisation status and the gain denominator.
//
// Algorithm contract (reference src/lm.cu:429-714, reproduced exactly):
//   cost = SSE / 2; lambda0 = opts.initial_lambda; nu reset to 2 every outer
//   iteration; per trial:
//     non-SPD damped V block            -> reject (lambda *= nu, nu *= 2)
//     Schur factorisation failure       -> reject
//     denom = sum delta (lambda d delta + b) <= 0 -> reject
//     anomaly counter moved / trial SSE not finite -> reject
//     rho = (sse - trial_sse) / (0.5 denom)     (2x the textbook ratio: both in SSE units)
//     accept iff rho > 0 && trial_sse < sse: lambda *= max(1/3, 1 - (2 rho - 1)^3)
//   all inner trials rejected -> FAILURE; after an accept, iterations++ and
//   CONVERGENCE if (sse - trial) / max(sse, 1) < rel_decrease_tol; else
//   re-accumulate; MAX_ITERATIONS when the loop ends.

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <memory>

#include "camera_model.cuh"
#include "common.cuh"
#include "lm_internal.hpp"
#include "solver.hpp"

namespace gba {

namespace {
using Clock = std::chrono::steady_clock;
double seconds_since(Clock::time_point t) { return std::chrono::duration<double>(Clock::now() - t).count(); }
}  // namespace

LMResult run_lm(Solver& s, const LMOptions& opts, Clock::time_point t0) {
    LMResult res;
    const bool plain = s.form() == SolverForm::Plain;
    const bool learned = s.form() == SolverForm::MixedLearned;
    auto phase = [&](double& acc, auto&& fn) {
        const auto ta = Clock::now();
        auto r = fn();
        acc += seconds_since(ta);
        return r;
    };

    s.begin_solve();
    s.set_loss(opts.loss, opts.huber_delta);
    if (plain)
        s.set_schur_layout(opts.schur_layout);
    else
        s.set_matvec(opts.deterministic ? 1 : 0);
    double sse = phase(res.t_accumulate, [&] { return s.accumulate(); });
    res.initial_cost = sse / 2.0;
    res.trajectory.push_back(res.initial_cost);
    res.trajectory_time_s.push_back(seconds_since(t0));
    if (opts.target_cost > 0.0 && res.initial_cost <= opts.target_cost) res.time_to_target_s = seconds_since(t0);

    double lambda = opts.initial_lambda;
    bool converged = false, failed = false, at_target = false;
    if (opts.stop_at_target && res.time_to_target_s >= 0.0) at_target = true;
    double rel_decrease = 0.0;
    unsigned long long anomalies = s.anomalies();

    while (res.iterations < opts.max_iterations && !converged && !failed && !at_target) {
        double nu = 2.0;
        bool accepted = false;
        for (int trial = 0; trial < opts.max_inner_trials; ++trial) {
            ++res.trials;
            if (!plain) {
                // Mixed forms: the same trial with three host reads (non-SPD
                // count with the right-hand side norm; the PCG checks; the
                // denominator, trial SSE and its non-finite count together).
                phase(res.t_damp, [&] { s.damp_launch(lambda); return 0; });
                unsigned long long bad = 0;
                const PcgStats st = phase(res.t_schur, [&] { return s.schur_pcg(lambda, opts, learned, &bad); });
                if (bad) {
                    s.add_nonspd(bad);
                    if (opts.verbose)
                        std::fprintf(stderr, "  iter %d trial: lambda %.3g non-SPD point blocks %llu: reject\n",
                                     res.iterations, lambda, bad);
                    lambda *= nu;
                    nu *= 2.0;
                    continue;
                }
                res.pcg_iterations += st.pcg_iterations;
                res.refine_steps += st.refine_steps;
                if (std::isfinite(st.rel_residual))
                    res.max_refine_residual = std::max(res.max_refine_residual, st.rel_residual);
                if (!std::isfinite(st.rel_residual)) {
                    lambda *= nu;
                    nu *= 2.0;
                    continue;
                }
                double denom = 0.0, trial_sse = 0.0;
                unsigned long long cost_anom = 0;
                phase(res.t_backsub, [&] { s.backsub_launch(lambda, true); return 0; });
                phase(res.t_cost, [&] {
                    s.zero_cost_scratch();
                    s.trial_cost_launch(s.counters_.get() + 2);
                    s.read_trial(&denom, &trial_sse, &cost_anom);
                    return 0;
                });
                if (!(denom > 0.0)) {  // rejected before its cost counts (the cost pass ran speculatively)
                    if (opts.verbose)
                        std::fprintf(stderr, "  iter %d trial: lambda %.3g denominator %.3g: reject\n",
                                     res.iterations, lambda, denom);
                    lambda *= nu;
                    nu *= 2.0;
                    continue;
                }
                if (cost_anom) {
                    s.commit_cost_anomalies();
                    anomalies += cost_anom;
                }
                if (cost_anom || !std::isfinite(trial_sse)) {
                    lambda *= nu;
                    nu *= 2.0;
                    continue;
                }
                const double rho = (sse - trial_sse) / (0.5 * denom);
                if (opts.verbose)
                    std::fprintf(stderr, "  iter %d trial: lambda %.3g cost %.9g rho %.3g %s\n", res.iterations,
                                 lambda, trial_sse / 2.0, rho, rho > 0.0 ? "accept" : "reject");
                if (rho > 0.0 && trial_sse < sse) {
                    s.accept();
                    rel_decrease = (sse - trial_sse) / std::max(sse, 1.0);
                    sse = trial_sse;
                    lambda *= std::max(1.0 / 3.0, 1.0 - std::pow(2.0 * rho - 1.0, 3.0));
                    accepted = true;
                    break;
                }
                lambda *= nu;
                nu *= 2.0;
                continue;
            }
            const unsigned long long before = anomalies;
            const unsigned long long bad = phase(res.t_damp, [&] { return s.damp_invert_v(lambda); });
            if (bad) {
                if (opts.verbose)
                    std::fprintf(stderr, "  iter %d trial: lambda %.3g non-SPD point blocks %llu: reject\n",
                                 res.iterations, lambda, bad);
                lambda *= nu;
                nu *= 2.0;
                continue;
            }
            if (plain) {
                const int info = phase(res.t_schur, [&] { return s.schur_dense(lambda); });
                if (info != 0) {
                    if (opts.verbose)
                        std::fprintf(stderr, "  iter %d trial: lambda %.3g Cholesky failed at column %d: reject\n",
                                     res.iterations, lambda, info);
                    lambda *= nu;
                    nu *= 2.0;
                    continue;
                }
            } else {
                const PcgStats st = phase(res.t_schur, [&] { return s.schur_pcg(lambda, opts, learned); });
                res.pcg_iterations += st.pcg_iterations;
                res.refine_steps += st.refine_steps;
                if (std::isfinite(st.rel_residual))
                    res.max_refine_residual = std::max(res.max_refine_residual, st.rel_residual);
                if (!std::isfinite(st.rel_residual)) {
                    lambda *= nu;
                    nu *= 2.0;
                    continue;
                }
            }
            const double denom = phase(res.t_backsub, [&] { return s.back_substitute(lambda); });
            if (!(denom > 0.0)) {
                if (opts.verbose)
                    std::fprintf(stderr, "  iter %d trial: lambda %.3g denominator %.3g: reject\n", res.iterations,
                                 lambda, denom);
                lambda *= nu;
                nu *= 2.0;
                continue;
            }
            const double trial_sse = phase(res.t_cost, [&] { return s.trial_cost(); });
            anomalies = s.anomalies();
            if (anomalies != before || !std::isfinite(trial_sse)) {
                lambda *= nu;
                nu *= 2.0;
                continue;
            }
            const double rho = (sse - trial_sse) / (0.5 * denom);
            if (opts.verbose)
                std::fprintf(stderr, "  iter %d trial: lambda %.3g cost %.9g rho %.3g %s\n", res.iterations, lambda,
                             trial_sse / 2.0, rho, rho > 0.0 ? "accept" : "reject");
            if (rho > 0.0 && trial_sse < sse) {
                s.accept();
                rel_decrease = (sse - trial_sse) / std::max(sse, 1.0);
                sse = trial_sse;
                lambda *= std::max(1.0 / 3.0, 1.0 - std::pow(2.0 * rho - 1.0, 3.0));
                accepted = true;
                break;
            }
            lambda *= nu;
            nu *= 2.0;
        }
        if (!accepted) {
            failed = true;
            break;
        }
        ++res.iterations;
        res.trajectory.push_back(sse / 2.0);
        res.trajectory_time_s.push_back(seconds_since(t0));
        if (opts.target_cost > 0.0 && res.time_to_target_s < 0.0 && sse / 2.0 <= opts.target_cost)
            res.time_to_target_s = seconds_since(t0);
        if (rel_decrease < opts.rel_decrease_tol) {
            converged = true;
            break;
        }
        if (opts.stop_at_target && res.time_to_target_s >= 0.0) {
            at_target = true;
            break;
        }
        // the new normal equations; the mixed forms already hold the SSE (the
        // accepted trial's), so nothing is read back here
        if (plain) {
            phase(res.t_accumulate, [&] { return s.accumulate(); });
        } else {
            phase(res.t_accumulate, [&] { s.accumulate_launch(); return 0; });
        }
    }

    res.final_cost = sse / 2.0;
    res.anomalies = s.anomalies();
    res.schur_band_rows = s.band_mode_ ? s.band_ldb_ : 0;
    res.learned_choice = s.learned_choice_;
    res.judge_iters_block_jacobi = s.judge_iters_[0];
    res.judge_iters_learned = s.judge_iters_[1];
    res.termination = converged ? "CONVERGENCE" : failed ? "FAILURE" : at_target ? "TARGET_COST" : "MAX_ITERATIONS";
    return res;
}

LMResult solve_bal_gpu(BALProblem& prob, const LMOptions& opts) {
    const auto t0 = Clock::now();
    if (prob.num_cameras <= 0 || prob.num_points <= 0 || prob.num_observations <= 0 ||
        prob.cameras.size() != 9ull * prob.num_cameras || prob.points.size() != 3ull * prob.num_points ||
        prob.obs_camera.size() != static_cast<size_t>(prob.num_observations) ||
        prob.obs_point.size() != static_cast<size_t>(prob.num_observations) ||
        prob.obs_pixel.size() != 2ull * prob.num_observations)
        throw std::invalid_argument("inconsistent BALProblem sizes");
    validate_problem(prob.num_cameras, prob.num_points, prob.num_observations, prob.cameras.data(),
                     prob.points.data(), prob.obs_camera.data(), prob.obs_point.data(), prob.obs_pixel.data());
    cudaStream_t stream = nullptr;
    GBA_CUDA_CHECK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } guard{stream};

    LMResult res;
    {
        Solver s(prob.num_cameras, prob.num_points, prob.num_observations, prob.cameras.data(), prob.points.data(),
                 prob.obs_camera.data(), prob.obs_point.data(), prob.obs_pixel.data(), opts.form, stream);
        if (opts.form == SolverForm::MixedLearned) s.load_model(opts.model_path);
        const double t_setup = seconds_since(t0);
        res = run_lm(s, opts, t0);
        res.t_setup = t_setup;
        s.get_params(prob.cameras.data(), prob.points.data());
    }
    res.total_time_s = seconds_since(t0);
    if (opts.verbose)
        std::fprintf(stderr,
                     "  phases: setup %.3fs, edge-accumulate %.3fs, damp+Vinv %.3fs, Schur solve %.3fs, "
                     "backsub %.3fs, trial cost %.3fs\n",
                     res.t_setup, res.t_accumulate, res.t_damp, res.t_schur, res.t_backsub, res.t_cost);
    return res;
}

void edge_residual_jacobian_host(const double* camera9, const double* point3, const double* observed2,
                                 double* out_residual2, double* out_Jc, double* out_Jp) {
    model::residual_jacobian(camera9, point3, observed2, out_residual2, out_Jc, out_Jp);
}

}  // namespace gba
