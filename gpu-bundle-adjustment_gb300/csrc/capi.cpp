// extern "C" layer over the C++ library: status codes instead of exceptions.

#include "gba_capi.h"

#include <chrono>
#include <cstring>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>

#include "common.cuh"
#include "gba/bal_problem.hpp"
#include "gba/lm.hpp"
#include "lm_internal.hpp"
#include "mlp.hpp"
#include "noalloc.hpp"
#include "solver.hpp"
#include "synthetic.hpp"

struct gba_host_problem {
    gba::BALProblem p;
};

struct gba_solver {
    std::unique_ptr<gba::Solver> s;
    cudaStream_t own_stream = nullptr;
};

namespace {

thread_local std::string g_err;

template <typename F>
int guarded(F&& f) {
    try {
        f();
        return GBA_OK;
    } catch (const gba::CudaError& e) {
        g_err = e.what();
        return GBA_ERR_CUDA;
    } catch (const std::invalid_argument& e) {
        g_err = e.what();
        return GBA_ERR_INVALID;
    } catch (const std::bad_alloc& e) {
        g_err = "host allocation failed";
        return GBA_ERR_INTERNAL;
    } catch (const std::runtime_error& e) {
        g_err = e.what();
        return GBA_ERR_IO;
    } catch (const std::exception& e) {
        g_err = e.what();
        return GBA_ERR_INTERNAL;
    } catch (...) {
        g_err = "unknown exception";
        return GBA_ERR_INTERNAL;
    }
}

void need(bool ok, const char* what) {
    if (!ok) throw std::invalid_argument(what);
}

gba::LMOptions to_options(const gba_lm_options* o) {
    gba::LMOptions r;
    if (!o) return r;
    r.max_iterations = o->max_iterations;
    r.initial_lambda = o->initial_lambda;
    r.rel_decrease_tol = o->rel_decrease_tol;
    r.max_inner_trials = o->max_inner_trials;
    r.verbose = o->verbose != 0;
    need(o->form >= GBA_FORM_PLAIN && o->form <= GBA_FORM_MIXED_LEARNED, "bad solver form");
    r.form = static_cast<gba::SolverForm>(o->form);
    r.refine_tol = o->refine_tol;
    r.refine_max_steps = o->refine_max_steps;
    r.pcg_tol = o->pcg_tol;
    r.pcg_max_iters = o->pcg_max_iters;
    r.model_path = o->model_path ? o->model_path : "";
    r.target_cost = o->target_cost;
    r.stop_at_target = o->stop_at_target != 0;
    need(o->loss == GBA_LOSS_NONE || o->loss == GBA_LOSS_HUBER, "bad loss");
    r.loss = static_cast<gba::Loss>(o->loss);
    r.huber_delta = o->huber_delta;
    need(r.loss == gba::Loss::None || r.huber_delta > 0.0, "huber_delta must be positive");
    need(o->schur_layout >= GBA_SCHUR_AUTO && o->schur_layout <= GBA_SCHUR_BAND, "bad schur_layout");
    r.schur_layout = o->schur_layout;
    r.deterministic = o->deterministic != 0;
    return r;
}

void fill_result(const gba::LMResult& r, gba_lm_result* out) {
    out->initial_cost = r.initial_cost;
    out->final_cost = r.final_cost;
    out->iterations = r.iterations;
    out->termination = r.termination == "CONVERGENCE"   ? GBA_TERM_CONVERGENCE
                       : r.termination == "FAILURE"     ? GBA_TERM_FAILURE
                       : r.termination == "TARGET_COST" ? GBA_TERM_TARGET_COST
                                                        : GBA_TERM_MAX_ITERATIONS;
    out->anomalies = r.anomalies;
    out->total_time_s = r.total_time_s;
    out->trials = r.trials;
    out->pcg_iterations = r.pcg_iterations;
    out->refine_steps = r.refine_steps;
    out->time_to_target_s = r.time_to_target_s;
    out->t_setup = r.t_setup;
    out->t_accumulate = r.t_accumulate;
    out->t_damp = r.t_damp;
    out->t_schur = r.t_schur;
    out->t_backsub = r.t_backsub;
    out->t_cost = r.t_cost;
    out->learned_choice = r.learned_choice;
    out->judge_iters_block_jacobi = r.judge_iters_block_jacobi;
    out->judge_iters_learned = r.judge_iters_learned;
    out->max_refine_residual = r.max_refine_residual;
    out->schur_band_rows = r.schur_band_rows;
    out->trajectory_len = static_cast<int>(r.trajectory.size());
    const int n = std::min<int>(out->trajectory_len, std::max(0, out->trajectory_capacity));
    for (int i = 0; i < n; ++i) {
        if (out->trajectory) out->trajectory[i] = r.trajectory[i];
        if (out->trajectory_time_s) out->trajectory_time_s[i] = r.trajectory_time_s[i];
    }
}

gba::Solver& S(gba_solver* s) {
    need(s && s->s, "null solver");
    return *s->s;
}

}  // namespace

extern "C" {

const char* gba_last_error(void) { return g_err.c_str(); }
const char* gba_version(void) { return "gba-gb300 1.0 (sm_103a)"; }

void gba_lm_options_default(gba_lm_options* o) {
    if (!o) return;
    const gba::LMOptions d;
    o->max_iterations = d.max_iterations;
    o->initial_lambda = d.initial_lambda;
    o->rel_decrease_tol = d.rel_decrease_tol;
    o->max_inner_trials = d.max_inner_trials;
    o->verbose = d.verbose ? 1 : 0;
    o->form = GBA_FORM_PLAIN;
    o->refine_tol = d.refine_tol;
    o->refine_max_steps = d.refine_max_steps;
    o->pcg_tol = d.pcg_tol;
    o->pcg_max_iters = d.pcg_max_iters;
    o->model_path = nullptr;
    o->target_cost = d.target_cost;
    o->stop_at_target = 0;
    o->loss = GBA_LOSS_NONE;
    o->huber_delta = d.huber_delta;
    o->schur_layout = GBA_SCHUR_AUTO;
    o->deterministic = 0;
}

unsigned long long gba_launch_count(void) { return gba::launch_count(); }

int gba_release_cached_memory(void) {
    return guarded([&] { gba::release_cached_memory(); });
}

int gba_solver_set_harvest(gba_solver* s, int enable) {
    return guarded([&] {
        need(S(s).form() == gba::SolverForm::Plain, "harvest needs the plain form");
        S(s).harvest_ = enable != 0;
    });
}

int gba_solver_features(gba_solver* s, double lambda, float* feat) {
    return guarded([&] {
        need(feat != nullptr, "null features buffer");
        need(S(s).Sdiag_.get() != nullptr, "no diagonal blocks yet (run schur_pcg, or schur_dense with harvest)");
        gba::mlp_features(S(s), lambda, feat);
        S(s).sync();
    });
}

int gba_solver_set_preconditioner(gba_solver* s, int mode) {
    return guarded([&] {
        need(mode >= 0 && mode <= 2, "mode must be 0 (judge), 1 (learned) or 2 (block-Jacobi)");
        S(s).precond_force_ = mode;
    });
}

int gba_solver_judge_info(gba_solver* s, long long* iters, double* btx) {
    return guarded([&] {
        if (iters) {
            iters[0] = S(s).judge_iters_[0];
            iters[1] = S(s).judge_iters_[1];
        }
        if (btx) {
            btx[0] = S(s).judge_btx_[0];
            btx[1] = S(s).judge_btx_[1];
        }
    });
}

long long gba_mlp_num_params(void) { return gba::kMlpParams; }

int gba_mlp_create(uint64_t seed, int cap, gba_mlp** out) {
    return guarded([&] {
        need(out != nullptr && cap > 0, "bad argument");
        *out = reinterpret_cast<gba_mlp*>(new gba::Mlp(cap, seed));
    });
}

int gba_mlp_load(const char* path, int cap, gba_mlp** out) {
    return guarded([&] {
        need(path && out && cap > 0, "bad argument");
        *out = reinterpret_cast<gba_mlp*>(new gba::Mlp(std::string(path), cap));
    });
}

int gba_mlp_save(const gba_mlp* m, const char* path) {
    return guarded([&] {
        need(m && path, "null argument");
        reinterpret_cast<const gba::Mlp*>(m)->save(path);
    });
}

void gba_mlp_destroy(gba_mlp* m) { delete reinterpret_cast<gba::Mlp*>(m); }

int gba_mlp_get_params(const gba_mlp* m, float* p) {
    return guarded([&] {
        need(m && p, "null argument");
        reinterpret_cast<const gba::Mlp*>(m)->get_params(p);
    });
}

int gba_mlp_set_params(gba_mlp* m, const float* p) {
    return guarded([&] {
        need(m && p, "null argument");
        reinterpret_cast<gba::Mlp*>(m)->set_params(p);
    });
}

int gba_mlp_get_grads(const gba_mlp* m, float* g) {
    return guarded([&] {
        need(m && g, "null argument");
        reinterpret_cast<const gba::Mlp*>(m)->grads(g);
    });
}

int gba_mlp_forward(gba_mlp* m, const float* feat, int B, float* out, void* stream) {
    return guarded([&] {
        need(m && feat && out && B > 0, "bad argument");
        auto st = static_cast<cudaStream_t>(stream);
        reinterpret_cast<gba::Mlp*>(m)->forward(feat, B, out, st);
        GBA_CUDA_CHECK(cudaStreamSynchronize(st));
    });
}

int gba_mlp_backward(gba_mlp* m, const float* feat, const float* d_out, int B, void* stream) {
    return guarded([&] {
        need(m && feat && d_out && B > 0, "bad argument");
        auto st = static_cast<cudaStream_t>(stream);
        reinterpret_cast<gba::Mlp*>(m)->backward(feat, d_out, B, st);
        GBA_CUDA_CHECK(cudaStreamSynchronize(st));
    });
}

int gba_mlp_adam_step(gba_mlp* m, float lr, float b1, float b2, float eps, void* stream) {
    return guarded([&] {
        need(m != nullptr, "null model");
        auto st = static_cast<cudaStream_t>(stream);
        reinterpret_cast<gba::Mlp*>(m)->adam_step(lr, b1, b2, eps, st);
        GBA_CUDA_CHECK(cudaStreamSynchronize(st));
    });
}

int gba_solver_run(gba_solver* s, const gba_lm_options* opts, gba_lm_result* result) {
    return guarded([&] {
        need(result != nullptr, "null result");
        const gba::LMOptions o = to_options(opts);
        need(o.form == S(s).form(), "options form differs from the solver's form");
        if (o.form == gba::SolverForm::MixedLearned && !S(s).model()) S(s).load_model(o.model_path);
        const auto t0 = std::chrono::steady_clock::now();
        gba::LMResult r = gba::run_lm(S(s), o, t0);
        r.total_time_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        fill_result(r, result);
    });
}

int gba_solver_set_loss(gba_solver* s, int loss, double delta) {
    return guarded([&] {
        need(loss == GBA_LOSS_NONE || loss == GBA_LOSS_HUBER, "bad loss");
        need(loss == GBA_LOSS_NONE || delta > 0.0, "huber_delta must be positive");
        S(s).set_loss(static_cast<gba::Loss>(loss), delta);
    });
}

int gba_solver_reset_params(gba_solver* s) {
    return guarded([&] { S(s).reset_params(); });
}

int gba_solver_profile(gba_solver* s, int enable) {
    return guarded([&] { S(s).set_profiling(enable != 0); });
}

int gba_solver_kernel_stats(gba_solver* s, const char* name, long long* launches, double* ms) {
    return guarded([&] {
        need(name != nullptr, "null name");
        S(s).kernel_stats(name, launches, ms);
    });
}

int gba_solver_profile_reset(gba_solver* s) {
    return guarded([&] { S(s).prof_reset(); });
}

int gba_solve_bal(int C, int P, int E, double* cameras, double* points, const int* obs_camera,
                  const int* obs_point, const double* obs_pixel, const gba_lm_options* opts, gba_lm_result* result) {
    return guarded([&] {
        need(cameras && points && obs_camera && obs_point && obs_pixel && result, "null argument");
        gba::validate_problem(C, P, E, cameras, points, obs_camera, obs_point, obs_pixel);
        const gba::LMOptions o = to_options(opts);
        const auto t0 = std::chrono::steady_clock::now();
        cudaStream_t stream = nullptr;
        GBA_CUDA_CHECK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        struct Guard {
            cudaStream_t s;
            ~Guard() { cudaStreamDestroy(s); }
        } g{stream};
        gba::LMResult r;
        {
            gba::Solver s(C, P, E, cameras, points, obs_camera, obs_point, obs_pixel, o.form, stream);
            if (o.form == gba::SolverForm::MixedLearned) s.load_model(o.model_path);
            const double t_setup = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            r = gba::run_lm(s, o, t0);
            r.t_setup = t_setup;
            s.get_params(cameras, points);
        }
        r.total_time_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        fill_result(r, result);
    });
}

int gba_edge_residual_jacobian_host(const double* cam, const double* pt, const double* obs, double* r, double* Jc,
                                    double* Jp) {
    return guarded([&] {
        need(cam && pt && obs && r && Jc && Jp, "null argument");
        gba::edge_residual_jacobian_host(cam, pt, obs, r, Jc, Jp);
    });
}

int gba_snavely_residual(const double* cam, const double* pt, const double* obs, double* out2) {
    return guarded([&] {
        need(cam && pt && obs && out2, "null argument");
        gba::snavely_residual(cam, pt, obs, out2);
    });
}

int gba_total_squared_error(int C, int P, int E, const double* cams, const double* pts, const int* oc, const int* op,
                            const double* px, double* out) {
    return guarded([&] {
        need(cams && pts && oc && op && px && out, "null argument");
        need(C > 0 && P > 0 && E >= 0, "bad sizes");
        double sum = 0.0, r[2];
        for (int i = 0; i < E; ++i) {
            need(oc[i] >= 0 && oc[i] < C && op[i] >= 0 && op[i] < P, "observation index out of range");
            gba::snavely_residual(cams + 9ll * oc[i], pts + 3ll * op[i], px + 2ll * i, r);
            sum += r[0] * r[0] + r[1] * r[1];
        }
        *out = sum;
    });
}

int gba_host_problem_load(const char* path, gba_host_problem** out) {
    return guarded([&] {
        need(path && out, "null argument");
        auto h = std::make_unique<gba_host_problem>();
        h->p = gba::load_bal(path);
        *out = h.release();
    });
}

int gba_host_problem_synthetic(int workload, uint64_t seed, gba_host_problem** out, gba_host_problem** truth) {
    return guarded([&] {
        need(out != nullptr, "null argument");
        const gba::SyntheticConfig cfg = gba::synthetic_config(workload);
        auto h = std::make_unique<gba_host_problem>();
        std::unique_ptr<gba_host_problem> t;
        if (truth) t = std::make_unique<gba_host_problem>();
        h->p = gba::make_synthetic(cfg, seed, t ? &t->p : nullptr);
        *out = h.release();
        if (truth) *truth = t.release();
    });
}

int gba_host_problem_synthetic_custom(int C, int P, int kmin, int kmax, double alpha, double ofrac, double osig,
                                      uint64_t seed, gba_host_problem** out) {
    return guarded([&] {
        need(out != nullptr, "null argument");
        const gba::SyntheticConfig cfg{C, P, kmin, kmax, alpha, ofrac, osig};
        auto h = std::make_unique<gba_host_problem>();
        h->p = gba::make_synthetic(cfg, seed, nullptr);
        *out = h.release();
    });
}

int gba_host_problem_synthetic_local(int C, int P, int kmin, int kmax, double alpha, int window, uint64_t seed,
                                     gba_host_problem** out) {
    return guarded([&] {
        need(out != nullptr && window > 0, "bad argument (window must be positive)");
        gba::SyntheticConfig cfg{C, P, kmin, kmax, alpha, 0.0, 0.0};
        cfg.window = window;
        auto h = std::make_unique<gba_host_problem>();
        h->p = gba::make_synthetic(cfg, seed, nullptr);
        *out = h.release();
    });
}

int gba_host_problem_launch_bounds(int num_points, gba_host_problem** out) {
    return guarded([&] {
        need(out != nullptr && num_points > 0, "bad argument");
        auto h = std::make_unique<gba_host_problem>();
        h->p = gba::make_launch_bounds_problem(num_points);
        *out = h.release();
    });
}

int gba_host_problem_dims(const gba_host_problem* p, int* C, int* P, int* E) {
    return guarded([&] {
        need(p != nullptr, "null problem");
        if (C) *C = p->p.num_cameras;
        if (P) *P = p->p.num_points;
        if (E) *E = p->p.num_observations;
    });
}

int gba_host_problem_copy(const gba_host_problem* h, double* cams, double* pts, int* oc, int* op, double* px) {
    return guarded([&] {
        need(h != nullptr, "null problem");
        const auto& p = h->p;
        if (cams) std::memcpy(cams, p.cameras.data(), p.cameras.size() * sizeof(double));
        if (pts) std::memcpy(pts, p.points.data(), p.points.size() * sizeof(double));
        if (oc) std::memcpy(oc, p.obs_camera.data(), p.obs_camera.size() * sizeof(int));
        if (op) std::memcpy(op, p.obs_point.data(), p.obs_point.size() * sizeof(int));
        if (px) std::memcpy(px, p.obs_pixel.data(), p.obs_pixel.size() * sizeof(double));
    });
}

int gba_host_problem_save(const gba_host_problem* h, const char* path) {
    return guarded([&] {
        need(h && path, "null argument");
        gba::write_bal(path, h->p);
    });
}

void gba_host_problem_free(gba_host_problem* p) { delete p; }

int gba_solver_create(int C, int P, int E, const double* cams, const double* pts, const int* oc, const int* op,
                      const double* px, int form, void* stream, gba_solver** out) {
    return guarded([&] {
        need(out != nullptr, "null argument");
        need(form >= GBA_FORM_PLAIN && form <= GBA_FORM_MIXED_LEARNED, "bad solver form");
        gba::validate_problem(C, P, E, cams, pts, oc, op, px);
        auto h = std::make_unique<gba_solver>();
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        if (!st) {
            GBA_CUDA_CHECK(cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking));
            st = h->own_stream;
        }
        try {
            h->s = std::make_unique<gba::Solver>(C, P, E, cams, pts, oc, op, px, static_cast<gba::SolverForm>(form), st);
        } catch (...) {
            if (h->own_stream) cudaStreamDestroy(h->own_stream);
            throw;
        }
        *out = h.release();
    });
}

void gba_solver_destroy(gba_solver* s) {
    if (!s) return;
    s->s.reset();
    if (s->own_stream) cudaStreamDestroy(s->own_stream);
    delete s;
}

int gba_solver_set_params(gba_solver* s, const double* cams, const double* pts) {
    return guarded([&] {
        need(cams && pts, "null argument");
        S(s).set_params(cams, pts);
        S(s).sync();
    });
}

int gba_solver_get_params(gba_solver* s, double* cams, double* pts) {
    return guarded([&] { S(s).get_params(cams, pts); });
}

int gba_solver_accumulate(gba_solver* s, double* out_sse) {
    return guarded([&] {
        const double v = S(s).accumulate();
        if (out_sse) *out_sse = v;
    });
}

int gba_solver_damp_invert_v(gba_solver* s, double lambda, unsigned long long* out) {
    return guarded([&] {
        const unsigned long long v = S(s).damp_invert_v(lambda);
        if (out) *out = v;
    });
}

int gba_solver_schur_dense(gba_solver* s, double lambda, int* out_info) {
    return guarded([&] {
        need(S(s).form() == gba::SolverForm::Plain, "schur_dense needs the plain form");
        const int v = S(s).schur_dense(lambda);
        if (out_info) *out_info = v;
    });
}

int gba_solver_schur_pcg(gba_solver* s, double lambda, const gba_lm_options* opts, int learned, long long* iters,
                         int* steps, double* relres) {
    return guarded([&] {
        need(S(s).form() != gba::SolverForm::Plain, "schur_pcg needs a mixed form");
        const gba::LMOptions o = to_options(opts);
        const gba::PcgStats st = S(s).schur_pcg(lambda, o, learned != 0);
        if (iters) *iters = st.pcg_iterations;
        if (steps) *steps = st.refine_steps;
        if (relres) *relres = st.rel_residual;
    });
}

int gba_solver_back_substitute(gba_solver* s, double lambda, double* out_denom) {
    return guarded([&] {
        const double v = S(s).back_substitute(lambda);
        if (out_denom) *out_denom = v;
    });
}

int gba_solver_trial_cost(gba_solver* s, double* out_sse) {
    return guarded([&] {
        const double v = S(s).trial_cost();
        if (out_sse) *out_sse = v;
    });
}

int gba_solver_accept(gba_solver* s) {
    return guarded([&] { S(s).accept(); });
}

int gba_solver_counters(gba_solver* s, unsigned long long* a, unsigned long long* n) {
    return guarded([&] {
        if (a) *a = S(s).anomalies();
        if (n) *n = S(s).nonspd_total();
    });
}

int gba_solver_load_model(gba_solver* s, const char* path) {
    return guarded([&] {
        need(path != nullptr, "null path");
        S(s).load_model(path);
    });
}

int gba_solver_buffer_size(gba_solver* s, int buffer, size_t* out) {
    return guarded([&] {
        need(out != nullptr, "null argument");
        need(buffer >= GBA_BUF_U && buffer <= GBA_BUF_JP32, "bad buffer id");
        size_t bytes = 0;
        S(s).buffer(static_cast<gba::Solver::Buf>(buffer), &bytes);
        *out = bytes;
    });
}

int gba_solver_download(gba_solver* s, int buffer, void* dst, size_t bytes) {
    return guarded([&] {
        need(dst != nullptr, "null destination");
        need(buffer >= GBA_BUF_U && buffer <= GBA_BUF_JP32, "bad buffer id");
        size_t have = 0;
        const void* src = S(s).buffer(static_cast<gba::Solver::Buf>(buffer), &have);
        need(src != nullptr, "buffer not held by this solver form");
        need(bytes <= have, "download larger than the buffer");
        GBA_CUDA_CHECK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, S(s).stream()));
        S(s).sync();
    });
}

int gba_solver_device_ptr(gba_solver* s, int buffer, void** out) {
    return guarded([&] {
        need(out != nullptr, "null argument");
        need(buffer >= GBA_BUF_U && buffer <= GBA_BUF_JP32, "bad buffer id");
        size_t have = 0;
        *out = const_cast<void*>(S(s).buffer(static_cast<gba::Solver::Buf>(buffer), &have));
    });
}

int gba_solver_dims(gba_solver* s, int* C, int* P, int* E, int* n_pad) {
    return guarded([&] {
        if (C) *C = S(s).C();
        if (P) *P = S(s).P();
        if (E) *E = S(s).E();
        if (n_pad) *n_pad = S(s).n_pad();
    });
}

int gba_batch_chol9_factor_solve(const double* A, const double* b, double* x, int* ok, int n, void* stream) {
    return guarded([&] {
        need(n >= 0, "negative batch");
        need(n == 0 || (A && b && x && ok), "null argument");
        gba::launch_batch_chol9_factor_solve(A, b, x, ok, n, static_cast<cudaStream_t>(stream));
    });
}

int gba_batch_inverse3_spd(const double* A, double* Ainv, int* ok, int n, void* stream) {
    return guarded([&] {
        need(n >= 0, "negative batch");
        need(n == 0 || (A && Ainv && ok), "null argument");
        gba::launch_batch_inverse3_spd(A, Ainv, ok, n, static_cast<cudaStream_t>(stream));
    });
}

int gba_dense_potrf(double* A, int n, int lda, int* info, void* stream) {
    return guarded([&] {
        need(A && info, "null argument");
        need(n > 0 && n % 64 == 0 && lda >= n, "n must be a positive multiple of 64 and lda >= n");
        gba::dense_potrf(A, n, lda, n / 64 - 1, info, static_cast<cudaStream_t>(stream));
    });
}

int gba_dense_potrs(const double* L, int n, int lda, double* b, const int* info, void* stream) {
    return guarded([&] {
        need(L && b && info, "null argument");
        need(n > 0 && n % 64 == 0 && lda >= n, "n must be a positive multiple of 64 and lda >= n");
        gba::dense_potrs(L, n, lda, n / 64 - 1, b, info, static_cast<cudaStream_t>(stream));
    });
}

int gba_band_potrf(double* AB, int n, int ldb, int bt, int* info, void* stream) {
    return guarded([&] {
        need(AB && info, "null argument");
        need(n > 0 && n % 64 == 0, "n must be a positive multiple of 64");
        need(bt >= 0 && ldb >= (bt + 2) * 64, "ldb must be at least (bt + 2) * 64");
        gba::dense_potrf(AB, n, ldb - 1, bt, info, static_cast<cudaStream_t>(stream));
    });
}

int gba_band_potrs(const double* LB, int n, int ldb, int bt, double* b, const int* info, void* stream) {
    return guarded([&] {
        need(LB && b && info, "null argument");
        need(n > 0 && n % 64 == 0, "n must be a positive multiple of 64");
        need(bt >= 0 && ldb >= (bt + 2) * 64, "ldb must be at least (bt + 2) * 64");
        gba::dense_potrs(LB, n, ldb - 1, bt, b, info, static_cast<cudaStream_t>(stream));
    });
}

int gba_solver_set_matvec(gba_solver* s, int mode, int* out_one_pass) {
    return guarded([&] {
        need(S(s).form() != gba::SolverForm::Plain, "the PCG product belongs to the mixed forms");
        need(mode >= -1 && mode <= 2, "matvec mode: -1 query, 0 auto, 1 two-pass, 2 one-pass");
        if (mode >= 0) S(s).set_matvec(mode);
        if (out_one_pass) *out_one_pass = S(s).one_pass_;
    });
}

int gba_solver_set_schur_layout(gba_solver* s, int layout) {
    return guarded([&] {
        need(layout >= GBA_SCHUR_AUTO && layout <= GBA_SCHUR_BAND, "unknown Schur layout");
        need(S(s).form() == gba::SolverForm::Plain, "the Schur layout applies to the plain form");
        S(s).set_schur_layout(layout);
    });
}

int gba_solver_schur_band(gba_solver* s, int* band_rows, int* band_tiles, int* perm) {
    return guarded([&] {
        auto& so = S(s);
        if (band_rows) *band_rows = so.band_mode_ ? so.band_ldb_ : 0;
        if (band_tiles) *band_tiles = so.band_mode_ ? so.band_bt_ : 0;
        if (perm && so.band_mode_) {
            GBA_CUDA_CHECK(cudaMemcpy(perm, so.cam_perm_.get(), so.cam_perm_.size() * sizeof(int),
                                      cudaMemcpyDeviceToHost));
        }
    });
}

int gba_cost_noalloc(const double* cams, const double* pts, const int* oc, const int* op, const double* px, int E,
                     double* out_sse, unsigned long long* out_nonfinite, void* stream) {
    return guarded([&] {
        need(out_sse != nullptr, "null out_sse");
        need(E >= 0, "negative observation count");
        need(E == 0 || (cams && pts && oc && op && px), "null argument");
        gba::cost_noalloc(cams, pts, oc, op, px, E, out_sse, out_nonfinite, static_cast<cudaStream_t>(stream));
    });
}

int gba_eval_edges(int precision, const double* cams, const double* pts, const int* oc, const int* op,
                   const double* px, int E, void* r, void* Jc, void* Jp, void* stream) {
    return guarded([&] {
        need(precision == 64 || precision == 32, "precision must be 64 or 32");
        need(E >= 0, "negative count");
        if (E == 0) return;
        need(cams && pts && oc && op && px && r, "null argument");
        if (precision == 64)
            gba::launch_eval_edges_f64(cams, pts, oc, op, px, E, static_cast<double*>(r), static_cast<double*>(Jc),
                                       static_cast<double*>(Jp), static_cast<cudaStream_t>(stream));
        else
            gba::launch_eval_edges_f32(cams, pts, oc, op, px, E, static_cast<float*>(r), static_cast<float*>(Jc),
                                       static_cast<float*>(Jp), static_cast<cudaStream_t>(stream));
    });
}

}  // extern "C"
