// bench_bal — command-line LM solve of a BAL problem on the GPU.
//
// Same flags, gates, exit codes and JSON keys (in the same order) as the
// reference CLI (benchmarks/bench_bal.cpp:4-134):
//   bench_bal <problem.txt[.bz2]> [--iterations=N] [--lambda=D] [--json=PATH] [--verbose]
//   exit 1 = arguments / IO, 2 = solver initial cost differs from the reader's
//   cost by more than 1e-9 max(1, |c|), 3 = device anomaly counter non-zero.
// Additive flags: --synthetic=W (workload 1..5 instead of a file),
// --custom=C,P,KMIN,KMAX,ALPHA[,WINDOW] (the seeded generator at other sizes:
// cameras, points, track lengths KMIN..KMAX with P(k) ~ k^-ALPHA, and with
// WINDOW > 0 tracks within +-WINDOW cameras along a path), --seed=S,
// --form=plain|mixed|learned, --model=PATH, --target-cost=D, --refine-tol=D and
// --pcg-tol=D (mixed forms' Schur solve targets), and the loss flags
// of the reference's Ceres benchmark (benchmarks/bench_ceres.cpp:10-11,117-131):
// --loss=none|huber, --delta=D (default 1.0); with Huber the initial-cost gate
// compares against sum rho(|r|^2) / 2 from the reader's own residual. Additive
// JSON keys after the reference's: form, trials, pcg_iterations,
// time_to_target_s, trajectory.

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>

#include "gba/bal_problem.hpp"
#include "gba/lm.hpp"
#include "synthetic.hpp"

namespace {

struct Args {
    std::string file;
    int iterations = 50;
    double lambda = 1e-3;
    std::string json;
    bool verbose = false;
    int synthetic = 0;
    std::string custom;
    unsigned long long seed = 0;
    bool seed_set = false;
    std::string form = "plain";
    std::string model;
    double target_cost = 0.0;
    std::string loss = "none";
    double delta = 1.0;
    double refine_tol = -1.0, pcg_tol = -1.0;  // < 0: library defaults
};

[[noreturn]] void usage_error(const std::string& msg) {
    std::fprintf(stderr, "%s\nusage: bench_bal <problem.txt[.bz2]> [--iterations=N] [--lambda=D] [--json=PATH] "
                         "[--verbose] [--synthetic=1..5 | --custom=C,P,KMIN,KMAX,ALPHA[,WINDOW]] [--seed=S] "
                         "[--form=plain|mixed|learned] [--model=PATH] "
                         "[--target-cost=D] [--loss=none|huber] [--delta=D] [--refine-tol=D] [--pcg-tol=D]\n",
                 msg.c_str());
    std::exit(1);
}

Args parse(int argc, char** argv) {
    Args a;
    for (int i = 1; i < argc; ++i) {
        const std::string s = argv[i];
        auto val = [&](const char* key) -> const char* {
            const size_t n = std::strlen(key);
            return s.compare(0, n, key) == 0 ? argv[i] + n : nullptr;
        };
        try {
            if (s == "--verbose") a.verbose = true;
            else if (const char* v = val("--iterations=")) a.iterations = std::stoi(v);
            else if (const char* v = val("--lambda=")) a.lambda = std::stod(v);
            else if (const char* v = val("--json=")) a.json = v;
            else if (const char* v = val("--synthetic=")) a.synthetic = std::stoi(v);
            else if (const char* v = val("--custom=")) a.custom = v;
            else if (const char* v = val("--seed=")) { a.seed = std::stoull(v); a.seed_set = true; }
            else if (const char* v = val("--form=")) a.form = v;
            else if (const char* v = val("--model=")) a.model = v;
            else if (const char* v = val("--target-cost=")) a.target_cost = std::stod(v);
            else if (const char* v = val("--loss=")) a.loss = v;
            else if (const char* v = val("--delta=")) a.delta = std::stod(v);
            else if (const char* v = val("--refine-tol=")) a.refine_tol = std::stod(v);
            else if (const char* v = val("--pcg-tol=")) a.pcg_tol = std::stod(v);
            else if (s.rfind("--", 0) != 0 && a.file.empty()) a.file = s;
            else usage_error("bad argument: " + s);
        } catch (const std::logic_error&) {
            usage_error("bad value: " + s);
        }
    }
    if ((a.file.empty() ? 0 : 1) + (a.synthetic ? 1 : 0) + (a.custom.empty() ? 0 : 1) != 1)
        usage_error("give exactly one of a problem file, --synthetic=W or --custom=...");
    if (a.loss != "none" && a.loss != "huber") usage_error("unknown loss: " + a.loss);
    if (a.loss == "huber" && !(a.delta > 0.0)) usage_error("--delta must be positive");
    return a;
}

}  // namespace

int main(int argc, char** argv) {
    const Args args = parse(argc, argv);
    gba::BALProblem bal;
    std::string name = args.file;
    try {
        if (args.synthetic) {
            const unsigned long long seed = args.seed_set ? args.seed : static_cast<unsigned long long>(args.synthetic);
            bal = gba::make_synthetic(gba::synthetic_config(args.synthetic), seed);
            name = "synthetic:" + std::to_string(args.synthetic) + ":seed" + std::to_string(seed);
        } else if (!args.custom.empty()) {
            gba::SyntheticConfig cfg{};
            int window = 0;
            const int n = std::sscanf(args.custom.c_str(), "%d,%d,%d,%d,%lf,%d", &cfg.num_cameras, &cfg.num_points,
                                      &cfg.track_min, &cfg.track_max, &cfg.track_alpha, &window);
            if (n < 5 || cfg.num_cameras <= 0 || cfg.num_points <= 0 || cfg.track_min < 1 ||
                cfg.track_max < cfg.track_min)
                usage_error("bad --custom: " + args.custom);
            cfg.window = window;
            const unsigned long long seed = args.seed_set ? args.seed : 1ull;
            bal = gba::make_synthetic(cfg, seed);
            name = "custom:" + args.custom + ":seed" + std::to_string(seed);
        } else {
            bal = gba::load_bal(args.file);
        }
    } catch (const std::exception& e) {
        std::fprintf(stderr, "cannot load problem: %s\n", e.what());
        return 1;
    }
    std::fprintf(stderr, "loaded %s: %d cameras, %d points, %d observations\n", name.c_str(), bal.num_cameras,
                 bal.num_points, bal.num_observations);
    double own_cost = gba::total_squared_error(bal) / 2.0;
    if (args.loss == "huber") {
        own_cost = 0.0;
        const double d2 = args.delta * args.delta;
        for (int i = 0; i < bal.num_observations; ++i) {
            double r[2];
            gba::snavely_residual(bal.camera(bal.obs_camera[i]), bal.point(bal.obs_point[i]), &bal.obs_pixel[2 * i],
                                  r);
            const double s = r[0] * r[0] + r[1] * r[1];
            own_cost += 0.5 * (s <= d2 ? s : 2.0 * args.delta * std::sqrt(s) - d2);
        }
    }

    cudaDeviceProp prop{};
    int dev = 0;
    cudaGetDevice(&dev);
    cudaGetDeviceProperties(&prop, dev);

    gba::LMOptions opts;
    opts.max_iterations = args.iterations;
    opts.initial_lambda = args.lambda;
    opts.verbose = args.verbose;
    opts.model_path = args.model;
    opts.target_cost = args.target_cost;
    opts.loss = args.loss == "huber" ? gba::Loss::Huber : gba::Loss::None;
    opts.huber_delta = args.delta;
    if (args.refine_tol > 0.0) opts.refine_tol = args.refine_tol;
    if (args.pcg_tol > 0.0) opts.pcg_tol = args.pcg_tol;
    if (args.form == "plain") opts.form = gba::SolverForm::Plain;
    else if (args.form == "mixed") opts.form = gba::SolverForm::Mixed;
    else if (args.form == "learned") opts.form = gba::SolverForm::MixedLearned;
    else usage_error("bad --form: " + args.form);

    gba::LMResult res;
    try {
        res = gba::solve_bal_gpu(bal, opts);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "solver failed: %s\n", e.what());
        return 1;
    }
    if (std::fabs(res.initial_cost - own_cost) > 1e-9 * std::max(1.0, std::fabs(own_cost))) {
        std::fprintf(stderr,
                     "MISMATCH: reader cost %.17g vs solver initial cost %.17g\n"
                     "camera model is broken; benchmark results void\n",
                     own_cost, res.initial_cost);
        return 2;
    }
    if (res.anomalies != 0) {
        std::fprintf(stderr, "device anomaly counter is %llu — refusing to report\n", res.anomalies);
        return 3;
    }
    const double per_iter = res.iterations > 0 ? res.total_time_s / res.iterations : 0.0;
    std::string traj = "[";
    for (size_t i = 0; i < res.trajectory.size(); ++i) {
        char b[40];
        std::snprintf(b, sizeof b, "%s%.17g", i ? ", " : "", res.trajectory[i]);
        traj += b;
    }
    traj += "]";
    const std::string form_name = args.form;
    std::string json;
    {
        char head[2048];
        std::snprintf(head, sizeof head,
                      "{\n"
                      "  \"file\": \"%s\",\n"
                      "  \"solver\": \"gba-gb300-lm\",\n"
                      "  \"loss\": \"%s\",\n"
                      "  \"num_cameras\": %d,\n"
                      "  \"num_points\": %d,\n"
                      "  \"num_observations\": %d,\n"
                      "  \"initial_cost\": %.17g,\n"
                      "  \"final_cost\": %.17g,\n"
                      "  \"iterations\": %d,\n"
                      "  \"total_time_s\": %.6f,\n"
                      "  \"per_iteration_s\": %.6f,\n"
                      "  \"termination\": \"%s\",\n"
                      "  \"device\": \"%s\",\n"
                      "  \"form\": \"%s\",\n"
                      "  \"trials\": %d,\n"
                      "  \"pcg_iterations\": %lld,\n"
                      "  \"time_to_target_s\": %.6f,\n"
                      "  \"trajectory\": ",
                      name.c_str(), args.loss.c_str(), bal.num_cameras, bal.num_points, bal.num_observations, res.initial_cost,
                      res.final_cost, res.iterations, res.total_time_s, per_iter, res.termination.c_str(), prop.name,
                      form_name.c_str(), res.trials, res.pcg_iterations, res.time_to_target_s);
        json = head + traj + "\n}";
    }
    std::printf("%s\n", json.c_str());
    if (!args.json.empty()) {
        FILE* fp = std::fopen(args.json.c_str(), "w");
        if (!fp) {
            std::fprintf(stderr, "cannot write %s\n", args.json.c_str());
            return 1;
        }
        std::fprintf(fp, "%s\n", json.c_str());
        std::fclose(fp);
    }
    return 0;
}
