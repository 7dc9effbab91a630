/*
 * gba_capi.h — C ABI of the GB300 bundle-adjustment library (libgba_gb300.so).
 *
 * Plain C types only: pointers, sizes, an opaque solver handle and a
 * cudaStream_t passed as void*. Every function returns an int status
 * (GBA_OK = 0) and never throws; gba_last_error() returns the message of the
 * last failure on the calling thread.
 *
 * The reference exposes a C++ API only (include/gba/lm.hpp, bal_problem.hpp,
 * schur.cuh); each entry point below names the reference interface it stands in
 * for. Pointers marked [host] are host memory; [device] are device memory of
 * the current CUDA device.
 */
#ifndef GBA_CAPI_H
#define GBA_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    GBA_OK = 0,
    GBA_ERR_INVALID = 1,  /* bad argument / malformed input */
    GBA_ERR_CUDA = 2,     /* CUDA runtime failure */
    GBA_ERR_NOT_SPD = 3,  /* a factorisation met a non-positive pivot */
    GBA_ERR_IO = 4,       /* file read / write failure */
    GBA_ERR_INTERNAL = 5
};

enum { GBA_FORM_PLAIN = 0, GBA_FORM_MIXED = 1, GBA_FORM_MIXED_LEARNED = 2 };
enum { GBA_TERM_CONVERGENCE = 0, GBA_TERM_MAX_ITERATIONS = 1, GBA_TERM_FAILURE = 2, GBA_TERM_TARGET_COST = 3 };

const char* gba_last_error(void);
const char* gba_version(void);

/* ------------------------------------------------------------ whole solve */

/* Mirrors gba::LMOptions (reference include/gba/lm.hpp:13-19) plus the
 * additive fields of this library. Fill with gba_lm_options_default. */
typedef struct gba_lm_options {
    int max_iterations;       /* 50 */
    double initial_lambda;    /* 1e-3 */
    double rel_decrease_tol;  /* 1e-6 */
    int max_inner_trials;     /* 16 */
    int verbose;              /* 0 */
    int form;                 /* GBA_FORM_* (plain) */
    double refine_tol;        /* 1e-8 */
    int refine_max_steps;     /* 12 */
    double pcg_tol;           /* 1e-4 */
    int pcg_max_iters;        /* 200 */
    const char* model_path;   /* learned-form weights, or NULL */
    double target_cost;       /* 0 = off */
    int stop_at_target;       /* 0; 1 = end the solve once cost <= target_cost */
    int loss;                 /* GBA_LOSS_NONE (0) or GBA_LOSS_HUBER (1) */
    double huber_delta;       /* 1.0 */
    int schur_layout;         /* plain form: GBA_SCHUR_AUTO (0), GBA_SCHUR_DENSE (1) or GBA_SCHUR_BAND (2) */
    int deterministic;        /* mixed forms: 0 = one-pass PCG product; 1 = ordered two-pass product,
                                 bit-identical reruns (gba_solver_set_matvec) */
} gba_lm_options;

/* Storage of the plain form's reduced camera system S: dense (9C)^2, or a band
 * of the cameras reordered by reverse Cuthill-McKee on the camera graph (block
 * rows of S within the band, the factor keeps the band). AUTO takes the band
 * when it holds at most a third of the dense matrix (sparse covisibility, e.g.
 * sequential captures); random covisibility stays dense. */
enum { GBA_SCHUR_AUTO = 0, GBA_SCHUR_DENSE = 1, GBA_SCHUR_BAND = 2 };

enum { GBA_LOSS_NONE = 0, GBA_LOSS_HUBER = 1 };

/* Mirrors gba::LMResult (reference include/gba/lm.hpp:21-29) plus additive
 * fields. trajectory / trajectory_time_s may be NULL; otherwise they hold
 * trajectory_capacity doubles and receive min(len, capacity) entries. */
typedef struct gba_lm_result {
    double initial_cost;
    double final_cost;
    int iterations;
    int termination;                 /* GBA_TERM_* */
    unsigned long long anomalies;
    double total_time_s;
    int trials;
    long long pcg_iterations;
    int refine_steps;
    double time_to_target_s;
    double t_setup, t_accumulate, t_damp, t_schur, t_backsub, t_cost;
    double* trajectory;              /* [host] out */
    double* trajectory_time_s;       /* [host] out */
    int trajectory_capacity;
    int trajectory_len;
    int learned_choice;              /* learned form: 1 learned, 2 block-Jacobi won the judged solve */
    long long judge_iters_block_jacobi;  /* the judged solve's block-Jacobi iterations (stopped at 5/4 of the
                                            learned count, when it could no longer win) */
    long long judge_iters_learned;
    double max_refine_residual;      /* mixed forms: largest relative residual of a refined Schur step */
    int schur_band_rows;             /* plain form: rows of the band S was stored in, 0 if dense */
} gba_lm_result;

void gba_lm_options_default(gba_lm_options* opts);

/* LM solve of a BAL problem held in host arrays (BAL layout); cameras and
 * points are updated in place. Replaces gba::solve_bal_gpu
 * (reference include/gba/lm.hpp:34, src/lm.cu:371-724). [host] all arrays.
 * Sizes (also gba_solver_create): at least one camera, point and observation;
 * 9 C <= INT_MAX / 2, 6 P <= INT_MAX, 2 E <= INT_MAX; otherwise status 1
 * before any array is read. Observation indices out of range: status 1. */
int gba_solve_bal(int num_cameras, int num_points, int num_observations, double* cameras, double* points,
                  const int* obs_camera, const int* obs_point, const double* obs_pixel,
                  const gba_lm_options* opts, gba_lm_result* result);

/* ------------------------------------------------------------ CPU model / IO */

/* Replaces gba::edge_residual_jacobian_host (reference include/gba/lm.hpp:40-42).
 * [host] cam9, pt3, obs2 in; r2, Jc18 (2x9 row-major), Jp6 (2x3 row-major) out. */
int gba_edge_residual_jacobian_host(const double* camera9, const double* point3, const double* observed2,
                                    double* out_residual2, double* out_Jc, double* out_Jp);

/* Replaces gba::snavely_residual (reference include/gba/bal_problem.hpp:45-46). [host] */
int gba_snavely_residual(const double* camera9, const double* point3, const double* observed2, double* out2);

/* Replaces gba::total_squared_error (reference include/gba/bal_problem.hpp:50). [host] */
int gba_total_squared_error(int num_cameras, int num_points, int num_observations, const double* cameras,
                            const double* points, const int* obs_camera, const int* obs_point,
                            const double* obs_pixel, double* out_sse);

/* Host-side problem handle: holds a BALProblem produced by the reader or the
 * synthetic generator until its arrays are copied out. */
typedef struct gba_host_problem gba_host_problem;

/* Replaces gba::load_bal (reference include/gba/bal_problem.hpp:36). */
int gba_host_problem_load(const char* path, gba_host_problem** out);
/* Seeded synthetic workload 1..5 (no reference counterpart: stands in for the
 * BAL datasets). If truth is non-NULL it receives the unperturbed problem. */
int gba_host_problem_synthetic(int workload, uint64_t seed, gba_host_problem** out, gba_host_problem** truth);
/* Same generator with explicit sizes (no reference counterpart). */
int gba_host_problem_synthetic_custom(int num_cameras, int num_points, int track_min, int track_max,
                                      double track_alpha, double outlier_fraction, double outlier_sigma,
                                      uint64_t seed, gba_host_problem** out);
/* Same generator with spatially local covisibility (no reference counterpart):
 * camera centres along a path (x = 0.5 c), each point's track drawn from the
 * cameras within +-window of the camera nearest to it, so the camera graph is
 * a band, as in sequential captures. */
int gba_host_problem_synthetic_local(int num_cameras, int num_points, int track_min, int track_max,
                                     double track_alpha, int window, uint64_t seed, gba_host_problem** out);
/* The reference launch-bounds regression problem (tests/test_launch_bounds.cpp:28-80). */
int gba_host_problem_launch_bounds(int num_points, gba_host_problem** out);
int gba_host_problem_dims(const gba_host_problem* p, int* num_cameras, int* num_points, int* num_observations);
/* Copies the arrays out; any destination may be NULL. [host] */
int gba_host_problem_copy(const gba_host_problem* p, double* cameras, double* points, int* obs_camera,
                          int* obs_point, double* obs_pixel);
/* Writes a BAL text file (no reference counterpart in the library). */
int gba_host_problem_save(const gba_host_problem* p, const char* path);
void gba_host_problem_free(gba_host_problem* p);

/* ------------------------------------------------------------ device stages */

/* Device-resident LM state for one problem (parameters, sorted observation
 * slots, normal equations, Schur buffers). The stage functions below are the
 * steps of one LM trial; gba_solve_bal runs exactly these. They replace the
 * per-stage code of reference src/lm.cu:371-724. */
typedef struct gba_solver gba_solver;

/* [host] arrays. stream: a cudaStream_t or NULL (the solver then creates one). */
int gba_solver_create(int num_cameras, int num_points, int num_observations, const double* cameras,
                      const double* points, const int* obs_camera, const int* obs_point, const double* obs_pixel,
                      int form, void* stream, gba_solver** out);
void gba_solver_destroy(gba_solver* s);
int gba_solver_set_params(gba_solver* s, const double* cameras, const double* points);   /* [host] in */
int gba_solver_get_params(gba_solver* s, double* cameras, double* points);               /* [host] out */
/* Normal equations at the current parameters (reference edge_kernel +
 * accumulate, src/lm.cu:205-252, 399-422). out_sse: FP64 SSE. */
int gba_solver_accumulate(gba_solver* s, double* out_sse);
/* Damped point-block inverses (reference damp_invert_v_kernel, src/lm.cu:289-302).
 * out_nonspd: number of non-SPD blocks in this call. */
int gba_solver_damp_invert_v(gba_solver* s, double lambda, unsigned long long* out_nonspd);
/* Plain form: dense S assembly + FP64 DMMA Cholesky + solve (reference
 * src/lm.cu:488-604). out_info: 0, or the failed pivot column (1-based). */
int gba_solver_schur_dense(gba_solver* s, double lambda, int* out_info);
/* Mixed forms: the FP32 product S p inside PCG. 0 (default) and 2 = one pass
 * over the observations, adding each observation's Jc^T u into per-camera
 * accumulators with device atomics (its Jacobian rows read once from HBM; the
 * order of the atomic adds varies between runs, so results agree to FP32
 * rounding, not bit for bit); 1 = two passes (point pass, then camera pass
 * over a camera-major copy of the Jacobian rows; ordered sums, bit-identical
 * reruns); -1 = query only. The refinement residual, right-hand side and
 * back-substitution are the ordered two-pass products in every mode.
 * [host] out_one_pass (may be NULL): 1 if the one-pass product is in use. */
int gba_solver_set_matvec(gba_solver* s, int mode, int* out_one_pass);
/* Plain form: storage of S from the next gba_solver_schur_dense on
 * (GBA_SCHUR_AUTO / DENSE / BAND; gba_solve takes gba_lm_options.schur_layout). */
int gba_solver_set_schur_layout(gba_solver* s, int layout);
/* Plain form, after gba_solver_schur_dense: the band S is stored in (rows per
 * column ldb and tiles below the diagonal tile bt; 0 and 0 for dense S) and, for
 * a band, the camera order (perm[c] = position of camera c). [host] band_rows,
 * band_tiles (may be NULL), perm (C ints, may be NULL). */
int gba_solver_schur_band(gba_solver* s, int* band_rows, int* band_tiles, int* perm);
/* Mixed forms: PCG + FP64 refinement (no reference counterpart). Its last
 * refinement check of a float-float target runs the back-substitution's point
 * pass; gba_solver_back_substitute recomputes it (only the solver's own LM
 * loop reuses it). */
int gba_solver_schur_pcg(gba_solver* s, double lambda, const gba_lm_options* opts, int learned,
                         long long* out_pcg_iters, int* out_refine_steps, double* out_rel_residual);
/* Back-substitution, gain denominator, trial parameters (reference src/lm.cu:606-654). */
int gba_solver_back_substitute(gba_solver* s, double lambda, double* out_denom);
/* FP64 SSE at the trial parameters (reference cost_kernel, src/lm.cu:255-281). */
int gba_solver_trial_cost(gba_solver* s, double* out_sse);
int gba_solver_accept(gba_solver* s);
int gba_solver_counters(gba_solver* s, unsigned long long* out_anomalies, unsigned long long* out_nonspd);
/* Loads the learned-preconditioner weights for the MixedLearned form. */
int gba_solver_load_model(gba_solver* s, const char* path);
/* Robust loss used by the stage functions from now on (GBA_LOSS_*; Huber
 * threshold delta > 0). The Ceres baseline's --loss=huber (reference
 * benchmarks/bench_ceres.cpp:120-142); the reference GPU solver has none. */
int gba_solver_set_loss(gba_solver* s, int loss, double huber_delta);
/* Runs the full LM loop on the solver's device-resident problem from its
 * current parameters (the stages above, in the reference's order; no host
 * copies of the problem). Same contract as gba_solve_bal; parameters stay on
 * the device (gba_solver_get_params). opts->form must match the solver's form. */
int gba_solver_run(gba_solver* s, const gba_lm_options* opts, gba_lm_result* result);
/* Restores the parameters the solver was created with (device copy). */
int gba_solver_reset_params(gba_solver* s);
/* Per-kernel device timing with CUDA events on the solver stream: enable /
 * disable, query (launches and total milliseconds of a named kernel since the
 * last reset), reset. Names: point_pass_f64, camera_pass_f64, cost_f64,
 * schur_assemble, dense_potrf, backsub (plain form); point_pass_f32,
 * camera_pass_f32, cost_ff, schur_rhs_point_pass, schur_rhs_camera_pass,
 * schur_point_pass_f32, schur_camera_pass_f32, schur_point_pass_ff,
 * schur_camera_pass_ff, backsub (mixed forms); coarse_prepare (the learned
 * form's whole coarse-space set-up per trial), within it coarse_basis (the MLP
 * and the basis; mlp_forward within that), coarse_point_pass9,
 * coarse_camera_pass9, coarse_gram; coarse_apply (the correction inside PCG). */
int gba_solver_profile(gba_solver* s, int enable);
int gba_solver_kernel_stats(gba_solver* s, const char* name, long long* out_launches, double* out_total_ms);
int gba_solver_profile_reset(gba_solver* s);

/* Number of kernels this library has launched in the process so far. */
unsigned long long gba_launch_count(void);

/* Solvers allocate their device working set stream-ordered from the current
 * device's default memory pool, which keeps up to 32 GiB of freed memory for
 * the next solve (repeated solves then make no driver allocation calls). This
 * synchronises the device and returns that cached memory to the driver. No
 * reference counterpart (the reference allocates with cudaMalloc per call). */
int gba_release_cached_memory(void);

/* ------------------------------------------------------------ learned preconditioner
 * No reference counterpart (the reference has no iterative solver). The MLP
 * maps per-camera features (58, padded to 64 floats: the damped diagonal block
 * S_cc, track statistics, the camera's parameters) to the camera's 9 x 9 rows
 * of a coarse basis Z (81 outputs, padded to 96); the learned form's PCG adds
 * the coarse-space correction of block-Jacobi built from Z. Layouts in
 * gpu-bundle-adjustment_gb300/csrc/mlp.hpp. */

/* Plain form: also keep the damped diagonal blocks S_cc (GBA_BUF_SDIAG) at each
 * gba_solver_schur_dense (training-data harvest). */
int gba_solver_set_harvest(gba_solver* s, int enable);
/* Features of the current S_cc blocks and cameras at damping lambda. [device] feat (C x 64 float). */
int gba_solver_features(gba_solver* s, double lambda, float* feat);
/* Learned form: 0 = block-Jacobi judges the learned correction on the first
 * inner solve of each LM solve (default), 1 = always use it, 2 = never. */
int gba_solver_set_preconditioner(gba_solver* s, int mode);
/* Learned form, last judged solve: inner PCG iterations and b.x of the
 * block-Jacobi and the learned steps (the larger b.x has the smaller S-norm
 * error). The learned solve runs first; block-Jacobi's stops once it has used
 * 5/4 of the learned iterations (it cannot win past that). [host] iters (2),
 * btx (2). */
int gba_solver_judge_info(gba_solver* s, long long* iters, double* btx);

typedef struct gba_mlp gba_mlp;
long long gba_mlp_num_params(void);
/* New network (He-initialised hidden layers, small random output layer, zero biases). */
int gba_mlp_create(uint64_t seed, int batch_capacity, gba_mlp** out);
int gba_mlp_load(const char* path, int batch_capacity, gba_mlp** out);
int gba_mlp_save(const gba_mlp* m, const char* path);
void gba_mlp_destroy(gba_mlp* m);
/* FP32 master parameters / last gradients, flat (gba_mlp_num_params floats). [host] */
int gba_mlp_get_params(const gba_mlp* m, float* params);
int gba_mlp_set_params(gba_mlp* m, const float* params);
int gba_mlp_get_grads(const gba_mlp* m, float* grads);
/* out (B x 96) = network(feat (B x 64)); keeps the activations for gba_mlp_backward. [device] */
int gba_mlp_forward(gba_mlp* m, const float* feat, int batch, float* out, void* stream);
/* Parameter gradients of a loss from its gradient d_out (B x 96 float) w.r.t.
 * the outputs of the last gba_mlp_forward on the same feat. [device] */
int gba_mlp_backward(gba_mlp* m, const float* feat, const float* d_out, int batch, void* stream);
/* One Adam step with the gradients of the last gba_mlp_backward. */
int gba_mlp_adam_step(gba_mlp* m, float lr, float beta1, float beta2, float eps, void* stream);

enum {
    GBA_BUF_U = 0,        /* double[81 C]  full symmetric 9x9 per camera */
    GBA_BUF_V = 1,        /* double[6 P]   packed lower 3x3 per point (00,10,11,20,21,22) */
    GBA_BUF_BC = 2,       /* double[9 C] */
    GBA_BUF_BP = 3,       /* double[3 P] */
    GBA_BUF_W = 4,        /* double[27 E]  9x3 row-major per slot (plain form) */
    GBA_BUF_VINV = 5,     /* double[6 P]   packed */
    GBA_BUF_S = 6,        /* double[n_pad^2] column-major, or the band double[n_pad * ldb] (plain form;
                             factor after schur_dense) */
    GBA_BUF_RHS = 7,      /* double[n_pad] (plain) or [9 C] (mixed) */
    GBA_BUF_DC = 8,       /* double[9 C] */
    GBA_BUF_DP = 9,       /* double[3 P] */
    GBA_BUF_ORDER = 10,   /* int[E]  original observation index of each slot */
    GBA_BUF_JC32 = 11,    /* float[18 js] Jc per slot (mixed forms), js = E rounded up to a multiple of 32:
                             component planes, float4 plane q (q = 0..3) at [4 q js, 4 (q + 1) js) holding
                             entries 4q..4q+3 of the 2x9 row-major Jc of slot s at 4 s, then a float2 plane
                             at [16 js, 18 js) holding entries 16, 17 */
    GBA_BUF_SDIAG = 12,   /* double[81 C] S diagonal blocks (mixed form) */
    GBA_BUF_CAMS = 13,    /* double[9 C] current cameras */
    GBA_BUF_PTS = 14,     /* double[3 P] current points */
    GBA_BUF_TRIAL_CAMS = 15,
    GBA_BUF_TRIAL_PTS = 16,
    GBA_BUF_JP32 = 17     /* float[6 js] Jp per slot (mixed forms): a float4 plane at [0, 4 js) holding
                             entries 0..3 of the 2x3 row-major Jp of slot s at 4 s, then a float2 plane at
                             [4 js, 6 js) holding entries 4, 5 */
};
/* Size in bytes of a solver buffer (0 if the form does not hold it). */
int gba_solver_buffer_size(gba_solver* s, int buffer, size_t* out_bytes);
/* Copies a solver buffer to the host. [host] dst of at least buffer_size bytes. */
int gba_solver_download(gba_solver* s, int buffer, void* dst, size_t bytes);
/* Device address of a solver buffer (for zero-copy use by the caller). */
int gba_solver_device_ptr(gba_solver* s, int buffer, void** out_ptr);
int gba_solver_dims(gba_solver* s, int* num_cameras, int* num_points, int* num_observations, int* n_pad);

/* ------------------------------------------------------------ standalone kernels */

/* Batched 9x9 SPD factor + solve, one block per thread; ok[i] = 0 where
 * A_i is not SPD. Replaces gba::batch_chol9_factor_solve (reference
 * include/gba/schur.cuh:104-109). [device] A (n x 81 row-major, lower read),
 * b (n x 9), x (n x 9), ok (n). */
int gba_batch_chol9_factor_solve(const double* A, const double* b, double* x, int* ok, int n, void* stream);

/* Batched 3x3 SPD inverse. Replaces gba::batch_inverse3_spd (reference
 * include/gba/schur.cuh:112-116). [device] A (n x 9 row-major, lower read), Ainv (n x 9). */
int gba_batch_inverse3_spd(const double* A, double* Ainv, int* ok, int n, void* stream);

/* Blocked FP64 Cholesky (lower, column-major, DMMA trailing update), in place.
 * Replaces Eigen::LLT<MatrixXd, Lower> (reference src/lm.cu:598-603).
 * n multiple of 64, lda >= n. [device] A, info (int: 0 or failed column). */
int gba_dense_potrf(double* A, int n, int lda, int* info, void* stream);
/* Solves L L^T x = b in place after gba_dense_potrf (reference src/lm.cu:604). [device] */
int gba_dense_potrs(const double* L, int n, int lda, double* b, const int* info, void* stream);

/* The same Cholesky on a symmetric band matrix in band storage: per column the
 * ldb rows from the diagonal down, element (i, j), 0 <= i - j < ldb, at
 * AB[(i - j) + j * ldb]; nonzeros no more than bt 64-row tiles below each
 * diagonal 64 x 64 tile; ldb >= (bt + 2) * 64 (the last 64 rows of each column
 * are work space). No counterpart in the reference, whose dense LLT
 * (src/lm.cu:598-604) this replaces when the plain form's camera graph is a
 * band (GBA_SCHUR_BAND). n multiple of 64. [device] AB, info. */
int gba_band_potrf(double* AB, int n, int ldb, int bt, int* info, void* stream);
/* Solves L L^T x = b in place after gba_band_potrf. [device] */
int gba_band_potrs(const double* LB, int n, int ldb, int bt, double* b, const int* info, void* stream);

/* FP64 reprojection cost that allocates no device memory (no counterpart in the
 * reference). For callers that cannot let a library allocate: host frameworks
 * that own the device-memory budget through their own pool, or per-frame loops
 * that must not call cudaMalloc / cudaFree because those calls synchronise the
 * device. Computes the sum of squared Snavely residuals of num_observations
 * observations (the same FP64 function as the solver's trial-cost kernel) and
 * the number of non-finite residuals. [device] cameras (9C), points (3P),
 * obs_camera, obs_point (E), obs_pixel (2E) in; out_sse (1 double) and
 * out_nonfinite (1 unsigned long long, may be NULL) out.
 * Limit: num_observations <= 67,108,864 (GBA_ERR_INVALID above). Partial sums
 * go to a fixed 512 KiB file-scope device array that every device loading the
 * library holds until exit; all calls share it (each call writes every slot it
 * reads), so calls that overlap on the GPU race and must be serialised by the
 * caller. The first call on a device looks up that array's device address;
 * make that first call before any stream capture. The looked-up address is
 * kept for the life of the process: after cudaDeviceReset (or anything else
 * that destroys the device's primary context) it is stale, so do not call
 * this entry point again on that device after such a reset.
 * Precondition, not checked (the call takes no camera or point counts):
 * every obs_camera[i] lies in [0, C) and every obs_point[i] in [0, P) of the
 * caller's cameras / points arrays. */
int gba_cost_noalloc(const double* cameras, const double* points, const int* obs_camera, const int* obs_point,
                     const double* obs_pixel, int num_observations, double* out_sse,
                     unsigned long long* out_nonfinite, void* stream);

/* Residual + analytic Jacobian of E observations on the device, FP64 or FP32
 * (precision 64 / 32). [device] cams (9C), pts (3P), obs_camera, obs_point,
 * obs_pixel (2E) in; r (2E), Jc (18E, may be NULL), Jp (6E, may be NULL) out,
 * of type double (64) or float (32). Same function as the reference
 * edge_residual_jacobian (src/lm.cu:93-191). */
int gba_eval_edges(int precision, const double* cameras, const double* points, const int* obs_camera,
                   const int* obs_point, const double* obs_pixel, int num_observations, void* r, void* Jc,
                   void* Jp, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GBA_CAPI_H */
