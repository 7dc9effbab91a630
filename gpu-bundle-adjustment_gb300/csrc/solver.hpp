#pragma once
// Device-resident LM state for one BAL problem and the stage functions the
// LM driver (lm.cpp) and the C-ABI (capi.cpp) call. Host-only header: the
// kernels live in structure.cu, edge.cu, blocks.cu, dense.cu, pcg.cu, mlp.cu.
//
// HBM layout (all device buffers owned by Solver, RAII):
//   parameters     cams[9C], pts[3P] (FP64, BAL layout) + trial copies
//   structure      observations stably sorted by point ("slots" s = 0..E-1):
//                  order[s] (original index), s_cam[s], s_pt[s], s_px[2s..2s+1],
//                  pt_off[P+1] (CSR), and a camera-major view cam_slots[] / cam_off[C+1]
//   work chunks    point chunks (whole points, <= 256 slots) for the point pass;
//                  camera chunks (<= kCamChunk slots of one camera) for the camera pass
//   normal eqs     U[81C] (full symmetric 9x9), bc[9C], V[6P] (packed lower 3x3),
//                  bp[3P], W[27 E] (FP64, slot order) or Jc32[18 E], Jp32[6 E] (FP32, slot order)
//   Schur (plain)  pair list sorted by camera-pair block, dense S (n_pad x n_pad,
//                  column-major, lower triangle), rhs, dc, dp
//   Schur (mixed)  PCG vectors (9C) and block-Jacobi factors (81C)

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <initializer_list>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "gba/lm.hpp"

namespace gba {

template <typename T>
class DevBuf {
public:
    DevBuf() = default;
    explicit DevBuf(size_t n) { alloc(n); }
    ~DevBuf() { release(); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p_(o.p_), n_(o.n_), s_(o.s_), async_(o.async_) { o.p_ = nullptr; o.n_ = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) {
            release();
            p_ = o.p_;
            n_ = o.n_;
            s_ = o.s_;
            async_ = o.async_;
            o.p_ = nullptr;
            o.n_ = 0;
        }
        return *this;
    }
    // Inside a StreamAllocScope: stream-ordered allocation on the scope's
    // stream from the device's memory pool; otherwise cudaMalloc. Defined in
    // structure.cu (throws CudaError).
    void alloc(size_t n);
    void release();
    T* get() const { return p_; }
    size_t size() const { return n_; }
    void swap(DevBuf& o) {
        std::swap(p_, o.p_);
        std::swap(n_, o.n_);
        std::swap(s_, o.s_);
        std::swap(async_, o.async_);
    }

private:
    T* p_ = nullptr;
    size_t n_ = 0;
    cudaStream_t s_ = nullptr;  // stream of a stream-ordered allocation (freed on it)
    bool async_ = false;
};

// While alive, DevBuf allocations on this thread are stream-ordered on stream s
// (cudaMallocAsync / cudaFreeAsync from the device's default memory pool),
// and the pool keeps up to kPoolKeepBytes of freed memory for the next solve
// instead of returning it to the driver: repeated solves then allocate and
// free their working set without driver calls. The stream must outlive the
// buffers allocated under the scope.
class StreamAllocScope {
public:
    static constexpr unsigned long long kPoolKeepBytes = 32ull << 30;
    explicit StreamAllocScope(cudaStream_t s);
    ~StreamAllocScope();
    StreamAllocScope(const StreamAllocScope&) = delete;
    StreamAllocScope& operator=(const StreamAllocScope&) = delete;

private:
    cudaStream_t prev_s_;
    bool prev_on_;
};

// Returns the memory the current device's pool keeps between solves to the driver.
void release_cached_memory();

struct PcgStats {
    int refine_steps = 0;
    long long pcg_iterations = 0;
    double rel_residual = 0.0;  // final ||rhs - S dc|| / ||rhs|| (FP64)
    bool converged = false;
    int fallbacks = 0;          // learned form: inner solves redone with plain block-Jacobi
};

struct PhaseTimes {
    double setup = 0, accumulate = 0, damp = 0, schur = 0, backsub = 0, cost = 0;
};

class LearnedPreconditioner;  // mlp.cu

class Solver {
public:
    // Copies the problem to the device and builds the slot structure. Host arrays
    // in the BAL layout; observation indices are bounds-checked on the host.
    Solver(int C, int P, int E, const double* cams, const double* pts, const int* obs_cam,
           const int* obs_pt, const double* obs_px, SolverForm form, cudaStream_t stream);
    ~Solver();

    int C() const { return C_; }
    int P() const { return P_; }
    int E() const { return E_; }
    int n_pad() const { return n_pad_; }
    SolverForm form() const { return form_; }
    cudaStream_t stream() const { return stream_; }

    void set_params(const double* cams, const double* pts);
    void get_params(double* cams, double* pts) const;

    // Normal equations at the current parameters: FP64 (plain) or FP32
    // Jacobians with FP64 accumulation (mixed). Returns the SSE; adds non-finite
    // edges to the anomaly counter.
    double accumulate();
    void accumulate_launch();  // the same passes, SSE left in scal_[0] (no host read)
    // V' = V + lambda * max(diag V, 1e-12), inverted per point. Returns the number
    // of non-SPD blocks found by this call.
    unsigned long long damp_invert_v(double lambda);
    // Plain form: assemble dense S and rhs, Cholesky-factor, solve for dc.
    // Returns 0 on success, else the (1-based) failed pivot column.
    int schur_dense(double lambda);
    // Mixed form: solve S dc = rhs by FP32 PCG inside FP64 iterative refinement.
    PcgStats schur_pcg(double lambda, const LMOptions& opts, bool learned);
    // The LM driver's fused trial (mixed forms): the stages above, launched
    // without their own host reads. damp_launch leaves the non-SPD count on the
    // device; schur_pcg with nonspd_out reads it together with the right-hand
    // side norm (and stops there if it is non-zero); backsub_launch and
    // trial_cost_launch (non-finite count to counters_[2]) are followed by one
    // read_trial() of the denominator, the SSE and that count.
    void damp_launch(double lambda);
    PcgStats schur_pcg(double lambda, const LMOptions& opts, bool learned, unsigned long long* nonspd_out);
    // reuse: the LM driver's trial, where schur_pcg's last refinement check may
    // already have run the point pass at this dc and lambda (backsub_ready_).
    void backsub_launch(double lambda, bool reuse = false);
    // Where the point pass writes its denominator partials (after the camera ones).
    double* backsub_part();
    bool backsub_ready_ = false;
    void trial_cost_launch(unsigned long long* anomalies);
    void read_trial(double* denom, double* sse, unsigned long long* cost_anomalies);
    void add_nonspd(unsigned long long n);     // adds to the cumulative non-SPD count
    void commit_cost_anomalies();              // counters_[0] += counters_[2] (device side)
    void zero_cost_scratch();                  // counters_[2] = 0 (device side)
    // dp = V'^-1 (bp - sum_e W_e^T dc), the gain denominator, and the trial
    // parameters (current + step). Returns the denominator (SSE units).
    double back_substitute(double lambda);
    // SSE at the trial parameters (FP64; float-float in the mixed forms); adds
    // non-finite residuals to the anomaly counter.
    double trial_cost();
    // Mixed forms: float-float cost pass at (cams, pts); SSE partials per point
    // chunk in sse_part_, FP32 residuals in r_out, non-finite count to anomalies.
    void cost_mixed(const double* cams, const double* pts, unsigned long long* anomalies, float2* r_out);
    // Mixed forms: float-float camera constants and points plus FP32 cameras of
    // (cams, pts) into cam_pre_ff_, pts_ff_, cams32_; ff_holds_ says whose.
    void prepare_ff(const double* cams, const double* pts);
    enum FfHolds { kFfNone, kFfCurrent, kFfTrial };
    FfHolds ff_holds_ = kFfNone;
    // pts_ff_ holds the split of tpts_, written by the mixed back-substitution
    // (the trial cost then skips the point split).
    bool pts_ff_trial_ = false;
    // Trial parameters become current.
    void accept();

    unsigned long long anomalies() const;     // cumulative counter[0]
    unsigned long long nonspd_total() const;  // cumulative counter[1]

    // Learned preconditioner (MixedLearned form).
    void load_model(const std::string& path);
    LearnedPreconditioner* model() { return model_; }

    // Raw views for the C-ABI download/inspection entry points.
    enum Buf { kU, kV, kBc, kBp, kW, kVinv, kS, kRhs, kDc, kDp, kOrder, kJc32, kSdiag, kCams, kPts,
               kTrialCams, kTrialPts, kJp32 };
    const void* buffer(Buf b, size_t* bytes) const;

    // Optional per-kernel device timing (CUDA events on the solver stream
    // around selected launches). prof_start returns null when profiling is off.
    void set_profiling(bool on);
    cudaEvent_t prof_start();
    void prof_stop(const char* name, cudaEvent_t start);
    // Launch count and total device milliseconds of the named kernel since the
    // last reset (synchronises the stream).
    void kernel_stats(const std::string& name, long long* launches, double* total_ms);
    void prof_reset();
    // Restores the parameters given at construction (device-to-device copy).
    void reset_params();

    // ---- internal state (public for the kernel translation units) ----
    int C_, P_, E_, n_pad_ = 0;
    SolverForm form_;
    cudaStream_t stream_;
    mutable cudaEvent_t sync_ev_ = nullptr;  // sync(): the event the host polls (created on first use)
    LearnedPreconditioner* model_ = nullptr;

    DevBuf<double> cams_, pts_, tcams_, tpts_, cams0_, pts0_;
    bool profiling_ = false;
    struct Timed {
        std::string name;
        cudaEvent_t a, b;
    };
    std::vector<Timed> timed_;
    // structure
    DevBuf<int> order_, pt_off_, s_cam_, s_pt_, cam_off_, cam_slots_;
    DevBuf<double> s_px_;
    int n_pchunk_ = 0, n_cchunk_ = 0;
    DevBuf<int> pchunk_, cchunk_begin_, cchunk_cam_, cam_chunk_off_;
    DevBuf<int> pchunk4_;  // per point chunk, int4 {first point, end point, first slot, end slot}
    // normal equations
    DevBuf<double> U_, bc_, V_, bp_, W_, JcR_, Vinv_;
    DevBuf<float> Jc32_, Jp32_;  // mixed: FP32 Jacobian rows, slot order, component-major (stride js_)
    long long js_ = 0;
    DevBuf<float> J32c_;    // mixed: camera record [Jc(18), r(2)] per slot in camera-major position
    DevBuf<float> Vinv32_;  // mixed: FP32 copy of V'^-1 (6 per point) for the FP32 matvec
    DevBuf<float> Vinv32lo_;  // mixed: V'^-1 - Vinv32_ rounded to FP32 (float-float matvec)
    DevBuf<float> dcff_;      // mixed: float-float copy of dc (hi, lo per entry) for the refinement residual
    DevBuf<float> pcg_p32_; // mixed: FP32 copy of the PCG direction for the FP32 matvec
    DevBuf<int> cam_pos_;   // camera-major position of each slot (inverse of cam_slots_)
    // mixed: the one-pass FP32 PCG product (pcg.cu): the point pass adds each
    // slot's Jc^T u into an accumulator of its camera (y_acc_, 12 floats each)
    // instead of leaving u for a camera pass; else the two-pass product. A
    // camera has one accumulator per kAccSlots of its observations (its
    // camera-major positions), so that no FP32 accumulator sums more terms
    // than a camera-pass thread and warp do (with 256 terms the refinement to
    // 1e-8 on workload 3 ran out of steps): camera c's at [acc_off_[c],
    // acc_off_[c + 1]), the slot's in acc_id_.
    static constexpr int kAccSlots = 32;
    bool one_pass_ = false;
    int n_acc_ = 0;
    // the warp-level point passes' work: warp chunks (whole points, at most
    // 32 slots: int2 {first, end slot}); points with 33 to 256 observations in
    // lists of at most 256 slots per CTA (lchunk_: int2 {first entry of lpts_,
    // entries}); longer points as ranges (int4 {p, p + 1, first slot, end
    // slot}) for the chunked point passes
    int n_wchunk_ = 0, n_lchunk_ = 0, n_huge_ = 0;
    DevBuf<int> wchunk_, lchunk_, lpts_, huge_range_;
    void build_point_groups();  // pcg.cu
    DevBuf<int> acc_id_, acc_off_;
    DevBuf<float> y_acc_;
    void set_matvec(int mode);  // 0 auto (one pass), 1 two-pass (deterministic), 2 one-pass
    DevBuf<double> cam_pre_;  // per-camera rotation matrix, translation, intrinsics (16 per camera)
    DevBuf<float> cam_pre_ff_;  // mixed: the same as float-float pairs (32 floats per camera)
    DevBuf<float> pts_ff_;      // mixed: float-float copy of the points being costed (6 floats per point)
    DevBuf<float> cm_pxff_;     // mixed: observations as float-float pairs (4 floats) at camera-major positions
    DevBuf<int> cm_pt_;         // mixed: point of each camera-major position
    DevBuf<float> cams32_;      // mixed: per-camera R, J_l, t, f, k1, k2, branch flag (28 floats) for the FP32 Jacobians
    DevBuf<float> r_cur_, r_trial_;  // mixed: float-float evaluated residuals (FP32, camera-major) at current / trial parameters
    bool resid_valid_ = false;       // r_cur_ and scal_[0] hold the current parameters' residuals / SSE
    DevBuf<double> sse_part_, cam_part_, scal_;  // scal_: [0] sse, [1] trial sse, [2] denom, [3..] scratch
    DevBuf<unsigned long long> counters_;        // [0] anomalies, [1] non-SPD V blocks
    // plain Schur
    long long n_pairs_ = 0;
    int n_blocks_ = 0;
    DevBuf<int> pair_e_, pair_f_, block_off_, block_ce_, block_cf_;
    DevBuf<double> T_, S_, rhs_, dc_, dp_, red_part_;
    DevBuf<int> info_;
    // mixed Schur
    DevBuf<double> Sdiag_, Pfac_;  // S diagonal blocks (81C), preconditioner factors (packed, 45 per camera)
    DevBuf<float> Pinv_;           // explicit preconditioner blocks M_c = (L L^T)^-1 (81C, FP32)
    DevBuf<double> pcg_x_;         // plain form: the dense solve's work vector
    DevBuf<double> ref_r_;         // mixed forms: the refinement residual, the inner solve's right-hand side
    // mixed forms: the inner PCG's FP32 vectors (9 per camera; its direction is
    // pcg_p32_), the learned step kept while block-Jacobi is judged, and the
    // damped camera blocks U_lambda in FP32 (81 per camera)
    DevBuf<float> pcg_e_, pcg_r_, pcg_z_, pcg_q_, judge_e_, ul32_;
    DevBuf<double> u_;       // per-slot 2-vectors u_e = Jp_e w_p (matvec intermediate; FP32 or float-float)
    DevBuf<float> g_cm_;     // per-slot G_e = Jp V'^-1 Jp^T (00, 01, 11, pad) at camera-major positions
    DevBuf<double> pcg_s_;   // PCG device scalars (see pcg.cu)
    DevBuf<float> mlp_stats_;  // learned form: per-camera track statistics (3 per camera)
    // learned form: coarse basis Z (kCoarse columns of 9C), S Z, E^-1 (+ SPD flag),
    // and the partial sums of the balancing preconditioner and of E
    DevBuf<double> cz_, csz_, ceinv_, cred_, cpart9_;
    DevBuf<float> cz32_, csz32_;  // Z and S Z in FP32 (the PCG's coarse correction)
    DevBuf<__nv_bfloat16> czb_;  // BF16 per-camera basis rows (the basis is used at BF16 precision)
    DevBuf<float> cu9_;          // per-slot u of the product S Z (18 floats in a 20-float record)
    void coarse_prepare(double lambda);  // pcg.cu
    // Learned form, per solve: 0 = not judged yet, 1 = the learned coarse
    // correction won the first inner solve, 2 = block-Jacobi won (used for the
    // rest of the solve).
    int learned_choice_ = 0;
    int precond_force_ = 0;              // learned form: 0 judge, 1 always learned, 2 always block-Jacobi
    long long judge_iters_[2] = {0, 0};  // inner PCG iterations of the judged solve: block-Jacobi, learned
    double judge_btx_[2] = {0, 0};       // b . x of the judged solve's two steps (larger: smaller S-norm error)
    int judge_attempts_ = 0;             // judgements made in this solve
    bool fast_solve_ = false;            // the last Schur solve ran the loose-target FP32 path
    int prev_inner_ = 0;                 // iterations of the last inner PCG solve (launch-batch predictor)
    void begin_solve() {
        learned_choice_ = 0;
        judge_attempts_ = 0;
        prev_inner_ = 0;
    }
    // Robust loss of the cost and the normal equations (<= 0: none). Changing it
    // invalidates the cached residuals / SSE of the current parameters.
    double huber_delta_ = 0.0;
    void set_loss(Loss loss, double delta) {
        const double d = loss == Loss::Huber ? delta : 0.0;
        if (d != huber_delta_) resid_valid_ = false;
        huber_delta_ = d;
    }
    bool harvest_ = false;     // plain form: keep the damped diagonal blocks S_cc in Sdiag_
    // plain form: storage of S. The camera graph (the nonzero 9x9 blocks) is
    // ordered by reverse Cuthill-McKee at set-up (cam_perm_: camera -> position);
    // in band mode S holds, per column, the band_ldb_ rows from the diagonal
    // down (element (i, j) at S_[i + j (band_ldb_ - 1)]), band_bt_ = 64-row
    // tiles below the diagonal tile that the band reaches.
    int schur_layout_ = 0;     // 0 auto, 1 dense, 2 band
    int schur_layout_planned_ = -1;  // the layout S_ was allocated for
    bool band_mode_ = false;
    bool band_beneficial_ = false;
    int band_ldb_ = 0, band_bt_ = 0;
    DevBuf<int> cam_perm_;
    void set_schur_layout(int layout) { schur_layout_ = layout; }
    void plan_schur_band();       // structure.cu: ordering and band size from the block list
    void ensure_schur_storage();  // dense.cu: allocates S for the chosen layout

    void build_structure(const int* obs_cam, const int* obs_pt, const double* obs_px, const double* cams,
                         const double* pts);
    void build_pairs();
    void sync() const;
    // Device -> host readback of a few scalars: each (dst, src, bytes) is
    // queued as an asynchronous copy into a pinned staging buffer, one sync()
    // completes them all, then they are copied to dst (host memory, pageable
    // is fine). At most 4 KiB in total.
    struct HostRead {
        void* dst;
        const void* src;
        size_t bytes;
    };
    void read_back(std::initializer_list<HostRead> reads) const;
};

// Host-side checks of a BAL problem (sizes, null arrays, index ranges); throws
// std::invalid_argument. Runs before any device work.
void validate_problem(int C, int P, int E, const double* cams, const double* pts, const int* obs_cam,
                      const int* obs_pt, const double* obs_px);

// Standalone kernels with raw device pointers (C-ABI entry points wrap these).
// Float-float split of n FP64 values into (hi, lo) float pairs (pcg.cu).
void launch_split_ff(const double* x, long long n, float* out, cudaStream_t s);

// Mixed-form back-substitution (pcg.cu): dp, trial points and the point terms
// of the gain denominator (one partial per point chunk in part).
void mixed_back_substitute(Solver& s, double lambda, double* part, bool with_u = false);

void launch_batch_chol9_factor_solve(const double* A, const double* b, double* x, int* ok, int n,
                                     cudaStream_t s);
void launch_batch_inverse3_spd(const double* A, double* Ainv, int* ok, int n, cudaStream_t s);
// Blocked Cholesky (lower, column-major), element (i, j) at A[i + j lda]. n
// must be a multiple of 64. Dense: bt = n / 64 - 1, lda >= n. Band of bt
// 64-row tiles below the diagonal tile: lda = ldb - 1, ldb >= (bt + 2) 64 rows
// kept per column from the diagonal down. info (device int) = 0 on success,
// else the 1-based failed column.
void dense_potrf(double* A, int n, int lda, int bt, int* info, cudaStream_t s);

// Solves L L^T x = b in place (b on the device, length n), L from dense_potrf.
void dense_potrs(const double* L, int n, int lda, int bt, double* b, const int* info, cudaStream_t s);
// Residual + Jacobian for E independent observations (device pointers, original
// layout). Jc, Jp may be null. FP64 or FP32 arithmetic.
void launch_eval_edges_f64(const double* cams, const double* pts, const int* oc, const int* op,
                           const double* px, int E, double* r, double* Jc, double* Jp,
                           cudaStream_t s);
void launch_eval_edges_f32(const double* cams, const double* pts, const int* oc, const int* op,
                           const double* px, int E, float* r, float* Jc, float* Jp,
                           cudaStream_t s);

}  // namespace gba
