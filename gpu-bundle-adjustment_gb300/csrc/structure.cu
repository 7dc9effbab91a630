// Problem upload and slot structure: observations stably sorted by point
// (CSR over points), a camera-major view of the same slots, the work chunks of
// the point and camera passes, and (plain form) the list of edge pairs that
// feed each camera-pair block of the reduced camera system.
//
// The reference keeps observations in file order and builds a host adjacency
// list point -> edges (src/lm.cu:380-381); there is no sorted layout there. This
// layout is what lets every reduction in this library run without atomics.

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_run_length_encode.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <atomic>
#include <climits>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "solver.hpp"

namespace gba {

namespace {
thread_local cudaStream_t t_alloc_stream = nullptr;
thread_local bool t_alloc_async = false;

cudaMemPool_t device_pool() {
    int dev = 0;
    GBA_CUDA_CHECK(cudaGetDevice(&dev));
    cudaMemPool_t pool;
    GBA_CUDA_CHECK(cudaDeviceGetDefaultMemPool(&pool, dev));
    return pool;
}
}  // namespace

StreamAllocScope::StreamAllocScope(cudaStream_t s) : prev_s_(t_alloc_stream), prev_on_(t_alloc_async) {
    unsigned long long keep = kPoolKeepBytes;  // the attribute is a 64-bit unsigned value
    GBA_CUDA_CHECK(cudaMemPoolSetAttribute(device_pool(), cudaMemPoolAttrReleaseThreshold, &keep));
    t_alloc_stream = s;
    t_alloc_async = true;
}

StreamAllocScope::~StreamAllocScope() {
    t_alloc_stream = prev_s_;
    t_alloc_async = prev_on_;
}

void release_cached_memory() {
    GBA_CUDA_CHECK(cudaDeviceSynchronize());
    GBA_CUDA_CHECK(cudaMemPoolTrimTo(device_pool(), 0));
}

template <typename T>
void DevBuf<T>::alloc(size_t n) {
    release();
    if (n == 0) return;
    if (t_alloc_async) {
        GBA_CUDA_CHECK(cudaMallocAsync(reinterpret_cast<void**>(&p_), n * sizeof(T), t_alloc_stream));
        s_ = t_alloc_stream;
        async_ = true;
    } else {
        GBA_CUDA_CHECK(cudaMalloc(reinterpret_cast<void**>(&p_), n * sizeof(T)));
        async_ = false;
    }
    n_ = n;
}
template <typename T>
void DevBuf<T>::release() {
    if (p_) {
        if (async_) {
            cudaFreeAsync(p_, s_);
        } else {
            cudaFree(p_);
        }
    }
    p_ = nullptr;
    n_ = 0;
}
template class DevBuf<double>;
template class DevBuf<float>;
template class DevBuf<int>;
template class DevBuf<unsigned long long>;
template class DevBuf<unsigned int>;
template class DevBuf<unsigned char>;
template class DevBuf<long long>;
template class DevBuf<__nv_bfloat16>;

namespace {
std::atomic<unsigned long long> g_launches{0};
}
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
unsigned long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

int device_sm_count() {
    static int cached = 0;
    if (!cached) {
        int dev = 0;
        GBA_CUDA_CHECK(cudaGetDevice(&dev));
        GBA_CUDA_CHECK(cudaDeviceGetAttribute(&cached, cudaDevAttrMultiProcessorCount, dev));
    }
    return cached;
}

namespace {

constexpr int kPointChunk = 256;   // max slots (and max points) per point-pass CTA
constexpr int kCamChunk = 1024;    // max slots per camera-pass CTA

__global__ void iota_kernel(int* v, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = i;
}

__global__ void gather_obs_kernel(const int* __restrict__ order, const int* __restrict__ oc,
                                  const double* __restrict__ px, int E, int* __restrict__ s_cam,
                                  double2* __restrict__ s_px) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < E; s += gridDim.x * blockDim.x) {
        const int e = order[s];
        s_cam[s] = oc[e];
        s_px[s] = make_double2(px[2ll * e], px[2ll * e + 1]);
    }
}

// pos[perm[i]] = i
__global__ void inverse_perm_kernel(const int* __restrict__ perm, int n, int* __restrict__ pos) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) pos[perm[i]] = i;
}

// Count of observations whose camera or point index is out of range.
__global__ void check_indices_kernel(const int* __restrict__ oc, const int* __restrict__ op, int n, int C, int P,
                                     unsigned long long* __restrict__ bad) {
    unsigned long long cnt = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        cnt += (oc[i] < 0 || oc[i] >= C || op[i] < 0 || op[i] >= P) ? 1ull : 0ull;
    cnt = __reduce_add_sync(0xffffffffu, static_cast<unsigned>(cnt));
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(bad, cnt);
}

// Greedy point chunk from point p: points p .. q-1 with q the largest index in
// [p + 1, min(P, p + kPointChunk)] whose slots fit in kPointChunk (p + 1 when
// point p alone has more). next[P] = P.
__global__ void chunk_next_kernel(const int* __restrict__ pt_off, int P, int* __restrict__ next) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p <= P; p += gridDim.x * blockDim.x) {
        if (p == P) {
            next[p] = P;
            continue;
        }
        const int base = pt_off[p];
        int lo = p + 1, hi = min(P, p + kPointChunk);  // lo always qualifies as the answer's floor
        while (lo < hi) {
            const int mid = lo + (hi - lo + 1) / 2;
            if (pt_off[mid] - base <= kPointChunk) {
                lo = mid;
            } else {
                hi = mid - 1;
            }
        }
        next[p] = lo;
    }
}

// One binary-lifting level: out[p] = in[in[p]].
__global__ void lift_kernel(const int* __restrict__ in, int P, int* __restrict__ out) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p <= P; p += gridDim.x * blockDim.x) out[p] = in[in[p]];
}

// Number of greedy chunks: lifted walk from point 0 while short of P.
__global__ void chunk_count_kernel(const int* __restrict__ jump, int levels, int P, int* __restrict__ n) {
    int cur = 0, cnt = 0;
    for (int k = levels - 1; k >= 0; --k) {
        const int nx = jump[static_cast<size_t>(k) * (P + 1ull) + cur];
        if (nx < P) {
            cur = nx;
            cnt += 1 << k;
        }
    }
    *n = cnt + 1;
}

// starts[i] = next^i(0) for i < n, starts[n] = P.
__global__ void chunk_starts_kernel(const int* __restrict__ jump, int levels, int P, int n,
                                    int* __restrict__ starts) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += gridDim.x * blockDim.x) {
        if (i == n) {
            starts[i] = P;
            continue;
        }
        int cur = 0;
        for (int k = 0; k < levels; ++k)
            if ((i >> k) & 1) cur = jump[static_cast<size_t>(k) * (P + 1ull) + cur];
        starts[i] = cur;
    }
}

// Per point chunk {p0, p1, s0, s1}: the point-side passes read their ranges
// with one 16-byte load instead of two dependent loads (chunk table, CSR).
__global__ void chunk_ranges_kernel(const int* __restrict__ pchunk, const int* __restrict__ pt_off, int n,
                                    int4* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int p0 = pchunk[i], p1 = pchunk[i + 1];
        out[i] = make_int4(p0, p1, pt_off[p0], pt_off[p1]);
    }
}

// Camera-major copies of per-slot data: point index and observation (as
// float-float pairs) of camera-major position i (slot cam_slots[i]).
__global__ void gather_cm_kernel(const int* __restrict__ cam_slots, const int* __restrict__ s_pt,
                                 const double2* __restrict__ s_px, int n, int* __restrict__ cm_pt,
                                 float4* __restrict__ cm_pxff) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int s = cam_slots[i];
        cm_pt[i] = s_pt[s];
        const double2 o = s_px[s];
        const float hx = __double2float_rn(o.x), hy = __double2float_rn(o.y);
        cm_pxff[i] = make_float4(hx, __double2float_rn(o.x - static_cast<double>(hx)), hy,
                                 __double2float_rn(o.y - static_cast<double>(hy)));
    }
}

// acc_id[s] = acc_off[cam(s)] + (camera-major position of s - cam_off[cam(s)]) / per
__global__ void acc_id_kernel(const int* __restrict__ s_cam, const int* __restrict__ cam_pos,
                              const int* __restrict__ cam_off, const int* __restrict__ acc_off, int E, int per,
                              int* __restrict__ acc_id) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < E; s += gridDim.x * blockDim.x) {
        const int c = s_cam[s];
        acc_id[s] = acc_off[c] + (cam_pos[s] - cam_off[c]) / per;
    }
}

// offsets[k] = first position i with keys[i] >= k, for k = 0..nk (keys sorted).
__global__ void csr_offsets_kernel(const int* __restrict__ keys, int n, int nk, int* __restrict__ off) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int prev = i == 0 ? -1 : keys[i - 1];
        const int cur = keys[i];
        for (int k = prev + 1; k <= cur; ++k) off[k] = i;
        if (i == n - 1)
            for (int k = cur + 1; k <= nk; ++k) off[k] = n;
    }
}

// Number of ordered slot pairs (e, f) of point p with cam(e) >= cam(f).
__global__ void pair_count_kernel(const int* __restrict__ pt_off, const int* __restrict__ s_cam, int P,
                                  long long* __restrict__ cnt) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
        const int b = pt_off[p], e = pt_off[p + 1];
        long long n = 0;
        for (int i = b; i < e; ++i) {
            const int ci = s_cam[i];
            for (int j = b; j < e; ++j) n += (s_cam[j] <= ci);
        }
        cnt[p] = n;
    }
}

__global__ void pair_fill_kernel(const int* __restrict__ pt_off, const int* __restrict__ s_cam, int P,
                                 int C, const long long* __restrict__ base,
                                 unsigned long long* __restrict__ key, unsigned long long* __restrict__ val) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
        const int b = pt_off[p], e = pt_off[p + 1];
        long long o = base[p];
        for (int i = b; i < e; ++i) {
            const int ci = s_cam[i];
            for (int j = b; j < e; ++j) {
                const int cj = s_cam[j];
                if (cj <= ci) {
                    key[o] = static_cast<unsigned long long>(ci) * static_cast<unsigned long long>(C) + cj;
                    val[o] = (static_cast<unsigned long long>(static_cast<unsigned>(i)) << 32) |
                             static_cast<unsigned>(j);
                    ++o;
                }
            }
        }
    }
}

__global__ void pair_split_kernel(const unsigned long long* __restrict__ val, long long n, int* __restrict__ pe,
                                  int* __restrict__ pf) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long v = val[i];
        pe[i] = static_cast<int>(v >> 32);
        pf[i] = static_cast<int>(v & 0xffffffffu);
    }
}

__global__ void block_split_kernel(const unsigned long long* __restrict__ ukey, int nb, int C,
                                   int* __restrict__ ce, int* __restrict__ cf) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += gridDim.x * blockDim.x) {
        const unsigned long long k = ukey[i];
        ce[i] = static_cast<int>(k / static_cast<unsigned long long>(C));
        cf[i] = static_cast<int>(k % static_cast<unsigned long long>(C));
    }
}

int bits_for(long long n) {
    int b = 1;
    while ((1LL << b) < n) ++b;
    return b;
}

int grid_for(long long n, int threads = 256) {
    const long long want = (n + threads - 1) / threads;
    const long long cap = 32LL * device_sm_count();
    return static_cast<int>(std::max<long long>(1, std::min(want, cap)));
}

}  // namespace

// Host-side checks (sizes, pointers); the observation indices are checked on
// the device when the solver is built (build_structure).
void validate_problem(int C, int P, int E, const double* cams, const double* pts, const int* obs_cam,
                      const int* obs_pt, const double* obs_px) {
    if (C <= 0 || P <= 0 || E <= 0) throw std::invalid_argument("empty BAL problem");
    if (!cams || !pts || !obs_cam || !obs_pt || !obs_px) throw std::invalid_argument("null problem array");
    if (static_cast<long long>(C) * 9 > INT_MAX / 2) throw std::invalid_argument("too many cameras");
    // 32-bit per-point and per-observation index arithmetic stays in range
    // (both limits lie beyond what one GPU's memory holds)
    if (static_cast<long long>(P) * 6 > INT_MAX) throw std::invalid_argument("too many points");
    if (static_cast<long long>(E) * 2 > INT_MAX) throw std::invalid_argument("too many observations");
}

Solver::Solver(int C, int P, int E, const double* cams, const double* pts, const int* obs_cam,
               const int* obs_pt, const double* obs_px, SolverForm form, cudaStream_t stream)
    : C_(C), P_(P), E_(E), form_(form), stream_(stream) {
    validate_problem(C, P, E, cams, pts, obs_cam, obs_pt, obs_px);
    StreamAllocScope alloc_scope(stream_);

    cams_.alloc(9ull * C);
    pts_.alloc(3ull * P);
    tcams_.alloc(9ull * C);
    tpts_.alloc(3ull * P);
    counters_.alloc(4);  // [0] anomalies, [1] non-SPD V blocks, [2] scratch, [3] per-call non-SPD
    cam_pre_.alloc(16ull * C);
    scal_.alloc(8);
    GBA_CUDA_CHECK(cudaMemsetAsync(counters_.get(), 0, 4 * sizeof(unsigned long long), stream_));
    cams0_.alloc(9ull * C);
    pts0_.alloc(3ull * P);
    resid_valid_ = false;
    ff_holds_ = kFfNone;
    // copies cams / pts to the device (after the observation indices) while it
    // builds the structure; the stream has waited for them when this returns
    build_structure(obs_cam, obs_pt, obs_px, cams, pts);
    GBA_CUDA_CHECK(cudaMemcpyAsync(cams0_.get(), cams_.get(), 9ull * C * sizeof(double), cudaMemcpyDeviceToDevice,
                                   stream_));
    GBA_CUDA_CHECK(cudaMemcpyAsync(pts0_.get(), pts_.get(), 3ull * P * sizeof(double), cudaMemcpyDeviceToDevice,
                                   stream_));

    // normal equations (both forms)
    U_.alloc(81ull * C);
    bc_.alloc(9ull * C);
    V_.alloc(6ull * P);
    bp_.alloc(3ull * P);
    if (form_ == SolverForm::Plain) Vinv_.alloc(6ull * P);  // the mixed forms hold V'^-1 as float-float parts
    dc_.alloc(9ull * C);
    dp_.alloc(3ull * P);
    sse_part_.alloc(std::max({n_pchunk_, n_cchunk_, 1}));
    cam_part_.alloc(54ull * std::max(n_cchunk_, 1));
    // block partials: the largest single reduction, or the PCG layout
    // [r.r | r.z | p.q] = max(9C/256, C/32) + C/32 + 9C/256 (+ separators)
    red_part_.alloc(std::max(n_pchunk_, ceil_div(P, 256)) + 2 * ceil_div(9ll * C, 256) + 2 * ceil_div(C, 32) +
                    ceil_div(C, 8) + 64);
    if (form_ == SolverForm::Plain) {
        W_.alloc(27ull * E);
        JcR_.alloc(20ull * E);
        T_.alloc(27ull * E);
        n_pad_ = ((9 * C + 63) / 64) * 64;  // S itself is allocated at the first dense Schur step
        rhs_.alloc(n_pad_);
        pcg_x_.alloc(n_pad_);  // dense solve work vector
        info_.alloc(1);
        build_pairs();
    } else {
        js_ = jacobian_stride(E);
        Jc32_.alloc(18ull * js_);
        Jp32_.alloc(6ull * js_);
        J32c_.alloc(20ull * E);
        judge_e_.alloc(9ull * C);
        Vinv32_.alloc(6ull * P);
        cam_pre_ff_.alloc(32ull * C);
        pts_ff_.alloc(6ull * P);
        cams32_.alloc(28ull * C);
        Vinv32lo_.alloc(6ull * P);
        dcff_.alloc(18ull * C);
        pcg_p32_.alloc(12ull * C);  // padded FP32 camera vector (12 floats per camera; pads zeroed)
        if (C > 0) GBA_CUDA_CHECK(cudaMemsetAsync(pcg_p32_.get(), 0, 12ull * C * sizeof(float), stream_));
        r_cur_.alloc(2ull * E);
        r_trial_.alloc(2ull * E);
        Sdiag_.alloc(81ull * C);
        Pfac_.alloc(81ull * C);
        Pinv_.alloc(81ull * C);
        rhs_.alloc(9ull * C);
        pcg_e_.alloc(9ull * C);
        pcg_r_.alloc(9ull * C);
        pcg_z_.alloc(9ull * C);
        pcg_q_.alloc(9ull * C);
        ul32_.alloc(81ull * C);
        ref_r_.alloc(9ull * C);
        u_.alloc(2ull * E);
        g_cm_.alloc(4ull * E);
        pcg_s_.alloc(16);
        build_point_groups();
        set_matvec(0);
    }
    sync();
}

namespace {
// Pinned staging for scalar readbacks, one per host thread (a thread's solver
// calls never overlap); allocated on first use and kept for the thread.
constexpr size_t kPinnedBytes = 4096;
struct PinnedScratch {
    void* p = nullptr;
    ~PinnedScratch() {
        if (p) cudaFreeHost(p);
    }
};
thread_local PinnedScratch t_pinned;
}  // namespace

void Solver::read_back(std::initializer_list<HostRead> reads) const {
    if (!t_pinned.p) GBA_CUDA_CHECK(cudaMallocHost(&t_pinned.p, kPinnedBytes));
    char* stage = static_cast<char*>(t_pinned.p);
    size_t off = 0;
    for (const HostRead& r : reads) {
        if (off + r.bytes > kPinnedBytes) throw std::logic_error("read_back: more than the staging buffer");
        GBA_CUDA_CHECK(cudaMemcpyAsync(stage + off, r.src, r.bytes, cudaMemcpyDeviceToHost, stream_));
        off += (r.bytes + 15) & ~size_t{15};
    }
    sync();
    off = 0;
    for (const HostRead& r : reads) {
        std::memcpy(r.dst, stage + off, r.bytes);
        off += (r.bytes + 15) & ~size_t{15};
    }
}

// Waits for the solver stream by polling an event: the host resumes as soon as
// the stream drains, whatever scheduling mode the context was created with (a
// yielding or blocking stream synchronisation adds tens of microseconds per
// wait, and a solve waits some forty times). A device error ends the wait
// with that error.
void Solver::sync() const {
    if (!sync_ev_) GBA_CUDA_CHECK(cudaEventCreateWithFlags(&sync_ev_, cudaEventDisableTiming));
    GBA_CUDA_CHECK(cudaEventRecord(sync_ev_, stream_));
    cudaError_t e;
    while ((e = cudaEventQuery(sync_ev_)) == cudaErrorNotReady) {
    }
    GBA_CUDA_CHECK(e);
}

void Solver::set_params(const double* cams, const double* pts) {
    resid_valid_ = false;
    ff_holds_ = kFfNone;
    GBA_CUDA_CHECK(cudaMemcpyAsync(cams_.get(), cams, 9ull * C_ * sizeof(double), cudaMemcpyHostToDevice,
                                   stream_));
    GBA_CUDA_CHECK(cudaMemcpyAsync(pts_.get(), pts, 3ull * P_ * sizeof(double), cudaMemcpyHostToDevice,
                                   stream_));
}

void Solver::get_params(double* cams, double* pts) const {
    if (cams)
        GBA_CUDA_CHECK(cudaMemcpyAsync(cams, cams_.get(), 9ull * C_ * sizeof(double), cudaMemcpyDeviceToHost,
                                       stream_));
    if (pts)
        GBA_CUDA_CHECK(cudaMemcpyAsync(pts, pts_.get(), 3ull * P_ * sizeof(double), cudaMemcpyDeviceToHost,
                                       stream_));
    sync();
}

void Solver::build_structure(const int* obs_cam, const int* obs_pt, const double* obs_px, const double* cams,
                             const double* pts) {
    const int E = E_, P = P_, C = C_;
    DevBuf<int> d_oc(E), d_op(E), keys_sorted(E), iota(E);
    DevBuf<double> d_px(2ull * E);
    // The observation indices cross first, alone on the link: the index check
    // and the sort by point wait for them. The pixels (16 B per observation,
    // the bulk of the problem) and the parameters follow on a side stream while
    // the check and the sort run; the main stream waits for them only before
    // the gather that reads the pixels.
    struct SideCopy {
        cudaStream_t s = nullptr;
        cudaEvent_t ready = nullptr, done = nullptr;
        ~SideCopy() {  // runs before d_px is freed (declared after it): its copy must have landed
            if (s) cudaStreamSynchronize(s);
            if (done) cudaEventDestroy(done);
            if (ready) cudaEventDestroy(ready);
            if (s) cudaStreamDestroy(s);
        }
    } side;
    GBA_CUDA_CHECK(cudaStreamCreateWithFlags(&side.s, cudaStreamNonBlocking));
    GBA_CUDA_CHECK(cudaEventCreateWithFlags(&side.ready, cudaEventDisableTiming));
    GBA_CUDA_CHECK(cudaEventCreateWithFlags(&side.done, cudaEventDisableTiming));
    GBA_CUDA_CHECK(cudaMemcpyAsync(d_oc.get(), obs_cam, E * sizeof(int), cudaMemcpyHostToDevice, stream_));
    GBA_CUDA_CHECK(cudaMemcpyAsync(d_op.get(), obs_pt, E * sizeof(int), cudaMemcpyHostToDevice, stream_));
    GBA_CUDA_CHECK(cudaEventRecord(side.ready, stream_));  // after the index copies and the stream-ordered allocations
    GBA_CUDA_CHECK(cudaStreamWaitEvent(side.s, side.ready, 0));
    GBA_CUDA_CHECK(
        cudaMemcpyAsync(d_px.get(), obs_px, 2ull * E * sizeof(double), cudaMemcpyHostToDevice, side.s));
    GBA_CUDA_CHECK(cudaMemcpyAsync(cams_.get(), cams, 9ull * C * sizeof(double), cudaMemcpyHostToDevice, side.s));
    GBA_CUDA_CHECK(cudaMemcpyAsync(pts_.get(), pts, 3ull * P * sizeof(double), cudaMemcpyHostToDevice, side.s));
    GBA_CUDA_CHECK(cudaEventRecord(side.done, side.s));

    order_.alloc(E);
    s_cam_.alloc(E);
    s_pt_.alloc(E);
    s_px_.alloc(2ull * E);
    pt_off_.alloc(P + 1ull);
    cam_off_.alloc(C + 1ull);
    cam_slots_.alloc(E);

    // 0. observation indices in range, checked on the device before any kernel
    //    indexes with them
    {
        DevBuf<unsigned long long> bad(1);
        GBA_CUDA_CHECK(cudaMemsetAsync(bad.get(), 0, sizeof(unsigned long long), stream_));
        check_indices_kernel<<<grid_for(E), 256, 0, stream_>>>(d_oc.get(), d_op.get(), E, C, P, bad.get());
        GBA_LAUNCH_CHECK();
        unsigned long long h_bad = 0;
        GBA_CUDA_CHECK(cudaMemcpyAsync(&h_bad, bad.get(), sizeof h_bad, cudaMemcpyDeviceToHost, stream_));
        sync();
        if (h_bad) throw std::invalid_argument("observation index out of range");
    }

    iota_kernel<<<grid_for(E), 256, 0, stream_>>>(iota.get(), E);
    GBA_LAUNCH_CHECK();

    // 1. stable sort of observations by point
    size_t tmp_bytes = 0, tmp2 = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, d_op.get(), s_pt_.get(), iota.get(), order_.get(), E,
                                    0, bits_for(P + 1), stream_);
    cub::DeviceRadixSort::SortPairs(nullptr, tmp2, d_oc.get(), keys_sorted.get(), iota.get(),
                                    cam_slots_.get(), E, 0, bits_for(C + 1), stream_);
    DevBuf<unsigned char> tmp(std::max(tmp_bytes, tmp2));
    size_t tb = tmp.size();
    GBA_CUDA_CHECK(cub::DeviceRadixSort::SortPairs(tmp.get(), tb, d_op.get(), s_pt_.get(), iota.get(),
                                                   order_.get(), E, 0, bits_for(P + 1), stream_));
    GBA_CUDA_CHECK(cudaStreamWaitEvent(stream_, side.done, 0));
    gather_obs_kernel<<<grid_for(E), 256, 0, stream_>>>(order_.get(), d_oc.get(), d_px.get(), E, s_cam_.get(),
                                                        reinterpret_cast<double2*>(s_px_.get()));
    GBA_LAUNCH_CHECK();
    csr_offsets_kernel<<<grid_for(E), 256, 0, stream_>>>(s_pt_.get(), E, P, pt_off_.get());
    GBA_LAUNCH_CHECK();

    // 2. camera-major view of the slots (stable: slot order within a camera)
    tb = tmp.size();
    GBA_CUDA_CHECK(cub::DeviceRadixSort::SortPairs(tmp.get(), tb, s_cam_.get(), keys_sorted.get(), iota.get(),
                                                   cam_slots_.get(), E, 0, bits_for(C + 1), stream_));
    csr_offsets_kernel<<<grid_for(E), 256, 0, stream_>>>(keys_sorted.get(), E, C, cam_off_.get());
    GBA_LAUNCH_CHECK();
    cam_pos_.alloc(E);
    inverse_perm_kernel<<<grid_for(E), 256, 0, stream_>>>(cam_slots_.get(), E, cam_pos_.get());
    GBA_LAUNCH_CHECK();
    if (form_ != SolverForm::Plain) {
        cm_pt_.alloc(E);
        cm_pxff_.alloc(4ull * E);
        gather_cm_kernel<<<grid_for(E), 256, 0, stream_>>>(cam_slots_.get(), s_pt_.get(),
                                                           reinterpret_cast<const double2*>(s_px_.get()), E,
                                                           cm_pt_.get(), reinterpret_cast<float4*>(cm_pxff_.get()));
        GBA_LAUNCH_CHECK();
    }

    // 3. work chunks. Point chunks: the greedy packing (whole points, at most
    //    kPointChunk slots and points per chunk; a longer point alone) computed
    //    on the device by binary lifting: next[p] = end of the greedy chunk
    //    that starts at p (binary search on the CSR offsets), J_{k+1} =
    //    J_k(J_k), the chunk count from one lifted walk from point 0, and
    //    chunk i's start = next^i(0). Camera chunks are built on the host.
    int levels = 1;
    while ((1ll << levels) <= P) ++levels;
    {
        DevBuf<int> jump(static_cast<size_t>(levels) * (P + 1ull));
        chunk_next_kernel<<<grid_for(P + 1ll), 256, 0, stream_>>>(pt_off_.get(), P, jump.get());
        GBA_LAUNCH_CHECK();
        for (int k = 0; k + 1 < levels; ++k) {
            lift_kernel<<<grid_for(P + 1ll), 256, 0, stream_>>>(jump.get() + static_cast<size_t>(k) * (P + 1ull), P,
                                                               jump.get() + static_cast<size_t>(k + 1) * (P + 1ull));
            GBA_LAUNCH_CHECK();
        }
        DevBuf<int> d_n(1);
        chunk_count_kernel<<<1, 1, 0, stream_>>>(jump.get(), levels, P, d_n.get());
        GBA_LAUNCH_CHECK();
        int n = 0;
        GBA_CUDA_CHECK(cudaMemcpyAsync(&n, d_n.get(), sizeof n, cudaMemcpyDeviceToHost, stream_));
        sync();
        n_pchunk_ = n;
        pchunk_.alloc(n + 1ull);
        chunk_starts_kernel<<<grid_for(n + 1ll), 256, 0, stream_>>>(jump.get(), levels, P, n, pchunk_.get());
        GBA_LAUNCH_CHECK();
        pchunk4_.alloc(4ull * std::max(n, 1));
        if (n > 0) {
            chunk_ranges_kernel<<<grid_for(n), 256, 0, stream_>>>(pchunk_.get(), pt_off_.get(), n,
                                                                 reinterpret_cast<int4*>(pchunk4_.get()));
            GBA_LAUNCH_CHECK();
        }
    }
    std::vector<int> h_cam_off(C + 1);
    GBA_CUDA_CHECK(cudaMemcpyAsync(h_cam_off.data(), cam_off_.get(), (C + 1) * sizeof(int),
                                   cudaMemcpyDeviceToHost, stream_));
    sync();

    std::vector<int> cbeg, ccam, cam_chunk_off(C + 1);
    for (int c = 0; c < C; ++c) {
        cam_chunk_off[c] = static_cast<int>(cbeg.size());
        for (int b = h_cam_off[c]; b < h_cam_off[c + 1]; b += kCamChunk) {
            cbeg.push_back(b);
            ccam.push_back(c);
        }
    }
    cam_chunk_off[C] = static_cast<int>(cbeg.size());
    n_cchunk_ = static_cast<int>(cbeg.size());
    if (form_ != SolverForm::Plain) {  // the one-pass product's accumulators
        std::vector<int> acc_off(C + 1, 0);
        for (int c = 0; c < C; ++c)
            acc_off[c + 1] = acc_off[c] + (h_cam_off[c + 1] - h_cam_off[c] + kAccSlots - 1) / kAccSlots;
        n_acc_ = acc_off[C];
        acc_off_.alloc(C + 1ull);
        acc_id_.alloc(E);
        GBA_CUDA_CHECK(cudaMemcpyAsync(acc_off_.get(), acc_off.data(), (C + 1) * sizeof(int), cudaMemcpyHostToDevice,
                                       stream_));
        acc_id_kernel<<<grid_for(E), 256, 0, stream_>>>(s_cam_.get(), cam_pos_.get(), cam_off_.get(), acc_off_.get(),
                                                        E, kAccSlots, acc_id_.get());
        GBA_LAUNCH_CHECK();
        sync();  // acc_off dies at scope exit
    }

    cchunk_begin_.alloc(std::max<size_t>(cbeg.size(), 1));
    cchunk_cam_.alloc(std::max<size_t>(ccam.size(), 1));
    cam_chunk_off_.alloc(C + 1ull);
    if (!cbeg.empty()) {
        GBA_CUDA_CHECK(cudaMemcpyAsync(cchunk_begin_.get(), cbeg.data(), cbeg.size() * sizeof(int),
                                       cudaMemcpyHostToDevice, stream_));
        GBA_CUDA_CHECK(cudaMemcpyAsync(cchunk_cam_.get(), ccam.data(), ccam.size() * sizeof(int),
                                       cudaMemcpyHostToDevice, stream_));
    }
    GBA_CUDA_CHECK(cudaMemcpyAsync(cam_chunk_off_.get(), cam_chunk_off.data(), (C + 1) * sizeof(int),
                                   cudaMemcpyHostToDevice, stream_));
    sync();  // host vectors die at scope exit
}

void Solver::build_pairs() {
    const int P = P_, C = C_;
    DevBuf<long long> cnt(P + 1ull), base(P + 1ull);
    pair_count_kernel<<<grid_for(P), 256, 0, stream_>>>(pt_off_.get(), s_cam_.get(), P, cnt.get());
    GBA_LAUNCH_CHECK();
    GBA_CUDA_CHECK(cudaMemsetAsync(cnt.get() + P, 0, sizeof(long long), stream_));
    size_t tb = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tb, cnt.get(), base.get(), P + 1, stream_);
    {
        DevBuf<unsigned char> tmp(tb);
        GBA_CUDA_CHECK(cub::DeviceScan::ExclusiveSum(tmp.get(), tb, cnt.get(), base.get(), P + 1, stream_));
    }
    long long npairs = 0;
    GBA_CUDA_CHECK(cudaMemcpyAsync(&npairs, base.get() + P, sizeof(long long), cudaMemcpyDeviceToHost, stream_));
    sync();
    if (npairs <= 0 || npairs > INT_MAX) throw std::invalid_argument("Schur pair list size out of range");
    n_pairs_ = npairs;

    DevBuf<unsigned long long> key(npairs), key2(npairs), val(npairs), val2(npairs);
    pair_fill_kernel<<<grid_for(P), 256, 0, stream_>>>(pt_off_.get(), s_cam_.get(), P, C, base.get(), key.get(),
                                                       val.get());
    GBA_LAUNCH_CHECK();
    const int kb = bits_for(static_cast<long long>(C) * C + 1);
    tb = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tb, key.get(), key2.get(), val.get(), val2.get(), npairs, 0, kb,
                                    stream_);
    {
        DevBuf<unsigned char> tmp(tb);
        GBA_CUDA_CHECK(cub::DeviceRadixSort::SortPairs(tmp.get(), tb, key.get(), key2.get(), val.get(), val2.get(),
                                                       npairs, 0, kb, stream_));
    }
    pair_e_.alloc(npairs);
    pair_f_.alloc(npairs);
    pair_split_kernel<<<grid_for(npairs), 256, 0, stream_>>>(val2.get(), npairs, pair_e_.get(), pair_f_.get());
    GBA_LAUNCH_CHECK();
    val.release();
    val2.release();

    // run-length encode the block keys -> blocks and their pair ranges
    DevBuf<unsigned long long> ukey(npairs);
    DevBuf<int> counts(npairs + 1), nruns(1);
    tb = 0;
    cub::DeviceRunLengthEncode::Encode(nullptr, tb, key2.get(), ukey.get(), counts.get(), nruns.get(),
                                       static_cast<int>(npairs), stream_);
    {
        DevBuf<unsigned char> tmp(tb);
        GBA_CUDA_CHECK(cub::DeviceRunLengthEncode::Encode(tmp.get(), tb, key2.get(), ukey.get(), counts.get(),
                                                          nruns.get(), static_cast<int>(npairs), stream_));
    }
    int nb = 0;
    GBA_CUDA_CHECK(cudaMemcpyAsync(&nb, nruns.get(), sizeof(int), cudaMemcpyDeviceToHost, stream_));
    sync();
    n_blocks_ = nb;
    block_off_.alloc(nb + 1ull);
    block_ce_.alloc(nb);
    block_cf_.alloc(nb);
    GBA_CUDA_CHECK(cudaMemsetAsync(counts.get() + nb, 0, sizeof(int), stream_));
    tb = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tb, counts.get(), block_off_.get(), nb + 1, stream_);
    {
        DevBuf<unsigned char> tmp(tb);
        GBA_CUDA_CHECK(
            cub::DeviceScan::ExclusiveSum(tmp.get(), tb, counts.get(), block_off_.get(), nb + 1, stream_));
    }
    block_split_kernel<<<grid_for(nb), 256, 0, stream_>>>(ukey.get(), nb, C, block_ce_.get(), block_cf_.get());
    GBA_LAUNCH_CHECK();
    sync();
}

// Reverse Cuthill-McKee order of the camera graph (cameras adjacent when they
// share a point: the nonzero off-diagonal blocks of S), its block bandwidth,
// and whether a band holding it is at most a third of the dense matrix. Each
// component is started from a camera of least degree; neighbours are visited
// in increasing degree (ties by index), and the whole order is reversed. The
// cameras' own order is kept when its bandwidth is no larger.
// Host work O(blocks log), once per solver (the block list is fixed).
void Solver::plan_schur_band() {
    const int C = C_, nb = n_blocks_;
    std::vector<int> ce(nb), cf(nb);
    if (nb > 0) {
        GBA_CUDA_CHECK(cudaMemcpyAsync(ce.data(), block_ce_.get(), nb * sizeof(int), cudaMemcpyDeviceToHost, stream_));
        GBA_CUDA_CHECK(cudaMemcpyAsync(cf.data(), block_cf_.get(), nb * sizeof(int), cudaMemcpyDeviceToHost, stream_));
        sync();
    }
    std::vector<int> deg(C, 0);
    for (int b = 0; b < nb; ++b)
        if (ce[b] != cf[b]) {
            ++deg[ce[b]];
            ++deg[cf[b]];
        }
    std::vector<int> off(C + 1, 0);
    for (int c = 0; c < C; ++c) off[c + 1] = off[c] + deg[c];
    std::vector<int> adj(off[C]), fill(off.begin(), off.end() - 1);
    for (int b = 0; b < nb; ++b)
        if (ce[b] != cf[b]) {
            adj[fill[ce[b]]++] = cf[b];
            adj[fill[cf[b]]++] = ce[b];
        }
    for (int c = 0; c < C; ++c)
        std::sort(adj.begin() + off[c], adj.begin() + off[c + 1],
                  [&](int a, int b) { return deg[a] != deg[b] ? deg[a] < deg[b] : a < b; });
    std::vector<int> order;
    order.reserve(C);
    std::vector<char> seen(C, 0);
    std::vector<int> by_degree(C);
    for (int c = 0; c < C; ++c) by_degree[c] = c;
    std::stable_sort(by_degree.begin(), by_degree.end(), [&](int a, int b) { return deg[a] < deg[b]; });
    for (int start : by_degree) {
        if (seen[start]) continue;
        size_t head = order.size();
        order.push_back(start);
        seen[start] = 1;
        while (head < order.size()) {
            const int u = order[head++];
            for (int k = off[u]; k < off[u + 1]; ++k)
                if (!seen[adj[k]]) {
                    seen[adj[k]] = 1;
                    order.push_back(adj[k]);
                }
        }
    }
    std::vector<int> perm(C);
    for (int i = 0; i < C; ++i) perm[order[C - 1 - i]] = i;
    int w = 0, w_given = 0;
    for (int b = 0; b < nb; ++b) {
        w = std::max(w, std::abs(perm[ce[b]] - perm[cf[b]]));
        w_given = std::max(w_given, std::abs(ce[b] - cf[b]));
    }
    if (w_given <= w) {  // the cameras' own order is at least as narrow (e.g. a sequential capture)
        for (int c = 0; c < C; ++c) perm[c] = c;
        w = w_given;
    }
    const int band_rows = 9 * (w + 1);
    constexpr int kTile = 64;
    band_bt_ = (band_rows - 1 + kTile - 1) / kTile;
    band_ldb_ = (band_bt_ + 2) * kTile;
    band_beneficial_ = 3ll * band_ldb_ <= n_pad_;
    cam_perm_.alloc(C);
    GBA_CUDA_CHECK(cudaMemcpyAsync(cam_perm_.get(), perm.data(), C * sizeof(int), cudaMemcpyHostToDevice, stream_));
    sync();
}

unsigned long long Solver::anomalies() const {
    unsigned long long h[2];
    GBA_CUDA_CHECK(cudaMemcpyAsync(h, counters_.get(), sizeof h, cudaMemcpyDeviceToHost, stream_));
    sync();
    return h[0];
}

unsigned long long Solver::nonspd_total() const {
    unsigned long long h[2];
    GBA_CUDA_CHECK(cudaMemcpyAsync(h, counters_.get(), sizeof h, cudaMemcpyDeviceToHost, stream_));
    sync();
    return h[1];
}

void Solver::accept() {
    cams_.swap(tcams_);
    pts_.swap(tpts_);
    ff_holds_ = ff_holds_ == kFfTrial ? kFfCurrent : kFfNone;
    pts_ff_trial_ = false;
    if (form_ != SolverForm::Plain) {
        // the trial evaluation is the current one now: residuals and SSE
        r_cur_.swap(r_trial_);
        GBA_CUDA_CHECK(cudaMemcpyAsync(scal_.get(), scal_.get() + 1, sizeof(double), cudaMemcpyDeviceToDevice, stream_));
        resid_valid_ = true;
    }
}

const void* Solver::buffer(Buf b, size_t* bytes) const {
    auto ret = [&](const auto& buf) -> const void* {
        *bytes = buf.size() * sizeof(*buf.get());
        return buf.get();
    };
    switch (b) {
        case kU: return ret(U_);
        case kV: return ret(V_);
        case kBc: return ret(bc_);
        case kBp: return ret(bp_);
        case kW: return ret(W_);
        case kVinv: return ret(Vinv_);
        case kS: return ret(S_);
        case kRhs: return ret(rhs_);
        case kDc: return ret(dc_);
        case kDp: return ret(dp_);
        case kOrder: return ret(order_);
        case kJc32: return ret(Jc32_);
        case kJp32: return ret(Jp32_);
        case kSdiag: return ret(Sdiag_);
        case kCams: return ret(cams_);
        case kPts: return ret(pts_);
        case kTrialCams: return ret(tcams_);
        case kTrialPts: return ret(tpts_);
    }
    *bytes = 0;
    return nullptr;
}

}  // namespace gba

namespace gba {

void Solver::reset_params() {
    resid_valid_ = false;
    ff_holds_ = kFfNone;
    GBA_CUDA_CHECK(cudaMemcpyAsync(cams_.get(), cams0_.get(), 9ull * C_ * sizeof(double), cudaMemcpyDeviceToDevice,
                                   stream_));
    GBA_CUDA_CHECK(cudaMemcpyAsync(pts_.get(), pts0_.get(), 3ull * P_ * sizeof(double), cudaMemcpyDeviceToDevice,
                                   stream_));
}

void Solver::set_profiling(bool on) { profiling_ = on; }

cudaEvent_t Solver::prof_start() {
    if (!profiling_) return nullptr;
    cudaEvent_t e = nullptr;
    GBA_CUDA_CHECK(cudaEventCreate(&e));
    GBA_CUDA_CHECK(cudaEventRecord(e, stream_));
    return e;
}

void Solver::prof_stop(const char* name, cudaEvent_t start) {
    if (!start) return;
    cudaEvent_t e = nullptr;
    GBA_CUDA_CHECK(cudaEventCreate(&e));
    GBA_CUDA_CHECK(cudaEventRecord(e, stream_));
    timed_.push_back({name, start, e});
}

void Solver::kernel_stats(const std::string& name, long long* launches, double* total_ms) {
    sync();
    long long n = 0;
    double ms = 0.0;
    for (const Timed& t : timed_) {
        if (t.name != name) continue;
        float v = 0.f;
        GBA_CUDA_CHECK(cudaEventElapsedTime(&v, t.a, t.b));
        ms += v;
        ++n;
    }
    if (launches) *launches = n;
    if (total_ms) *total_ms = ms;
}

void Solver::prof_reset() {
    sync();
    for (Timed& t : timed_) {
        cudaEventDestroy(t.a);
        cudaEventDestroy(t.b);
    }
    timed_.clear();
}

}  // namespace gba
