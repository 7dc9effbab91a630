// Plain form: on-device assembly of the dense reduced camera system and its
// blocked FP64 Cholesky on the DMMA tensor cores.
//
// Reference: the host assembly src/lm.cu:488-594 (T_e = W_e V'^-1, privatised
// S -= T_e W_f^T over edge pairs of each point, merge, rhs, damped U blocks) and
// the host Eigen LLT src/lm.cu:598-604. Here:
//   * T_e is computed per slot on the device;
//   * S is assembled output-stationary: the edge pairs (e, f) of every point
//     with cam(e) >= cam(f) are sorted once by camera-pair block, and each
//     9x9 block is written once as the ordered sum of its pairs (no atomics,
//     deterministic), then the damped U blocks are added;
//   * the factorisation is right-looking blocked Cholesky (panel width 64):
//     diagonal-block potrf in shared memory, panel triangular solve, and the
//     trailing update C -= A B^T with mma.sync.m8n8k4 FP64 (DMMA).
// S is column-major, n_pad x n_pad (n_pad = 9C rounded up to 64, identity on
// the padding), lower triangle meaningful; the upper triangle is never read.
//
// Band layout (for camera graphs of local covisibility, where S is mostly
// zero): cameras are renumbered by reverse Cuthill-McKee so the nonzero blocks
// gather near the diagonal, and S keeps per column only the ldb rows from the
// diagonal down: element (i, j), 0 <= i - j < ldb, at S[i + j (ldb - 1)]. Every
// kernel below addresses S as A[i + j lda], so the same kernels run on the band
// with lda = ldb - 1; the panel loops stop bt tiles below the diagonal tile
// (Cholesky creates no fill outside the band). Writes to the strict upper
// triangle of a diagonal tile (i - j in [-63, -1]) land in rows ldb - 63 ..
// ldb - 1 of the previous column, which ldb = (bt + 2) 64 keeps outside the band.

#include "common.cuh"
#include "solver.hpp"

namespace gba {
namespace {

constexpr int NB = 64;       // panel width / tile size
constexpr int kSP = NB + 8;  // shared-memory stride (doubles) of K-major tiles: conflict-free DMMA fragments

__global__ void compute_T_kernel(const double* __restrict__ W, const double* __restrict__ Vinv,
                                 const int* __restrict__ s_pt, int E, double* __restrict__ T) {
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < E; s += (long long)gridDim.x * blockDim.x) {
        const double* Vi = Vinv + 6ll * s_pt[s];
        const double v00 = Vi[0], v10 = Vi[1], v11 = Vi[2], v20 = Vi[3], v21 = Vi[4], v22 = Vi[5];
        const double* We = W + 27 * s;
        double* Te = T + 27 * s;
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const double w0 = We[3 * i], w1 = We[3 * i + 1], w2 = We[3 * i + 2];
            Te[3 * i] = w0 * v00 + w1 * v10 + w2 * v20;
            Te[3 * i + 1] = w0 * v10 + w1 * v11 + w2 * v21;
            Te[3 * i + 2] = w0 * v20 + w1 * v21 + w2 * v22;
        }
    }
}

// One thread per (block, row i): S(9ce+i, 9cf+j) = -sum_{(e,f) in block} T_e(i,:) . W_f(j,:)
__global__ void __launch_bounds__(288) assemble_kernel(const int* __restrict__ block_off,
                                                      const int* __restrict__ block_ce,
                                                      const int* __restrict__ block_cf, const int* __restrict__ pe,
                                                      const int* __restrict__ pf, const double* __restrict__ T,
                                                      const double* __restrict__ W, int nblocks, int lda,
                                                      const int* __restrict__ perm, double* __restrict__ S) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long b = t / 9;
    const int i = static_cast<int>(t % 9);
    if (b >= nblocks) return;
    double acc[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) acc[j] = 0.0;
    for (int q = block_off[b]; q < block_off[b + 1]; ++q) {
        const double* Te = T + 27ll * pe[q] + 3 * i;
        const double t0 = Te[0], t1 = Te[1], t2 = Te[2];
        const double* Wf = W + 27ll * pf[q];
#pragma unroll
        for (int j = 0; j < 9; ++j) acc[j] += t0 * Wf[3 * j] + t1 * Wf[3 * j + 1] + t2 * Wf[3 * j + 2];
    }
    const int pe_ = perm ? perm[block_ce[b]] : block_ce[b];
    const int pf_ = perm ? perm[block_cf[b]] : block_cf[b];
    if (pe_ >= pf_) {
        const long long row = 9ll * pe_ + i;
        const long long col0 = 9ll * pf_;
#pragma unroll
        for (int j = 0; j < 9; ++j) S[row + (col0 + j) * lda] = -acc[j];
    } else {  // the renumbering put the block above the diagonal: store its transpose
        const long long col = 9ll * pe_ + i;
        const long long row0 = 9ll * pf_;
#pragma unroll
        for (int j = 0; j < 9; ++j) S[(row0 + j) + col * lda] = -acc[j];
    }
}

// Diagonal blocks += U_c + lambda * max(diag U_c, 1e-12); identity on padding.
__global__ void add_damped_u_kernel(const double* __restrict__ U, double lambda, int C, int n_pad, int lda,
                                    const int* __restrict__ perm, double* __restrict__ S) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < 81 * C) {
        const int c = t / 81, i = (t % 81) / 9, j = t % 9;
        double v = U[t];
        if (i == j) v += lambda * (v > 0.0 ? v : 1e-12);
        const long long pc = perm ? perm[c] : c;
        S[(9 * pc + i) + (9 * pc + j) * lda] += v;
    } else if (t < 81 * C + (n_pad - 9 * C)) {
        const long long r = 9ll * C + (t - 81 * C);
        S[r + r * lda] = 1.0;
    }
}

// Copies the assembled diagonal blocks S_cc (lower triangle mirrored) to Sdiag.
__global__ void extract_diag_blocks(const double* __restrict__ S, int C, int lda, const int* __restrict__ perm,
                                    double* __restrict__ Sdiag) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 81 * C) return;
    const int c = t / 81, i = (t % 81) / 9, j = t % 9;
    const int r = i >= j ? i : j, q = i >= j ? j : i;
    const long long pc = perm ? perm[c] : c;
    Sdiag[t] = S[(9 * pc + r) + (9 * pc + q) * lda];
}

// x[9 perm(c) + k] = v[9c + k] (to_band) or v[9c + k] = x[9 perm(c) + k].
__global__ void permute_cameras(const int* __restrict__ perm, int C, bool to_band, const double* __restrict__ in,
                                double* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 9 * C) return;
    const int c = t / 9, k = t % 9;
    const long long pos = 9ll * perm[c] + k;
    if (to_band)
        out[pos] = in[t];
    else
        out[t] = in[pos];
}

// rhs_c = bc_c - sum_{e in c} T_e bp_{p(e)}; one CTA per camera, ordered sums.
__global__ void __launch_bounds__(128) rhs_kernel(const int* __restrict__ cam_off, const int* __restrict__ cam_slots,
                                                 const int* __restrict__ s_pt, const double* __restrict__ T,
                                                 const double* __restrict__ bp, const double* __restrict__ bc,
                                                 double* __restrict__ rhs) {
    __shared__ double wpart[4][9];
    const int c = blockIdx.x;
    double acc[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[k] = 0.0;
    for (int i = cam_off[c] + threadIdx.x; i < cam_off[c + 1]; i += 128) {
        const int s = cam_slots[i];
        const double* Te = T + 27ll * s;
        const double* b = bp + 3ll * s_pt[s];
        const double b0 = b[0], b1 = b[1], b2 = b[2];
#pragma unroll
        for (int k = 0; k < 9; ++k) acc[k] += Te[3 * k] * b0 + Te[3 * k + 1] * b1 + Te[3 * k + 2] * b2;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const double v = warp_sum(acc[k]);
        if (lane == 0) wpart[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < 9) {
        const double v = wpart[0][threadIdx.x] + wpart[1][threadIdx.x] + wpart[2][threadIdx.x] + wpart[3][threadIdx.x];
        rhs[9ll * c + threadIdx.x] = bc[9ll * c + threadIdx.x] - v;
    }
}

// ---------------------------------------------------------------- Cholesky

// Factor the NB x NB diagonal block at (j0, j0) in shared memory.
// The pivot's square root and its reciprocal are taken once per column (by
// thread 0) and the column is scaled by multiplication: FP64 square roots and
// divisions expand into many instructions on GB300's narrow FP64 pipe, and the
// kernel runs on one SM, on the factorisation's critical path.
__global__ void __launch_bounds__(256) potrf_diag_kernel(double* __restrict__ A, int j0, int lda, int* __restrict__ info) {
    __shared__ double a[NB][NB + 1];  // a[col][row]
    __shared__ double lk[2];          // L_kk, 1 / L_kk
    __shared__ int failed;
    if (*info) return;
    const int tid = threadIdx.x;
    for (int idx = tid; idx < NB * NB; idx += 256) {
        const int r = idx % NB, c = idx / NB;
        a[c][r] = r >= c ? A[(j0 + r) + (long long)(j0 + c) * lda] : 0.0;
    }
    if (tid == 0) failed = 0;
    __syncthreads();
    for (int k = 0; k < NB; ++k) {
        const double piv = a[k][k];
        if (!(piv > 0.0)) {
            if (tid == 0) {
                failed = 1;
                *info = j0 + k + 1;
            }
            break;  // every thread read the same pivot
        }
        if (tid == 0) {
            const double lkk = sqrt(piv);
            lk[0] = lkk;
            lk[1] = 1.0 / lkk;
        }
        __syncthreads();
        const double inv = lk[1];
        for (int r = k + 1 + tid; r < NB; r += 256) a[k][r] *= inv;
        if (tid == 0) a[k][k] = lk[0];
        __syncthreads();
        for (int idx = tid; idx < NB * NB; idx += 256) {
            const int r = idx % NB, c = idx / NB;
            if (c > k && r >= c) a[c][r] -= a[k][r] * a[k][c];
        }
        __syncthreads();
    }
    __syncthreads();
    if (failed) return;
    for (int idx = tid; idx < NB * NB; idx += 256) {
        const int r = idx % NB, c = idx / NB;
        if (r >= c) A[(j0 + r) + (long long)(j0 + c) * lda] = a[c][r];
    }
}

// Panel solve: rows [j0+NB, n) of columns [j0, j0+NB) := B L_jj^{-T}.
// Rows are independent in X L^T = B: a CTA takes `rows` (a divisor of NB) rows
// of one panel tile, so that a narrow panel (a band's few tiles) still spreads
// over NB / rows CTAs per tile.
__global__ void __launch_bounds__(256) trsm_panel_kernel(double* __restrict__ A, int j0, int lda, int rows,
                                                        const int* __restrict__ info) {
    extern __shared__ double tsm[];
    double(*L)[NB + 1] = reinterpret_cast<double(*)[NB + 1]>(tsm);                  // L[col][row]
    double(*X)[NB + 1] = reinterpret_cast<double(*)[NB + 1]>(tsm + NB * (NB + 1));  // X[col][row < rows]
    if (*info) return;
    const int tid = threadIdx.x;
    const int parts = NB / rows;
    const long long r0 = j0 + NB + (long long)NB * (blockIdx.x / parts) + (long long)rows * (blockIdx.x % parts);
    __shared__ double rinv[NB];  // 1 / L_kk, one division per column
    for (int idx = tid; idx < NB * NB; idx += 256) {
        const int r = idx % NB, c = idx / NB;
        L[c][r] = r >= c ? A[(j0 + r) + (long long)(j0 + c) * lda] : 0.0;
    }
    for (int idx = tid; idx < rows * NB; idx += 256) {
        const int r = idx % rows, c = idx / rows;
        X[c][r] = A[(r0 + r) + (long long)(j0 + c) * lda];
    }
    if (tid < NB) rinv[tid] = 1.0 / A[(j0 + tid) + (long long)(j0 + tid) * lda];
    __syncthreads();
    for (int k = 0; k < NB; ++k) {
        const double d = rinv[k];
        for (int r = tid; r < rows; r += 256) X[k][r] *= d;
        __syncthreads();
        for (int idx = tid; idx < rows * NB; idx += 256) {
            const int r = idx % rows, c = idx / rows;
            if (c > k) X[c][r] -= X[k][r] * L[k][c];
        }
        __syncthreads();
    }
    for (int idx = tid; idx < rows * NB; idx += 256) {
        const int r = idx % rows, c = idx / rows;
        A[(r0 + r) + (long long)(j0 + c) * lda] = X[c][r];
    }
}

__device__ __forceinline__ void dmma_m8n8k4(double (&d)[2], double a, double b) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                 : "+d"(d[0]), "+d"(d[1])
                 : "d"(a), "d"(b));
}

// Trailing update of the lower tiles: C(ti,tj) -= A(ti) A(tj)^T, K = NB (the
// panel). 8 warps per 64x64 tile, each warp 32x16 = 4x2 DMMA tiles.
__global__ void __launch_bounds__(256) syrk_update_kernel(double* __restrict__ A, int j0, int ntiles, int lda,
                                                         const int* __restrict__ info) {
    extern __shared__ double smem[];
    double* As = smem;             // [k][row], stride kSP
    double* Bs = smem + NB * kSP;  // [k][col]
    if (*info) return;
    // lower-triangular tile index from the linear block index
    const long long bidx = blockIdx.x;
    int ti = static_cast<int>((sqrt(8.0 * (double)bidx + 1.0) - 1.0) * 0.5);
    while ((long long)(ti + 1) * (ti + 2) / 2 <= bidx) ++ti;
    while ((long long)ti * (ti + 1) / 2 > bidx) --ti;
    const int tj = static_cast<int>(bidx - (long long)ti * (ti + 1) / 2);
    if (ti >= ntiles) return;
    const long long R0 = j0 + NB + (long long)NB * ti, C0 = j0 + NB + (long long)NB * tj;
    const int tid = threadIdx.x;
    for (int idx = tid; idx < NB * NB; idx += 256) {
        const int r = idx % NB, k = idx / NB;
        As[k * kSP + r] = A[(R0 + r) + (long long)(j0 + k) * lda];
        Bs[k * kSP + r] = A[(C0 + r) + (long long)(j0 + k) * lda];
    }
    __syncthreads();
    const int warp = tid >> 5, lane = tid & 31;
    const int wm = (warp & 1) * 32, wn = (warp >> 1) * 16;
    const int fr = lane >> 2, fk = lane & 3;
    double acc[4][2][2];
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int n = 0; n < 2; ++n) acc[m][n][0] = acc[m][n][1] = 0.0;
#pragma unroll 4
    for (int kk = 0; kk < NB; kk += 4) {
        const double* ak = As + (kk + fk) * kSP + wm + fr;
        const double* bk = Bs + (kk + fk) * kSP + wn + fr;
        double af[4], bf[2];
#pragma unroll
        for (int m = 0; m < 4; ++m) af[m] = ak[8 * m];
#pragma unroll
        for (int n = 0; n < 2; ++n) bf[n] = bk[8 * n];
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
            for (int n = 0; n < 2; ++n) dmma_m8n8k4(acc[m][n], af[m], bf[n]);
    }
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int n = 0; n < 2; ++n) {
            const long long row = R0 + wm + 8 * m + fr;
            const long long col = C0 + wn + 8 * n + 2 * fk;
            A[row + col * lda] -= acc[m][n][0];
            A[row + (col + 1) * lda] -= acc[m][n][1];
        }
}

// The trailing update by 32 x 32 quadrants (four CTAs per 64 x 64 tile, the
// upper quadrant of a diagonal tile skipped): for steps with few tiles (a
// band's bt(bt+1)/2), so that the update spreads over four times as many SMs.
// 8 warps per quadrant, each warp 8 x 16 = 1 x 2 DMMA tiles.
constexpr int kSPq = 32 + 8;  // shared-memory stride (doubles) of the quadrant's K-major operands
__global__ void __launch_bounds__(256) syrk_update_quad_kernel(double* __restrict__ A, int j0, int ntiles, int lda,
                                                              const int* __restrict__ info) {
    __shared__ double As[NB * kSPq];  // [k][row]
    __shared__ double Bs[NB * kSPq];  // [k][col]
    if (*info) return;
    const long long bidx = blockIdx.x >> 2;
    const int quad = blockIdx.x & 3, qr = quad >> 1, qc = quad & 1;
    int ti = static_cast<int>((sqrt(8.0 * (double)bidx + 1.0) - 1.0) * 0.5);
    while ((long long)(ti + 1) * (ti + 2) / 2 <= bidx) ++ti;
    while ((long long)ti * (ti + 1) / 2 > bidx) --ti;
    const int tj = static_cast<int>(bidx - (long long)ti * (ti + 1) / 2);
    if (ti >= ntiles || (ti == tj && qr < qc)) return;
    const long long R0 = j0 + NB + (long long)NB * ti + 32 * qr, C0 = j0 + NB + (long long)NB * tj + 32 * qc;
    const int tid = threadIdx.x;
    for (int idx = tid; idx < 32 * NB; idx += 256) {
        const int r = idx % 32, k = idx / 32;
        As[k * kSPq + r] = A[(R0 + r) + (long long)(j0 + k) * lda];
        Bs[k * kSPq + r] = A[(C0 + r) + (long long)(j0 + k) * lda];
    }
    __syncthreads();
    const int warp = tid >> 5, lane = tid & 31;
    const int wm = (warp & 3) * 8, wn = (warp >> 2) * 16;
    const int fr = lane >> 2, fk = lane & 3;
    double acc[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
#pragma unroll 4
    for (int kk = 0; kk < NB; kk += 4) {
        const double af = As[(kk + fk) * kSPq + wm + fr];
        const double* bk = Bs + (kk + fk) * kSPq + wn + fr;
        dmma_m8n8k4(acc[0], af, bk[0]);
        dmma_m8n8k4(acc[1], af, bk[8]);
    }
#pragma unroll
    for (int n = 0; n < 2; ++n) {
        const long long row = R0 + wm + fr;
        const long long col = C0 + wn + 8 * n + 2 * fk;
        A[row + col * lda] -= acc[n][0];
        A[row + (col + 1) * lda] -= acc[n][1];
    }
}

// ---------------------------------------------------------------- triangular solves

// The diagonal block L_jj (lower triangle) and the reciprocals of its diagonal
// into shared memory: the triangular solves below then take their 64 dependent
// steps from shared memory, with multiplications (one division per column).
__device__ __forceinline__ void load_diag_tile(const double* __restrict__ L, int j0, int lda, double (*t)[NB + 1],
                                               double* rinv) {
    for (int idx = threadIdx.x; idx < NB * NB; idx += NB) {
        const int r = idx % NB, c = idx / NB;
        t[c][r] = r >= c ? L[(j0 + r) + (long long)(j0 + c) * lda] : 0.0;
    }
    __syncthreads();
    rinv[threadIdx.x] = 1.0 / t[threadIdx.x][threadIdx.x];
    __syncthreads();
}

// y_j = L_jj^{-1} b_j (forward) for the diagonal block at j0; one CTA of NB threads.
__global__ void trsv_lower_diag(const double* __restrict__ L, int j0, int lda, double* __restrict__ b,
                                const int* __restrict__ info) {
    __shared__ double x[NB];
    __shared__ double t[NB][NB + 1];  // t[col][row]
    __shared__ double rinv[NB];
    if (*info) return;
    const int tr = threadIdx.x;  // NB threads
    load_diag_tile(L, j0, lda, t, rinv);
    x[tr] = b[j0 + tr];
    __syncthreads();
    for (int k = 0; k < NB; ++k) {
        if (tr == k) x[k] *= rinv[k];
        __syncthreads();
        if (tr > k) x[tr] -= t[k][tr] * x[k];
        __syncthreads();
    }
    b[j0 + tr] = x[tr];
}

// b[j0+NB : n) -= L[j0+NB:n, j0:j0+NB] b[j0 : j0+NB); thread per row.
__global__ void gemv_lower_below(const double* __restrict__ L, int j0, int n, int lda, double* __restrict__ b,
                                 const int* __restrict__ info) {
    __shared__ double x[NB];
    if (*info) return;
    if (threadIdx.x < NB) x[threadIdx.x] = b[j0 + threadIdx.x];
    __syncthreads();
    const long long r = j0 + NB + blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= n) return;
    double s = 0.0;
#pragma unroll 8
    for (int k = 0; k < NB; ++k) s += L[r + (long long)(j0 + k) * lda] * x[k];
    b[r] -= s;
}

// x_j = L_jj^{-T} y_j (backward) for the diagonal block at j0; one CTA of NB threads.
__global__ void trsv_upper_diag(const double* __restrict__ L, int j0, int lda, double* __restrict__ b,
                                const int* __restrict__ info) {
    __shared__ double x[NB];
    __shared__ double t[NB][NB + 1];  // t[col][row]
    __shared__ double rinv[NB];
    if (*info) return;
    const int tr = threadIdx.x;
    load_diag_tile(L, j0, lda, t, rinv);
    x[tr] = b[j0 + tr];
    __syncthreads();
    for (int k = NB - 1; k >= 0; --k) {
        if (tr == k) x[k] *= rinv[k];
        __syncthreads();
        // row tr of L^T is column tr of L: (L^T)(tr, k) = L(k, tr), k > tr
        if (tr < k) x[tr] -= t[tr][k] * x[k];
        __syncthreads();
    }
    b[j0 + tr] = x[tr];
}

// y[i0 : j0) -= L[j0:j0+NB, i0:j0]^T x_j; one warp per output row i (reads column i of L).
__global__ void gemv_upper_above(const double* __restrict__ L, int i0, int j0, int lda, double* __restrict__ b,
                                 const int* __restrict__ info) {
    __shared__ double x[NB];
    if (*info) return;
    if (threadIdx.x < NB) x[threadIdx.x] = b[j0 + threadIdx.x];
    __syncthreads();
    const int warp = i0 + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (warp >= j0) return;
    const double* col = L + (long long)warp * lda + j0;
    double s = col[lane] * x[lane] + col[lane + 32] * x[lane + 32];
    s = warp_sum(s);
    if (lane == 0) b[warp] -= s;
}

}  // namespace

// bt: tiles below the diagonal tile that hold nonzeros (n / 64 - 1 for a
// dense matrix; lda = ldb - 1 with ldb >= (bt + 2) 64 for a band).
void dense_potrf(double* A, int n, int lda, int bt, int* info, cudaStream_t s) {
    if (n % NB != 0 || bt < 0 || (bt < n / NB - 1 ? lda + 1 < (bt + 2) * NB : lda < n))
        throw std::invalid_argument("dense_potrf: n must be a multiple of 64 and lda hold the band");
    GBA_CUDA_CHECK(cudaMemsetAsync(info, 0, sizeof(int), s));
    static bool attr = false;
    const int smem = 2 * NB * kSP * sizeof(double);
    const int tsmem = 2 * NB * (NB + 1) * sizeof(double);
    if (!attr) {
        GBA_CUDA_CHECK(cudaFuncSetAttribute(syrk_update_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        GBA_CUDA_CHECK(cudaFuncSetAttribute(trsm_panel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, tsmem));
        attr = true;
    }
    const int nt = n / NB;
    for (int jb = 0; jb < nt; ++jb) {
        const int j0 = jb * NB;
        potrf_diag_kernel<<<1, 256, 0, s>>>(A, j0, lda, info);
        GBA_LAUNCH_CHECK();
        const int below = std::min(nt - jb - 1, bt);
        if (below == 0) {
            if (jb == nt - 1) break;
            continue;
        }
        // few panel tiles (a band, or the last steps of a dense matrix): split
        // them over more CTAs
        const int sms = device_sm_count();
        const int rows = below * 4 <= sms ? 16 : NB;
        trsm_panel_kernel<<<below * (NB / rows), 256, tsmem, s>>>(A, j0, lda, rows, info);
        GBA_LAUNCH_CHECK();
        const long long tiles = (long long)below * (below + 1) / 2;
        if (tiles * 2 <= sms)
            syrk_update_quad_kernel<<<static_cast<unsigned>(4 * tiles), 256, 0, s>>>(A, j0, below, lda, info);
        else
            syrk_update_kernel<<<static_cast<unsigned>(tiles), 256, smem, s>>>(A, j0, below, lda, info);
        GBA_LAUNCH_CHECK();
    }
}

void dense_potrs(const double* L, int n, int lda, int bt, double* b, const int* info, cudaStream_t s) {
    if (n % NB != 0 || bt < 0 || (bt < n / NB - 1 ? lda + 1 < (bt + 2) * NB : lda < n))
        throw std::invalid_argument("dense_potrs: n must be a multiple of 64 and lda hold the band");
    const int nt = n / NB;
    for (int jb = 0; jb < nt; ++jb) {
        const int j0 = jb * NB;
        trsv_lower_diag<<<1, NB, 0, s>>>(L, j0, lda, b, info);
        GBA_LAUNCH_CHECK();
        const int r_end = static_cast<int>(std::min<long long>(n, j0 + NB + (long long)bt * NB));
        if (j0 + NB < r_end) {
            gemv_lower_below<<<ceil_div(r_end - j0 - NB, 256), 256, 0, s>>>(L, j0, r_end, lda, b, info);
            GBA_LAUNCH_CHECK();
        }
    }
    for (int jb = nt - 1; jb >= 0; --jb) {
        const int j0 = jb * NB;
        trsv_upper_diag<<<1, NB, 0, s>>>(L, j0, lda, b, info);
        GBA_LAUNCH_CHECK();
        const int i0 = std::max(0, j0 - bt * NB);
        if (j0 > i0) {
            gemv_upper_above<<<ceil_div(32ll * (j0 - i0), 256), 256, 0, s>>>(L, i0, j0, lda, b, info);
            GBA_LAUNCH_CHECK();
        }
    }
}

void Solver::ensure_schur_storage() {
    const int want = schur_layout_;
    if (S_.get() && schur_layout_planned_ == want) return;
    bool band = false;
    if (want == 2) {
        plan_schur_band();
        band = true;
    } else if (want == 0 && C_ >= 2 && 3ll * n_blocks_ <= static_cast<long long>(C_) * C_) {
        plan_schur_band();  // a band can only pay with at most ~1/3 of the blocks present
        band = band_beneficial_;
    }
    band_mode_ = band;
    S_.release();
    S_.alloc(static_cast<size_t>(n_pad_) * (band ? band_ldb_ : n_pad_));
    schur_layout_planned_ = want;
}

int Solver::schur_dense(double lambda) {
    ensure_schur_storage();
    const int lda = band_mode_ ? band_ldb_ - 1 : n_pad_;
    const int bt = band_mode_ ? band_bt_ : n_pad_ / NB - 1;
    const int* perm = band_mode_ ? cam_perm_.get() : nullptr;
    compute_T_kernel<<<std::min(ceil_div(E_, 256), 32 * device_sm_count()), 256, 0, stream_>>>(
        W_.get(), Vinv_.get(), s_pt_.get(), E_, T_.get());
    GBA_LAUNCH_CHECK();
    GBA_CUDA_CHECK(cudaMemsetAsync(S_.get(), 0, S_.size() * sizeof(double), stream_));
    if (n_blocks_ > 0) {
        cudaEvent_t ev = prof_start();
        assemble_kernel<<<ceil_div(9ll * n_blocks_, 288), 288, 0, stream_>>>(
            block_off_.get(), block_ce_.get(), block_cf_.get(), pair_e_.get(), pair_f_.get(), T_.get(), W_.get(),
            n_blocks_, lda, perm, S_.get());
        GBA_LAUNCH_CHECK();
        prof_stop("schur_assemble", ev);
    }
    add_damped_u_kernel<<<ceil_div(81ll * C_ + (n_pad_ - 9 * C_), 256), 256, 0, stream_>>>(U_.get(), lambda, C_,
                                                                                        n_pad_, lda, perm, S_.get());
    GBA_LAUNCH_CHECK();
    GBA_CUDA_CHECK(cudaMemsetAsync(rhs_.get(), 0, rhs_.size() * sizeof(double), stream_));
    rhs_kernel<<<C_, 128, 0, stream_>>>(cam_off_.get(), cam_slots_.get(), s_pt_.get(), T_.get(), bp_.get(),
                                        bc_.get(), rhs_.get());
    GBA_LAUNCH_CHECK();
    if (harvest_) {
        if (!Sdiag_.get()) Sdiag_.alloc(81ull * C_);
        extract_diag_blocks<<<ceil_div(81ll * C_, 256), 256, 0, stream_>>>(S_.get(), C_, lda, perm, Sdiag_.get());
        GBA_LAUNCH_CHECK();
    }
    cudaEvent_t ev = prof_start();
    dense_potrf(S_.get(), n_pad_, lda, bt, info_.get(), stream_);
    prof_stop("dense_potrf", ev);
    int info = 0;
    read_back({{&info, info_.get(), sizeof info}});
    if (info != 0) return info;
    // solve in a copy so rhs stays the assembled right-hand side (in the band
    // layout the copy is in the renumbered camera order; the padding stays 0)
    if (band_mode_) {
        GBA_CUDA_CHECK(cudaMemsetAsync(pcg_x_.get(), 0, n_pad_ * sizeof(double), stream_));
        permute_cameras<<<ceil_div(9 * C_, 256), 256, 0, stream_>>>(perm, C_, true, rhs_.get(), pcg_x_.get());
        GBA_LAUNCH_CHECK();
    } else {
        GBA_CUDA_CHECK(cudaMemcpyAsync(pcg_x_.get(), rhs_.get(), n_pad_ * sizeof(double), cudaMemcpyDeviceToDevice,
                                       stream_));
    }
    dense_potrs(S_.get(), n_pad_, lda, bt, pcg_x_.get(), info_.get(), stream_);
    if (band_mode_) {
        permute_cameras<<<ceil_div(9 * C_, 256), 256, 0, stream_>>>(perm, C_, false, pcg_x_.get(), dc_.get());
        GBA_LAUNCH_CHECK();
    } else {
        GBA_CUDA_CHECK(cudaMemcpyAsync(dc_.get(), pcg_x_.get(), 9ull * C_ * sizeof(double), cudaMemcpyDeviceToDevice,
                                       stream_));
    }
    sync();
    return 0;
}

}  // namespace gba
