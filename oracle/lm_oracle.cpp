// ORACLE — test infrastructure only. CPU FP64 restatement of the reference
// LM bundle adjuster (FireHorseAutumn/gpu-bundle-adjustment, src/lm.cu) used
// as the parity checker and as the timed CPU baseline. Nothing in the product
// library links or calls this file.
//
// Pinning: the residual model is checked against the reference's own
// src/bal_reader.cpp compiled from source (oracle/_ref, see build_oracle.py);
// the Jacobian against central differences on the reference test's golden
// cases (tests/test_vs_ceres.cpp:34-39); the Schur/LLT stage against an
// independent dense solve (numpy) in the tests. The reference LM driver itself
// (src/lm.cu) needs Eigen and cannot be built here, so the LM trajectory is
// "parity pinned by restatement": every step below cites the reference line
// it follows.
//
// Deterministic: sums run in a fixed order (edge order for U/V/W/b, point
// order for S and rhs), independent of the thread count.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

namespace {

// ------------------------------------------------------------------ model
// Residual, src/lm.cu:58-82 (theta^2 > 1e-24 branch, first-order branch below).
void residual(const double* cam, const double* X, const double* obs, double* r) {
    const double* a = cam;
    double P[3];
    const double th2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
    if (th2 > 1e-24) {
        const double th = std::sqrt(th2);
        const double w[3] = {a[0] / th, a[1] / th, a[2] / th};
        const double c = std::cos(th), s = std::sin(th);
        const double wx[3] = {w[1] * X[2] - w[2] * X[1], w[2] * X[0] - w[0] * X[2], w[0] * X[1] - w[1] * X[0]};
        const double q = w[0] * X[0] + w[1] * X[1] + w[2] * X[2];
        for (int i = 0; i < 3; ++i) P[i] = X[i] * c + wx[i] * s + w[i] * q * (1.0 - c) + cam[3 + i];
    } else {
        const double ax[3] = {a[1] * X[2] - a[2] * X[1], a[2] * X[0] - a[0] * X[2], a[0] * X[1] - a[1] * X[0]};
        for (int i = 0; i < 3; ++i) P[i] = X[i] + ax[i] + cam[3 + i];
    }
    const double u = -P[0] / P[2], v = -P[1] / P[2];
    const double r2 = u * u + v * v;
    const double d = 1.0 + cam[7] * r2 + cam[8] * r2 * r2;
    r[0] = cam[6] * d * u - obs[0];
    r[1] = cam[6] * d * v - obs[1];
}

// Residual + Jacobian by the reference's derivation, src/lm.cu:93-191:
// dRX/dw = -s [X]x + (1-c)((w.X) I + w X^T), dRX/da = (dRX/dw - (dRX/dw w) w^T)/theta
// + (dRX/dtheta) w^T; first-order branch dRX/da = -[X]x, R = I.
void residual_jacobian(const double* cam, const double* X, const double* obs, double* r, double* Jc, double* Jp) {
    residual(cam, X, obs, r);
    const double* a = cam;
    const double th2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
    double R[9], D[9], RX[3];
    auto skew = [](const double* v, double* m) {  // [v]x, row-major
        m[0] = 0; m[1] = -v[2]; m[2] = v[1];
        m[3] = v[2]; m[4] = 0; m[5] = -v[0];
        m[6] = -v[1]; m[7] = v[0]; m[8] = 0;
    };
    if (th2 > 1e-24) {
        const double th = std::sqrt(th2);
        const double w[3] = {a[0] / th, a[1] / th, a[2] / th};
        const double c = std::cos(th), s = std::sin(th);
        const double wx[3] = {w[1] * X[2] - w[2] * X[1], w[2] * X[0] - w[0] * X[2], w[0] * X[1] - w[1] * X[0]};
        const double q = w[0] * X[0] + w[1] * X[1] + w[2] * X[2];
        for (int i = 0; i < 3; ++i) RX[i] = X[i] * c + wx[i] * s + w[i] * q * (1.0 - c);
        double W[9];
        skew(w, W);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) R[3 * i + j] = (i == j ? c : 0.0) + s * W[3 * i + j] + (1.0 - c) * w[i] * w[j];
        double dth[3];
        for (int i = 0; i < 3; ++i) dth[i] = -s * X[i] + c * wx[i] + s * q * w[i];
        double Xs[9], A[9];
        skew(X, Xs);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) A[3 * i + j] = -s * Xs[3 * i + j] + (1.0 - c) * ((i == j ? q : 0.0) + w[i] * X[j]);
        double Aw[3] = {0, 0, 0};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) Aw[i] += A[3 * i + j] * w[j];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) D[3 * i + j] = (A[3 * i + j] - Aw[i] * w[j]) / th + dth[i] * w[j];
    } else {
        const double ax[3] = {a[1] * X[2] - a[2] * X[1], a[2] * X[0] - a[0] * X[2], a[0] * X[1] - a[1] * X[0]};
        for (int i = 0; i < 3; ++i) RX[i] = X[i] + ax[i];
        for (int i = 0; i < 9; ++i) R[i] = (i % 4 == 0) ? 1.0 : 0.0;
        double Xs[9];
        skew(X, Xs);
        for (int i = 0; i < 9; ++i) D[i] = -Xs[i];
    }
    const double P[3] = {RX[0] + cam[3], RX[1] + cam[4], RX[2] + cam[5]};
    const double u = -P[0] / P[2], v = -P[1] / P[2];
    const double r2 = u * u + v * v;
    const double f = cam[6], k1 = cam[7], k2 = cam[8];
    const double d = 1.0 + k1 * r2 + k2 * r2 * r2;
    const double L = k1 + 2.0 * k2 * r2;
    const double D00 = f * (d + 2.0 * L * u * u), D01 = 2.0 * f * L * u * v, D11 = f * (d + 2.0 * L * v * v);
    const double iz = 1.0 / P[2];
    const double M[6] = {-iz, 0.0, P[0] * iz * iz, 0.0, -iz, P[1] * iz * iz};
    double DM[6];
    for (int j = 0; j < 3; ++j) {
        DM[j] = D00 * M[j] + D01 * M[3 + j];
        DM[3 + j] = D01 * M[j] + D11 * M[3 + j];
    }
    for (int row = 0; row < 2; ++row) {
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) s += DM[3 * row + k] * D[3 * k + j];
            Jc[9 * row + j] = s;
        }
        for (int j = 0; j < 3; ++j) Jc[9 * row + 3 + j] = DM[3 * row + j];
        const double p = row == 0 ? u : v;
        Jc[9 * row + 6] = d * p;
        Jc[9 * row + 7] = f * r2 * p;
        Jc[9 * row + 8] = f * r2 * r2 * p;
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) s += DM[3 * row + k] * R[3 * k + j];
            Jp[3 * row + j] = s;
        }
    }
}

// Huber loss on the squared residual norm (Ceres HuberLoss, the loss option of
// the reference's Ceres baseline, benchmarks/bench_ceres.cpp:120-142): rho(s) = s
// for s <= delta^2, else 2 delta sqrt(s) - delta^2; rows weighted by
// sqrt(rho'(s)) = sqrt(min(1, delta / sqrt(s))) (Ceres' corrector when rho'' <= 0).
// delta <= 0: no loss.
double huber_rho(double s, double delta) {
    return (delta > 0.0 && s > delta * delta) ? 2.0 * delta * std::sqrt(s) - delta * delta : s;
}
double huber_sqrt_weight(double s, double delta) {
    return (delta > 0.0 && s > delta * delta) ? std::sqrt(delta / std::sqrt(s)) : 1.0;
}

bool all_finite(const double* v, int n) {
    for (int i = 0; i < n; ++i)
        if (!std::isfinite(v[i])) return false;
    return true;
}

// ------------------------------------------------------------------ threads
template <typename F>
void parallel_for(int n, int threads, F&& f) {
    threads = std::max(1, std::min(threads, n));
    if (threads == 1) {
        f(0, n, 0);
        return;
    }
    std::vector<std::thread> pool;
    const int chunk = (n + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        const int b = t * chunk, e = std::min(n, b + chunk);
        if (b >= e) break;
        pool.emplace_back([&f, b, e, t] { f(b, e, t); });
    }
    for (auto& th : pool) th.join();
}

struct Problem {
    int C, P, E;
    const int* oc;
    const int* op;
    const double* px;
    std::vector<std::vector<int>> point_edges;  // src/lm.cu:380-381
    double delta = 0.0;                         // Huber threshold, <= 0: no loss
};

// Normal equations, edge order (src/lm.cu:205-252 accumulation, 399-422).
// U: 81C full symmetric; V: 9P full symmetric; W: 27E; non-finite edges skipped,
// their W zeroed.
void accumulate(const Problem& pr, const double* cams, const double* pts, double* U, double* V, double* W, double* bc,
                double* bp, double* sse, unsigned long long* anomalies) {
    std::fill(U, U + 81ll * pr.C, 0.0);
    std::fill(V, V + 9ll * pr.P, 0.0);
    std::fill(bc, bc + 9ll * pr.C, 0.0);
    std::fill(bp, bp + 3ll * pr.P, 0.0);
    double s = 0.0;
    for (int e = 0; e < pr.E; ++e) {
        const int c = pr.oc[e], p = pr.op[e];
        double r[2], Jc[18], Jp[6];
        residual_jacobian(cams + 9ll * c, pts + 3ll * p, pr.px + 2ll * e, r, Jc, Jp);
        double* We = W + 27ll * e;
        if (!(all_finite(r, 2) && all_finite(Jc, 18) && all_finite(Jp, 6))) {
            ++*anomalies;
            std::fill(We, We + 27, 0.0);
            continue;
        }
        const double sq = r[0] * r[0] + r[1] * r[1];
        s += huber_rho(sq, pr.delta);
        if (pr.delta > 0.0) {
            const double sw = huber_sqrt_weight(sq, pr.delta);
            for (double& v : r) v *= sw;
            for (double& v : Jc) v *= sw;
            for (double& v : Jp) v *= sw;
        }
        for (int i = 0; i < 9; ++i)
            for (int j = 0; j < 3; ++j) We[3 * i + j] = Jc[i] * Jp[j] + Jc[9 + i] * Jp[3 + j];
        double* Uc = U + 81ll * c;
        for (int i = 0; i < 9; ++i) {
            for (int j = 0; j <= i; ++j) Uc[9 * i + j] += Jc[i] * Jc[j] + Jc[9 + i] * Jc[9 + j];
            bc[9ll * c + i] -= Jc[i] * r[0] + Jc[9 + i] * r[1];
        }
        double* Vp = V + 9ll * p;
        for (int i = 0; i < 3; ++i) {
            for (int j = 0; j <= i; ++j) Vp[3 * i + j] += Jp[i] * Jp[j] + Jp[3 + i] * Jp[3 + j];
            bp[3ll * p + i] -= Jp[i] * r[0] + Jp[3 + i] * r[1];
        }
    }
    for (int c = 0; c < pr.C; ++c)
        for (int i = 0; i < 9; ++i)
            for (int j = 0; j < i; ++j) U[81ll * c + 9 * j + i] = U[81ll * c + 9 * i + j];
    for (int p = 0; p < pr.P; ++p)
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < i; ++j) V[9ll * p + 3 * j + i] = V[9ll * p + 3 * i + j];
    *sse = s;
}

double cost(const Problem& pr, const double* cams, const double* pts, unsigned long long* anomalies) {
    double s = 0.0;
    for (int e = 0; e < pr.E; ++e) {
        double r[2];
        residual(cams + 9ll * pr.oc[e], pts + 3ll * pr.op[e], pr.px + 2ll * e, r);
        if (!std::isfinite(r[0]) || !std::isfinite(r[1])) {
            ++*anomalies;
            continue;
        }
        s += huber_rho(r[0] * r[0] + r[1] * r[1], pr.delta);
    }
    return s;
}

// 3x3 SPD inverse through Cholesky (schur.cuh:66-96); false if not SPD.
bool inverse3_spd(const double* A, double* Ai) {
    double L[9] = {0};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j <= i; ++j) {
            double s = A[3 * i + j];
            for (int k = 0; k < j; ++k) s -= L[3 * i + k] * L[3 * j + k];
            if (i == j) {
                if (!(s > 0.0)) return false;
                L[3 * i + i] = std::sqrt(s);
            } else {
                L[3 * i + j] = s / L[3 * j + j];
            }
        }
    double Li[9] = {0};
    for (int i = 0; i < 3; ++i) {
        Li[3 * i + i] = 1.0 / L[3 * i + i];
        for (int j = 0; j < i; ++j) {
            double s = 0.0;
            for (int k = j; k < i; ++k) s -= L[3 * i + k] * Li[3 * k + j];
            Li[3 * i + j] = s / L[3 * i + i];
        }
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) s += Li[3 * k + i] * Li[3 * k + j];
            Ai[3 * i + j] = s;
        }
    return true;
}

// Blocked right-looking Cholesky of the lower triangle of a column-major n x n
// matrix (stands in for Eigen::LLT<MatrixXd, Lower>, src/lm.cu:598). Returns 0
// or the 1-based failed column.
int cholesky(double* A, int n, int threads) {
    const int nb = 64;
    auto at = [&](int i, int j) -> double& { return A[i + static_cast<long long>(j) * n]; };
    for (int k0 = 0; k0 < n; k0 += nb) {
        const int k1 = std::min(n, k0 + nb);
        // unblocked factor of the panel columns k0..k1 (rows k0..n)
        for (int k = k0; k < k1; ++k) {
            double piv = at(k, k);
            for (int m = k0; m < k; ++m) piv -= at(k, m) * at(k, m);
            if (!(piv > 0.0)) return k + 1;
            const double lkk = std::sqrt(piv);
            at(k, k) = lkk;
            const int rows = n - k - 1;
            parallel_for(rows, rows > 4096 ? threads : 1, [&](int b, int e, int) {
                for (int ii = b; ii < e; ++ii) {
                    const int i = k + 1 + ii;
                    double s = at(i, k);
                    for (int m = k0; m < k; ++m) s -= at(i, m) * at(k, m);
                    at(i, k) = s / lkk;
                }
            });
        }
        // trailing update A22 -= L21 L21^T (lower), parallel over columns
        const int m = n - k1;
        if (m <= 0) break;
        parallel_for(m, threads, [&](int b, int e, int) {
            for (int jj = b; jj < e; ++jj) {
                const int j = k1 + jj;
                double* colj = &at(0, j);
                for (int k = k0; k < k1; ++k) {
                    const double ljk = at(j, k);
                    if (ljk == 0.0) continue;
                    const double* colk = &at(0, k);
                    for (int i = j; i < n; ++i) colj[i] -= colk[i] * ljk;
                }
            }
        });
    }
    return 0;
}

void cholesky_solve(const double* L, int n, double* b) {
    for (int i = 0; i < n; ++i) {
        double s = b[i];
        for (int k = 0; k < i; ++k) s -= L[i + static_cast<long long>(k) * n] * b[k];
        b[i] = s / L[i + static_cast<long long>(i) * n];
    }
    for (int i = n - 1; i >= 0; --i) {
        double s = b[i];
        const double* col = L + static_cast<long long>(i) * n;
        for (int k = i + 1; k < n; ++k) s -= col[k] * b[k];
        b[i] = s / col[i];
    }
}

struct State {
    std::vector<double> U, V, W, bc, bp, Vinv, T, S, rhs, dc, dp;
};

// Damped point inverses, T_e, dense S (lower block triangle, column-major) and
// rhs (src/lm.cu:469-594). Returns false on a non-SPD damped V block.
bool assemble(const Problem& pr, State& st, double lambda, int threads) {
    const int C = pr.C, P = pr.P, E = pr.E, n = 9 * C;
    st.Vinv.assign(9ll * P, 0.0);
    for (int p = 0; p < P; ++p) {  // src/lm.cu:289-302
        const double* Vp = &st.V[9ll * p];
        double A[9];
        for (int k = 0; k < 9; ++k) A[k] = Vp[k];
        for (int i = 0; i < 3; ++i) A[4 * i] += lambda * (Vp[4 * i] > 0.0 ? Vp[4 * i] : 1e-12);
        if (!inverse3_spd(A, &st.Vinv[9ll * p])) return false;
    }
    st.T.assign(27ll * E, 0.0);  // T_e = W_e V'^-1, src/lm.cu:492-514
    parallel_for(E, threads, [&](int b, int e, int) {
        for (int k = b; k < e; ++k) {
            const double* We = &st.W[27ll * k];
            const double* Vi = &st.Vinv[9ll * pr.op[k]];
            double* Te = &st.T[27ll * k];
            for (int i = 0; i < 9; ++i)
                for (int j = 0; j < 3; ++j)
                    Te[3 * i + j] = We[3 * i] * Vi[j] + We[3 * i + 1] * Vi[3 + j] + We[3 * i + 2] * Vi[6 + j];
        }
    });
    // S lower block triangle -= T_e W_f^T over pairs with c_f <= c_e (src/lm.cu:515-559);
    // rows partitioned over threads by camera, points in order within each thread.
    st.S.assign(static_cast<size_t>(n) * n, 0.0);
    st.rhs.assign(n, 0.0);
    parallel_for(C, threads, [&](int cb, int ce_end, int) {
        for (int p = 0; p < P; ++p) {
            const auto& edges = pr.point_edges[p];
            for (int e : edges) {
                const int ce = pr.oc[e];
                if (ce < cb || ce >= ce_end) continue;
                const double* Te = &st.T[27ll * e];
                for (int f : edges) {
                    const int cf = pr.oc[f];
                    if (cf > ce) continue;
                    const double* Wf = &st.W[27ll * f];
                    for (int j = 0; j < 9; ++j) {
                        double* col = &st.S[static_cast<size_t>(9 * cf + j) * n + 9 * ce];
                        for (int i = 0; i < 9; ++i)
                            col[i] -= Te[3 * i] * Wf[3 * j] + Te[3 * i + 1] * Wf[3 * j + 1] + Te[3 * i + 2] * Wf[3 * j + 2];
                    }
                }
            }
        }
    });
    for (int p = 0; p < P; ++p) {  // rhs = bc - sum T_e bp (src/lm.cu:533-535, 580-584)
        const double* b = &st.bp[3ll * p];
        for (int e : pr.point_edges[p]) {
            const double* Te = &st.T[27ll * e];
            double* r = &st.rhs[9ll * pr.oc[e]];
            for (int i = 0; i < 9; ++i) r[i] -= Te[3 * i] * b[0] + Te[3 * i + 1] * b[1] + Te[3 * i + 2] * b[2];
        }
    }
    for (int i = 0; i < n; ++i) st.rhs[i] += st.bc[i];
    for (int c = 0; c < C; ++c)  // damped U blocks (src/lm.cu:585-594)
        for (int i = 0; i < 9; ++i) {
            const double dg = st.U[81ll * c + 10 * i];
            for (int j = 0; j <= i; ++j) {
                double v = st.U[81ll * c + 9 * i + j];
                if (i == j) v += lambda * (dg > 0.0 ? dg : 1e-12);
                st.S[static_cast<size_t>(9 * c + j) * n + 9 * c + i] += v;
            }
        }
    return true;
}

// Factor, solve, back-substitute, gain denominator (src/lm.cu:598-643).
// Returns 2 = Cholesky failure, 3 = denom <= 0, 0 = ok.
int solve_step(const Problem& pr, State& st, double lambda, int threads, double* denom_out) {
    const int C = pr.C, P = pr.P, n = 9 * C;
    if (cholesky(st.S.data(), n, threads) != 0) return 2;  // src/lm.cu:598-603
    st.dc = st.rhs;
    cholesky_solve(st.S.data(), n, st.dc.data());
    double denom = 0.0;  // src/lm.cu:607-638
    for (int c = 0; c < C; ++c)
        for (int i = 0; i < 9; ++i) {
            const double dg = st.U[81ll * c + 10 * i];
            const double d = st.dc[9ll * c + i];
            denom += d * (lambda * (dg > 0.0 ? dg : 1e-12) * d + st.bc[9ll * c + i]);
        }
    st.dp.assign(3ll * P, 0.0);
    for (int p = 0; p < P; ++p) {
        double m[3] = {st.bp[3ll * p], st.bp[3ll * p + 1], st.bp[3ll * p + 2]};
        for (int e : pr.point_edges[p]) {
            const double* We = &st.W[27ll * e];
            const double* d = &st.dc[9ll * pr.oc[e]];
            for (int i = 0; i < 9; ++i)
                for (int j = 0; j < 3; ++j) m[j] -= We[3 * i + j] * d[i];
        }
        const double* Vi = &st.Vinv[9ll * p];
        for (int j = 0; j < 3; ++j) st.dp[3ll * p + j] = Vi[3 * j] * m[0] + Vi[3 * j + 1] * m[1] + Vi[3 * j + 2] * m[2];
        for (int j = 0; j < 3; ++j) {
            const double dg = st.V[9ll * p + 4 * j];
            const double d = st.dp[3ll * p + j];
            denom += d * (lambda * (dg > 0.0 ? dg : 1e-12) * d + st.bp[3ll * p + j]);
        }
    }
    *denom_out = denom;
    if (!(denom > 0.0)) return 3;
    return 0;
}

// Returns 1 = non-SPD V, 2 = Cholesky failure, 3 = denom <= 0, 0 = ok.
int schur_step(const Problem& pr, State& st, double lambda, int threads, double* denom_out) {
    if (!assemble(pr, st, lambda, threads)) return 1;
    return solve_step(pr, st, lambda, threads, denom_out);
}

Problem make_problem(int C, int P, int E, const int* oc, const int* op, const double* px) {
    Problem pr{C, P, E, oc, op, px, {}};
    pr.point_edges.assign(P, {});
    for (int e = 0; e < E; ++e) pr.point_edges[op[e]].push_back(e);
    return pr;
}

int default_threads() {
    const unsigned h = std::thread::hardware_concurrency();
    return h ? static_cast<int>(h) : 1;
}

}  // namespace

extern "C" {

int oracle_residual_jacobian(const double* cam, const double* pt, const double* obs, double* r, double* Jc, double* Jp) {
    residual_jacobian(cam, pt, obs, r, Jc, Jp);
    return 0;
}

int oracle_residual(const double* cam, const double* pt, const double* obs, double* r) {
    residual(cam, pt, obs, r);
    return 0;
}

// Normal equations in edge order. U 81C, V 9P (full), W 27E, bc 9C, bp 3P.
// The _robust variants take the Huber threshold (<= 0: plain squared loss);
// rows are scaled by the first-order corrector sqrt(rho'(s)) and the cost sums
// rho(s) = s (s <= d^2) or 2 d sqrt(s) - d^2 per observation.
int oracle_accumulate_robust(int C, int P, int E, const double* cams, const double* pts, const int* oc,
                             const int* op, const double* px, double huber_delta, double* U, double* V, double* W,
                             double* bc, double* bp, double* sse, unsigned long long* anomalies) {
    Problem pr = make_problem(C, P, E, oc, op, px);
    pr.delta = huber_delta;
    *anomalies = 0;
    accumulate(pr, cams, pts, U, V, W, bc, bp, sse, anomalies);
    return 0;
}

int oracle_accumulate(int C, int P, int E, const double* cams, const double* pts, const int* oc, const int* op,
                      const double* px, double* U, double* V, double* W, double* bc, double* bp, double* sse,
                      unsigned long long* anomalies) {
    Problem pr = make_problem(C, P, E, oc, op, px);
    *anomalies = 0;
    accumulate(pr, cams, pts, U, V, W, bc, bp, sse, anomalies);
    return 0;
}

double oracle_cost(int C, int P, int E, const double* cams, const double* pts, const int* oc, const int* op,
                   const double* px) {
    Problem pr = make_problem(C, P, E, oc, op, px);
    unsigned long long a = 0;
    return cost(pr, cams, pts, &a);
}

double oracle_cost_robust(int C, int P, int E, const double* cams, const double* pts, const int* oc, const int* op,
                          const double* px, double huber_delta) {
    Problem pr = make_problem(C, P, E, oc, op, px);
    pr.delta = huber_delta;
    unsigned long long a = 0;
    return cost(pr, cams, pts, &a);
}

// One damped Schur step at the given parameters: dc (9C), dp (3P), rhs (9C),
// the assembled S before factorisation (9C x 9C column-major, lower block
// triangle; may be NULL) and the gain denominator. Returns the schur_step status.
int oracle_schur_step(int C, int P, int E, const double* cams, const double* pts, const int* oc, const int* op,
                      const double* px, double lambda, int threads, double* dc, double* dp, double* rhs, double* S,
                      double* denom) {
    Problem pr = make_problem(C, P, E, oc, op, px);
    State st;
    st.U.resize(81ll * C);
    st.V.resize(9ll * P);
    st.W.resize(27ll * E);
    st.bc.resize(9ll * C);
    st.bp.resize(3ll * P);
    double sse = 0.0;
    unsigned long long a = 0;
    accumulate(pr, cams, pts, st.U.data(), st.V.data(), st.W.data(), st.bc.data(), st.bp.data(), &sse, &a);
    if (threads <= 0) threads = default_threads();
    if (!assemble(pr, st, lambda, threads)) return 1;
    if (S) std::memcpy(S, st.S.data(), st.S.size() * sizeof(double));
    if (rhs) std::memcpy(rhs, st.rhs.data(), 9ll * C * sizeof(double));
    double denom_v = 0.0;
    const int status = solve_step(pr, st, lambda, threads, &denom_v);
    if (denom) *denom = denom_v;
    if (status == 0 || status == 3) {
        if (dc) std::memcpy(dc, st.dc.data(), 9ll * C * sizeof(double));
        if (dp) std::memcpy(dp, st.dp.data(), 3ll * P * sizeof(double));
    }
    return status;
}

// Blocked Cholesky of a column-major n x n matrix in place (lower); 0 or the
// failed column. And the matching solve.
int oracle_cholesky(double* A, int n, int threads) { return cholesky(A, n, threads <= 0 ? default_threads() : threads); }
int oracle_cholesky_solve(const double* L, int n, double* b) {
    cholesky_solve(L, n, b);
    return 0;
}

// Full LM solve (src/lm.cu:371-724). cams/pts updated in place. termination:
// 0 CONVERGENCE, 1 MAX_ITERATIONS, 2 FAILURE. trajectory: cost at start and
// after every accepted iteration (up to traj_cap entries; *traj_len = count).
int oracle_solve_robust(int C, int P, int E, double* cams, double* pts, const int* oc, const int* op,
                        const double* px, double huber_delta, int max_iterations, double lambda0, double rel_tol,
                        int max_trials, int threads, double* initial_cost, double* final_cost, int* iterations,
                        int* termination, unsigned long long* anomalies_out, double* trajectory, int traj_cap,
                        int* traj_len) {
    if (threads <= 0) threads = default_threads();
    Problem pr = make_problem(C, P, E, oc, op, px);
    pr.delta = huber_delta;
    State st;
    st.U.resize(81ll * C);
    st.V.resize(9ll * P);
    st.W.resize(27ll * E);
    st.bc.resize(9ll * C);
    st.bp.resize(3ll * P);
    unsigned long long anomalies = 0;
    double sse = 0.0;
    accumulate(pr, cams, pts, st.U.data(), st.V.data(), st.W.data(), st.bc.data(), st.bp.data(), &sse, &anomalies);
    *initial_cost = sse / 2.0;
    int tl = 0;
    if (trajectory && tl < traj_cap) trajectory[tl] = sse / 2.0;
    ++tl;
    double lambda = lambda0;
    int iters = 0;
    bool converged = false, failed = false;
    double rel = 0.0;
    std::vector<double> tc(9ll * C), tp(3ll * P);
    while (iters < max_iterations && !converged && !failed) {
        double nu = 2.0;
        bool accepted = false;
        for (int trial = 0; trial < max_trials; ++trial) {
            double denom = 0.0;
            const int status = schur_step(pr, st, lambda, threads, &denom);
            if (status != 0) {
                lambda *= nu;
                nu *= 2.0;
                continue;
            }
            for (size_t i = 0; i < tc.size(); ++i) tc[i] = cams[i] + st.dc[i];
            for (size_t i = 0; i < tp.size(); ++i) tp[i] = pts[i] + st.dp[i];
            unsigned long long before = anomalies;
            const double trial_sse = cost(pr, tc.data(), tp.data(), &anomalies);
            if (anomalies != before || !std::isfinite(trial_sse)) {
                lambda *= nu;
                nu *= 2.0;
                continue;
            }
            const double rho = (sse - trial_sse) / (0.5 * denom);  // src/lm.cu:672
            if (rho > 0.0 && trial_sse < sse) {
                std::memcpy(cams, tc.data(), tc.size() * sizeof(double));
                std::memcpy(pts, tp.data(), tp.size() * sizeof(double));
                rel = (sse - trial_sse) / std::max(sse, 1.0);
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
        ++iters;
        if (trajectory && tl < traj_cap) trajectory[tl] = sse / 2.0;
        ++tl;
        if (rel < rel_tol) {
            converged = true;
            break;
        }
        double sse_acc = 0.0;  // the reference keeps the trial SSE (src/lm.cu:682,700-702)
        accumulate(pr, cams, pts, st.U.data(), st.V.data(), st.W.data(), st.bc.data(), st.bp.data(), &sse_acc,
                   &anomalies);
    }
    *final_cost = sse / 2.0;
    *iterations = iters;
    *termination = converged ? 0 : failed ? 2 : 1;
    *anomalies_out = anomalies;
    if (traj_len) *traj_len = tl;
    return 0;
}

int oracle_solve(int C, int P, int E, double* cams, double* pts, const int* oc, const int* op, const double* px,
                 int max_iterations, double lambda0, double rel_tol, int max_trials, int threads, double* initial_cost,
                 double* final_cost, int* iterations, int* termination, unsigned long long* anomalies_out,
                 double* trajectory, int traj_cap, int* traj_len) {
    return oracle_solve_robust(C, P, E, cams, pts, oc, op, px, 0.0, max_iterations, lambda0, rel_tol, max_trials,
                               threads, initial_cost, final_cost, iterations, termination, anomalies_out, trajectory,
                               traj_cap, traj_len);
}

}  // extern "C"
