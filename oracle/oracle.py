"""ORACLE (test infrastructure only): ctypes access to the CPU restatement of
the reference LM (liboracle.so), to the reference's own compiled BAL reader
(_ref/libgba_ref_reader.so) and to the reference's own LM driver run on the
CPU (_ref/libgba_ref_lm_host.so: src/lm.cu compiled unmodified against the
Eigen stand-in, its kernels executed by the CPU stand-in for the CUDA
runtime). The _ref libraries exist only where the reference checkout was
available at build time. Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg use this module, as the checker.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from build_oracle import ORACLE_SO, REF_SO, build_oracle, build_reference_lm, build_reference_reader

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


build_oracle()
_lib = C.CDLL(str(ORACLE_SO))
_lib.oracle_residual_jacobian.argtypes = [_dp] * 6
_lib.oracle_residual.argtypes = [_dp] * 4
_lib.oracle_accumulate.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                                   C.POINTER(C.c_ulonglong)]
_lib.oracle_cost.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp]
_lib.oracle_cost.restype = C.c_double
_lib.oracle_accumulate_robust.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, C.c_double, _dp, _dp,
                                          _dp, _dp, _dp, _dp, C.POINTER(C.c_ulonglong)]
_lib.oracle_cost_robust.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, C.c_double]
_lib.oracle_cost_robust.restype = C.c_double
_lib.oracle_schur_step.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, C.c_double, C.c_int, _dp,
                                   _dp, _dp, _dp, _dp]
_lib.oracle_cholesky.argtypes = [_dp, C.c_int, C.c_int]
_lib.oracle_cholesky_solve.argtypes = [_dp, C.c_int, _dp]
_lib.oracle_solve.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, C.c_int, C.c_double, C.c_double,
                              C.c_int, C.c_int, _dp, _dp, _ip, _ip, C.POINTER(C.c_ulonglong), _dp, C.c_int, _ip]
_lib.oracle_solve_robust.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, C.c_double, C.c_int,
                                     C.c_double, C.c_double, C.c_int, C.c_int, _dp, _dp, _ip, _ip,
                                     C.POINTER(C.c_ulonglong), _dp, C.c_int, _ip]

_lib.oracle_synthetic.argtypes = [C.c_int, C.c_ulonglong, _ip, _ip, _ip]
_lib.oracle_synthetic_copy.argtypes = [_dp, _dp, _ip, _ip, _dp]

TERMINATION = {0: "CONVERGENCE", 1: "MAX_ITERATIONS", 2: "FAILURE"}


class Problem:
    """BAL-layout arrays (the fields of gba::BALProblem) for the oracle's own use."""

    def __init__(self, cameras, points, obs_camera, obs_point, obs_pixel):
        self.cameras, self.points = cameras, points
        self.obs_camera, self.obs_point, self.obs_pixel = obs_camera, obs_point, obs_pixel

    num_cameras = property(lambda self: self.cameras.size // 9)
    num_points = property(lambda self: self.points.size // 3)
    num_observations = property(lambda self: self.obs_camera.size)

    def arrays(self):
        return self.cameras, self.points, self.obs_camera, self.obs_point, self.obs_pixel


def synthetic(workload: int, seed: int | None = None) -> Problem:
    """Seeded workload 1..5 from the oracle's own generator (bit-identical to the product's)."""
    c, p, e = C.c_int(), C.c_int(), C.c_int()
    if _lib.oracle_synthetic(workload, workload if seed is None else seed, C.byref(c), C.byref(p), C.byref(e)):
        raise ValueError("workload id must be 1..5")
    prob = Problem(np.empty(9 * c.value), np.empty(3 * p.value), np.empty(e.value, np.int32),
                   np.empty(e.value, np.int32), np.empty(2 * e.value))
    _lib.oracle_synthetic_copy(_d(prob.cameras), _d(prob.points), _i(prob.obs_camera), _i(prob.obs_point),
                               _d(prob.obs_pixel))
    return prob


def residual_jacobian(cam, pt, obs):
    cam, pt, obs = (np.ascontiguousarray(x, np.float64) for x in (cam, pt, obs))
    r, jc, jp = np.empty(2), np.empty(18), np.empty(6)
    _lib.oracle_residual_jacobian(_d(cam), _d(pt), _d(obs), _d(r), _d(jc), _d(jp))
    return r, jc.reshape(2, 9), jp.reshape(2, 3)


def residual(cam, pt, obs):
    cam, pt, obs = (np.ascontiguousarray(x, np.float64) for x in (cam, pt, obs))
    r = np.empty(2)
    _lib.oracle_residual(_d(cam), _d(pt), _d(obs), _d(r))
    return r


def _args(prob):
    return (prob.num_cameras, prob.num_points, prob.num_observations)


def accumulate(prob, cams=None, pts=None, huber_delta=0.0):
    """Normal equations in observation order: dict U (C,9,9), V (P,3,3), W (E,9,3), bc, bp, sse, anomalies.

    huber_delta > 0 applies the Huber loss (rows scaled by sqrt(rho'), sse = sum of rho)."""
    C_, P_, E_ = _args(prob)
    cams = prob.cameras if cams is None else cams
    pts = prob.points if pts is None else pts
    U, V, W = np.empty(81 * C_), np.empty(9 * P_), np.empty(27 * E_)
    bc, bp, sse, an = np.empty(9 * C_), np.empty(3 * P_), np.empty(1), C.c_ulonglong()
    _lib.oracle_accumulate_robust(C_, P_, E_, _d(cams), _d(pts), _i(prob.obs_camera), _i(prob.obs_point),
                                  _d(prob.obs_pixel), float(huber_delta), _d(U), _d(V), _d(W), _d(bc), _d(bp),
                                  _d(sse), C.byref(an))
    return dict(U=U.reshape(C_, 9, 9), V=V.reshape(P_, 3, 3), W=W.reshape(E_, 9, 3), bc=bc, bp=bp, sse=sse[0],
                anomalies=an.value)


def cost(prob, cams=None, pts=None, huber_delta=0.0) -> float:
    """Sum over observations of rho(|r|^2) (plain squared error when huber_delta <= 0)."""
    cams = prob.cameras if cams is None else cams
    pts = prob.points if pts is None else pts
    return _lib.oracle_cost_robust(*_args(prob), _d(cams), _d(pts), _i(prob.obs_camera), _i(prob.obs_point),
                                   _d(prob.obs_pixel), float(huber_delta))


def schur_step(prob, lam, threads=0, want_S=False):
    C_, P_, E_ = _args(prob)
    dc, dp, rhs, den = np.zeros(9 * C_), np.zeros(3 * P_), np.zeros(9 * C_), np.zeros(1)
    S = np.zeros((9 * C_) * (9 * C_)) if want_S else None
    st = _lib.oracle_schur_step(C_, P_, E_, _d(prob.cameras), _d(prob.points), _i(prob.obs_camera),
                                _i(prob.obs_point), _d(prob.obs_pixel), lam, threads, _d(dc), _d(dp), _d(rhs),
                                _d(S) if want_S else None, _d(den))
    out = dict(status=st, dc=dc, dp=dp, rhs=rhs, denom=den[0])
    if want_S:
        out["S"] = S.reshape(9 * C_, 9 * C_).T  # column-major -> row-major view (lower triangle filled)
    return out


def cholesky(A_colmajor: np.ndarray, n: int, threads: int = 0) -> int:
    return _lib.oracle_cholesky(_d(A_colmajor), n, threads)


def solve(prob, max_iterations=50, initial_lambda=1e-3, rel_decrease_tol=1e-6, max_inner_trials=16, threads=0,
          huber_delta=0.0):
    """Full LM solve on copies of the parameters; returns (result dict, cams, pts)."""
    C_, P_, E_ = _args(prob)
    cams, pts = prob.cameras.copy(), prob.points.copy()
    init, fin, it, term = C.c_double(), C.c_double(), C.c_int(), C.c_int()
    an, tl = C.c_ulonglong(), C.c_int()
    cap = max_iterations + 2
    traj = np.zeros(cap)
    _lib.oracle_solve_robust(C_, P_, E_, _d(cams), _d(pts), _i(prob.obs_camera), _i(prob.obs_point),
                             _d(prob.obs_pixel), float(huber_delta), max_iterations, initial_lambda,
                             rel_decrease_tol, max_inner_trials, threads, C.byref(init), C.byref(fin), C.byref(it),
                             C.byref(term), C.byref(an), _d(traj), cap, C.byref(tl))
    res = dict(initial_cost=init.value, final_cost=fin.value, iterations=it.value,
               termination=TERMINATION[term.value], anomalies=an.value, trajectory=traj[:min(tl.value, cap)].tolist())
    return res, cams, pts


class ReferenceReader:
    """The reference's own src/bal_reader.cpp (compiled from source) via ctypes."""

    def __init__(self):
        path = build_reference_reader()
        if path is None or not Path(path).exists():
            raise FileNotFoundError("reference BAL reader not built (reference checkout unavailable)")
        self.lib = C.CDLL(str(path))
        self.lib.ref_snavely_residual.argtypes = [_dp] * 4
        self.lib.ref_total_squared_error.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp]
        self.lib.ref_total_squared_error.restype = C.c_double
        self.lib.ref_load_bal_dims.argtypes = [C.c_char_p, _ip, _ip, _ip]
        self.lib.ref_load_bal.argtypes = [C.c_char_p, _dp, _dp, _ip, _ip, _dp]

    def snavely_residual(self, cam, pt, obs):
        cam, pt, obs = (np.ascontiguousarray(x, np.float64) for x in (cam, pt, obs))
        out = np.empty(2)
        self.lib.ref_snavely_residual(_d(cam), _d(pt), _d(obs), _d(out))
        return out

    def total_squared_error(self, prob) -> float:
        return self.lib.ref_total_squared_error(*_args(prob), _d(prob.cameras), _d(prob.points),
                                                _i(prob.obs_camera), _i(prob.obs_point), _d(prob.obs_pixel))

    def load_bal(self, path):
        c, p, e = C.c_int(), C.c_int(), C.c_int()
        if self.lib.ref_load_bal_dims(str(path).encode(), C.byref(c), C.byref(p), C.byref(e)) != 0:
            raise ValueError("reference load_bal rejected " + str(path))
        arrs = (np.empty(9 * c.value), np.empty(3 * p.value), np.empty(e.value, np.int32), np.empty(e.value, np.int32),
                np.empty(2 * e.value))
        self.lib.ref_load_bal(str(path).encode(), _d(arrs[0]), _d(arrs[1]), _i(arrs[2]), _i(arrs[3]), _d(arrs[4]))
        return arrs


class ReferenceLM:
    """The reference's own LM driver, gba::solve_bal_gpu (src/lm.cu:371-724,
    compiled unmodified), run on the CPU: its host code (S assembly, LLT,
    back-substitution, gain ratio, damping, termination) is the reference's;
    its three kernels run as CPU restatements inside the CUDA-runtime stand-in
    (oracle/ref_host_runtime.cpp). The per-iteration cost trajectory is
    recovered at full precision from the stand-in's launch log: an accepted
    trial is a cost launch followed by a re-accumulation (edge launch)."""

    EDGE, COST, DAMP = 1, 2, 3

    def __init__(self):
        path = build_reference_lm()
        if path is None or not Path(path).exists():
            raise FileNotFoundError("reference LM driver not built (reference checkout unavailable)")
        self.lib = C.CDLL(str(path))
        self.lib.gba_ref_solve_bal.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, C.c_int,
                                               C.c_double, C.c_double, C.c_int, C.c_int, _dp, _dp, _ip, _ip,
                                               C.POINTER(C.c_ulonglong), _dp, C.c_char_p, C.c_int]
        self.lib.gba_ref_events.argtypes = [C.c_int, _ip, _dp, C.POINTER(C.c_ulonglong)]
        self.lib.gba_ref_events.restype = C.c_int
        self.lib.gba_ref_events_clear.argtypes = []

    def _events(self):
        n = self.lib.gba_ref_events(0, None, None, None)
        kinds, sse, cnt = np.zeros(n, np.int32), np.zeros(n), np.zeros(n, np.uint64)
        self.lib.gba_ref_events(n, _i(kinds), _d(sse), cnt.ctypes.data_as(C.POINTER(C.c_ulonglong)))
        return kinds, sse, cnt

    def solve(self, prob, max_iterations=50, initial_lambda=1e-3, rel_decrease_tol=1e-6, max_inner_trials=16):
        """Full solve on copies of the parameters; returns (result dict, cams, pts)."""
        C_, P_, E_ = _args(prob)
        cams, pts = prob.cameras.copy(), prob.points.copy()
        init, fin, tt = C.c_double(), C.c_double(), C.c_double()
        it, term, an = C.c_int(), C.c_int(), C.c_ulonglong()
        err = C.create_string_buffer(512)
        self.lib.gba_ref_events_clear()
        st = self.lib.gba_ref_solve_bal(C_, P_, E_, _d(cams), _d(pts), _i(prob.obs_camera), _i(prob.obs_point),
                                        _d(prob.obs_pixel), max_iterations, initial_lambda, rel_decrease_tol,
                                        max_inner_trials, 0, C.byref(init), C.byref(fin), C.byref(it),
                                        C.byref(term), C.byref(an), C.byref(tt), err, len(err))
        if st != 0:
            raise RuntimeError("reference solve_bal_gpu threw: " + err.value.decode())
        kinds, sse, _ = self._events()
        traj = [init.value]
        pending = None
        for k, s in zip(kinds[1:], sse[1:]):
            if k == self.COST:
                pending = s / 2.0
            elif k == self.EDGE and pending is not None:
                traj.append(pending)
                pending = None
        if len(traj) == it.value:  # the last accepted step ended the solve without a re-accumulation
            traj.append(fin.value)
        res = dict(initial_cost=init.value, final_cost=fin.value, iterations=it.value,
                   termination={0: "CONVERGENCE", 1: "MAX_ITERATIONS", 2: "FAILURE"}.get(term.value, "?"),
                   anomalies=an.value, trajectory=traj, trials=int(np.sum(kinds == self.DAMP)),
                   total_time_s=tt.value)
        return res, cams, pts
