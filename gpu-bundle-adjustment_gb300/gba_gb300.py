"""ctypes binding of libgba_gb300.so (the C ABI declared in include/gba_capi.h).

Host side of the library for Python callers (tests, bench): a BALProblem-like
container of numpy arrays, the whole-solve entry point, and the device stage
functions. Device buffers passed to the standalone kernels are raw addresses
(e.g. torch.Tensor.data_ptr()). The library is required: importing this
module fails loudly if libgba_gb300.so is missing, and nothing here computes
on the CPU.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libgba_gb300.so"

GBA_OK = 0
FORMS = {"plain": 0, "mixed": 1, "learned": 2}
LOSSES = {"none": 0, "huber": 1}
SCHUR_LAYOUTS = {"auto": 0, "dense": 1, "band": 2}
TERMINATION = {0: "CONVERGENCE", 1: "MAX_ITERATIONS", 2: "FAILURE", 3: "TARGET_COST"}
BUF = {
    "U": 0, "V": 1, "bc": 2, "bp": 3, "W": 4, "Vinv": 5, "S": 6, "rhs": 7, "dc": 8, "dp": 9,
    "order": 10, "Jc32": 11, "Sdiag": 12, "cams": 13, "pts": 14, "trial_cams": 15, "trial_pts": 16, "Jp32": 17,
}
_BUF_DTYPE = {"order": np.int32, "Jc32": np.float32, "Jp32": np.float32}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class GbaError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"gba status {status}: {msg}")
        self.status = status


class LMOptions(C.Structure):
    _fields_ = [
        ("max_iterations", C.c_int),
        ("initial_lambda", C.c_double),
        ("rel_decrease_tol", C.c_double),
        ("max_inner_trials", C.c_int),
        ("verbose", C.c_int),
        ("form", C.c_int),
        ("refine_tol", C.c_double),
        ("refine_max_steps", C.c_int),
        ("pcg_tol", C.c_double),
        ("pcg_max_iters", C.c_int),
        ("model_path", C.c_char_p),
        ("target_cost", C.c_double),
        ("stop_at_target", C.c_int),
        ("loss", C.c_int),
        ("huber_delta", C.c_double),
        ("schur_layout", C.c_int),
        ("deterministic", C.c_int),
    ]


class LMResultC(C.Structure):
    _fields_ = [
        ("initial_cost", C.c_double),
        ("final_cost", C.c_double),
        ("iterations", C.c_int),
        ("termination", C.c_int),
        ("anomalies", C.c_ulonglong),
        ("total_time_s", C.c_double),
        ("trials", C.c_int),
        ("pcg_iterations", C.c_longlong),
        ("refine_steps", C.c_int),
        ("time_to_target_s", C.c_double),
        ("t_setup", C.c_double),
        ("t_accumulate", C.c_double),
        ("t_damp", C.c_double),
        ("t_schur", C.c_double),
        ("t_backsub", C.c_double),
        ("t_cost", C.c_double),
        ("trajectory", _dp),
        ("trajectory_time_s", _dp),
        ("trajectory_capacity", C.c_int),
        ("trajectory_len", C.c_int),
        ("learned_choice", C.c_int),
        ("judge_iters_block_jacobi", C.c_longlong),
        ("judge_iters_learned", C.c_longlong),
        ("max_refine_residual", C.c_double),
        ("schur_band_rows", C.c_int),
    ]


def _load() -> C.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')"
        )
    return C.CDLL(str(LIB_PATH))


lib = _load()

_SIG = {
    "gba_last_error": (C.c_char_p, []),
    "gba_version": (C.c_char_p, []),
    "gba_lm_options_default": (None, [C.POINTER(LMOptions)]),
    "gba_solve_bal": (C.c_int, [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, C.POINTER(LMOptions),
                                C.POINTER(LMResultC)]),
    "gba_edge_residual_jacobian_host": (C.c_int, [_dp, _dp, _dp, _dp, _dp, _dp]),
    "gba_snavely_residual": (C.c_int, [_dp, _dp, _dp, _dp]),
    "gba_total_squared_error": (C.c_int, [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, _dp]),
    "gba_host_problem_load": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    "gba_host_problem_synthetic": (C.c_int, [C.c_int, C.c_uint64, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "gba_host_problem_synthetic_custom": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                                    C.c_double, C.c_uint64, C.POINTER(C.c_void_p)]),
    "gba_host_problem_synthetic_local": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int,
                                                   C.c_uint64, C.POINTER(C.c_void_p)]),
    "gba_host_problem_launch_bounds": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "gba_host_problem_dims": (C.c_int, [C.c_void_p, _ip, _ip, _ip]),
    "gba_host_problem_copy": (C.c_int, [C.c_void_p, _dp, _dp, _ip, _ip, _dp]),
    "gba_host_problem_save": (C.c_int, [C.c_void_p, C.c_char_p]),
    "gba_host_problem_free": (None, [C.c_void_p]),
    "gba_solver_create": (C.c_int, [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, C.c_int, C.c_void_p,
                                    C.POINTER(C.c_void_p)]),
    "gba_solver_destroy": (None, [C.c_void_p]),
    "gba_solver_set_params": (C.c_int, [C.c_void_p, _dp, _dp]),
    "gba_solver_get_params": (C.c_int, [C.c_void_p, _dp, _dp]),
    "gba_solver_accumulate": (C.c_int, [C.c_void_p, _dp]),
    "gba_solver_damp_invert_v": (C.c_int, [C.c_void_p, C.c_double, C.POINTER(C.c_ulonglong)]),
    "gba_solver_schur_dense": (C.c_int, [C.c_void_p, C.c_double, _ip]),
    "gba_solver_schur_pcg": (C.c_int, [C.c_void_p, C.c_double, C.POINTER(LMOptions), C.c_int,
                                       C.POINTER(C.c_longlong), _ip, _dp]),
    "gba_solver_back_substitute": (C.c_int, [C.c_void_p, C.c_double, _dp]),
    "gba_solver_trial_cost": (C.c_int, [C.c_void_p, _dp]),
    "gba_solver_accept": (C.c_int, [C.c_void_p]),
    "gba_solver_counters": (C.c_int, [C.c_void_p, C.POINTER(C.c_ulonglong), C.POINTER(C.c_ulonglong)]),
    "gba_solver_load_model": (C.c_int, [C.c_void_p, C.c_char_p]),
    "gba_solver_run": (C.c_int, [C.c_void_p, C.POINTER(LMOptions), C.POINTER(LMResultC)]),
    "gba_solver_reset_params": (C.c_int, [C.c_void_p]),
    "gba_solver_set_loss": (C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    "gba_solver_profile": (C.c_int, [C.c_void_p, C.c_int]),
    "gba_solver_kernel_stats": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_longlong), C.POINTER(C.c_double)]),
    "gba_solver_profile_reset": (C.c_int, [C.c_void_p]),
    "gba_launch_count": (C.c_ulonglong, []),
    "gba_release_cached_memory": (C.c_int, []),
    "gba_solver_set_harvest": (C.c_int, [C.c_void_p, C.c_int]),
    "gba_solver_features": (C.c_int, [C.c_void_p, C.c_double, C.c_void_p]),
    "gba_mlp_num_params": (C.c_longlong, []),
    "gba_mlp_create": (C.c_int, [C.c_uint64, C.c_int, C.POINTER(C.c_void_p)]),
    "gba_mlp_load": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_void_p)]),
    "gba_mlp_save": (C.c_int, [C.c_void_p, C.c_char_p]),
    "gba_mlp_destroy": (None, [C.c_void_p]),
    "gba_mlp_get_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "gba_mlp_set_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "gba_mlp_get_grads": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "gba_mlp_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "gba_mlp_backward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "gba_solver_set_preconditioner": (C.c_int, [C.c_void_p, C.c_int]),
    "gba_solver_set_schur_layout": (C.c_int, [C.c_void_p, C.c_int]),
    "gba_solver_set_matvec": (C.c_int, [C.c_void_p, C.c_int, _ip]),
    "gba_solver_schur_band": (C.c_int, [C.c_void_p, _ip, _ip, _ip]),
    "gba_band_potrf": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    "gba_band_potrs": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gba_solver_judge_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_double)]),
    "gba_mlp_adam_step": (C.c_int, [C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_float, C.c_void_p]),
    "gba_solver_buffer_size": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_size_t)]),
    "gba_solver_download": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t]),
    "gba_solver_device_ptr": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]),
    "gba_solver_dims": (C.c_int, [C.c_void_p, _ip, _ip, _ip, _ip]),
    "gba_batch_chol9_factor_solve": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                               C.c_void_p]),
    "gba_batch_inverse3_spd": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "gba_dense_potrf": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    "gba_dense_potrs": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gba_cost_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                   C.c_void_p, C.c_void_p]),
    "gba_eval_edges": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                 C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
}
for _name, (_res, _args) in _SIG.items():
    _f = getattr(lib, _name)
    _f.restype = _res
    _f.argtypes = _args

EXPORTED = tuple(_SIG)


def _check(status: int) -> None:
    if status != GBA_OK:
        raise GbaError(status, lib.gba_last_error().decode())


def _d(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _i(a: np.ndarray):
    return a.ctypes.data_as(_ip)


@dataclass
class BALProblem:
    """Mirror of gba::BALProblem (BAL structure-of-arrays layout)."""

    cameras: np.ndarray  # (9C,) float64
    points: np.ndarray  # (3P,) float64
    obs_camera: np.ndarray  # (E,) int32
    obs_point: np.ndarray  # (E,) int32
    obs_pixel: np.ndarray  # (2E,) float64

    @property
    def num_cameras(self) -> int:
        return self.cameras.size // 9

    @property
    def num_points(self) -> int:
        return self.points.size // 3

    @property
    def num_observations(self) -> int:
        return self.obs_camera.size

    def copy(self) -> "BALProblem":
        return BALProblem(*(a.copy() for a in (self.cameras, self.points, self.obs_camera, self.obs_point,
                                                 self.obs_pixel)))

    def arrays(self):
        return self.cameras, self.points, self.obs_camera, self.obs_point, self.obs_pixel


def _from_handle(h: C.c_void_p) -> BALProblem:
    c, p, e = C.c_int(), C.c_int(), C.c_int()
    _check(lib.gba_host_problem_dims(h, C.byref(c), C.byref(p), C.byref(e)))
    prob = BALProblem(
        np.empty(9 * c.value), np.empty(3 * p.value), np.empty(e.value, np.int32), np.empty(e.value, np.int32),
        np.empty(2 * e.value),
    )
    _check(lib.gba_host_problem_copy(h, _d(prob.cameras), _d(prob.points), _i(prob.obs_camera),
                                     _i(prob.obs_point), _d(prob.obs_pixel)))
    lib.gba_host_problem_free(h)
    return prob


def synthetic(workload: int, seed: int | None = None, with_truth: bool = False):
    """Seeded synthetic workload 1..5 (seed defaults to the workload id)."""
    h, t = C.c_void_p(), C.c_void_p()
    _check(lib.gba_host_problem_synthetic(workload, workload if seed is None else seed, C.byref(h),
                                          C.byref(t) if with_truth else None))
    prob = _from_handle(h)
    return (prob, _from_handle(t)) if with_truth else prob


def synthetic_custom(num_cameras: int, num_points: int, track_min: int = 2, track_max: int = 8,
                     alpha: float = 1.29, outlier_fraction: float = 0.0, outlier_sigma: float = 0.0,
                     seed: int = 1) -> BALProblem:
    h = C.c_void_p()
    _check(lib.gba_host_problem_synthetic_custom(num_cameras, num_points, track_min, track_max, alpha,
                                                 outlier_fraction, outlier_sigma, seed, C.byref(h)))
    return _from_handle(h)


def synthetic_local(num_cameras: int, num_points: int, track_min: int = 2, track_max: int = 8,
                    alpha: float = 1.5, window: int = 10, seed: int = 1) -> BALProblem:
    """Seeded problem with spatially local covisibility: the camera graph is a band of half-width ~window."""
    h = C.c_void_p()
    _check(lib.gba_host_problem_synthetic_local(num_cameras, num_points, track_min, track_max, alpha, window, seed,
                                                C.byref(h)))
    return _from_handle(h)


def launch_bounds_problem(num_points: int = 400000) -> BALProblem:
    h = C.c_void_p()
    _check(lib.gba_host_problem_launch_bounds(num_points, C.byref(h)))
    return _from_handle(h)


def load_bal(path: str | os.PathLike) -> BALProblem:
    h = C.c_void_p()
    _check(lib.gba_host_problem_load(str(path).encode(), C.byref(h)))
    return _from_handle(h)


def total_squared_error(prob: BALProblem) -> float:
    out = C.c_double()
    _check(lib.gba_total_squared_error(prob.num_cameras, prob.num_points, prob.num_observations,
                                       _d(prob.cameras), _d(prob.points), _i(prob.obs_camera), _i(prob.obs_point),
                                       _d(prob.obs_pixel), C.byref(out)))
    return out.value


def snavely_residual(cam, pt, obs) -> np.ndarray:
    cam, pt, obs = (np.ascontiguousarray(x, np.float64) for x in (cam, pt, obs))
    out = np.empty(2)
    _check(lib.gba_snavely_residual(_d(cam), _d(pt), _d(obs), _d(out)))
    return out


def edge_residual_jacobian_host(cam, pt, obs):
    cam, pt, obs = (np.ascontiguousarray(x, np.float64) for x in (cam, pt, obs))
    r, jc, jp = np.empty(2), np.empty(18), np.empty(6)
    _check(lib.gba_edge_residual_jacobian_host(_d(cam), _d(pt), _d(obs), _d(r), _d(jc), _d(jp)))
    return r, jc.reshape(2, 9), jp.reshape(2, 3)


def default_options(**kw) -> LMOptions:
    o = LMOptions()
    lib.gba_lm_options_default(C.byref(o))
    for k, v in kw.items():
        if k == "form":
            v = FORMS[v] if isinstance(v, str) else v
        if k == "loss":
            v = LOSSES[v] if isinstance(v, str) else v
        if k == "schur_layout":
            v = SCHUR_LAYOUTS[v] if isinstance(v, str) else v
        if k == "model_path" and v is not None:
            v = str(v).encode()
        setattr(o, k, v)
    return o


@dataclass
class LMResult:
    initial_cost: float
    final_cost: float
    iterations: int
    termination: str
    anomalies: int
    total_time_s: float
    trials: int
    pcg_iterations: int
    refine_steps: int
    time_to_target_s: float
    phases: dict
    trajectory: list = field(default_factory=list)
    trajectory_time_s: list = field(default_factory=list)
    learned_choice: int = 0  # learned form: 1 learned, 2 block-Jacobi won the judged first inner solve
    judge_iters: tuple = (0, 0)  # that solve's inner PCG iterations: (block-Jacobi, learned)
    max_refine_residual: float = 0.0  # mixed forms: largest relative residual of a refined Schur step
    schur_band_rows: int = 0  # plain form: rows of the band S was stored in (0: dense)


def _result_struct(cap: int):
    traj, ttime = np.zeros(cap), np.zeros(cap)
    r = LMResultC()
    r.trajectory = _d(traj)
    r.trajectory_time_s = _d(ttime)
    r.trajectory_capacity = cap
    return r, traj, ttime


def _to_result(r, traj, ttime, cap) -> "LMResult":
    n = min(r.trajectory_len, cap)
    return LMResult(
        r.initial_cost, r.final_cost, r.iterations, TERMINATION[r.termination], r.anomalies, r.total_time_s,
        r.trials, r.pcg_iterations, r.refine_steps, r.time_to_target_s,
        dict(setup=r.t_setup, accumulate=r.t_accumulate, damp=r.t_damp, schur=r.t_schur, backsub=r.t_backsub,
             cost=r.t_cost),
        traj[:n].tolist(), ttime[:n].tolist(), r.learned_choice,
        (r.judge_iters_block_jacobi, r.judge_iters_learned), r.max_refine_residual, r.schur_band_rows,
    )


def release_cached_memory() -> None:
    """Return the device memory the solvers' pool keeps between solves to the driver."""
    _check(lib.gba_release_cached_memory())


def launch_count() -> int:
    """Kernels launched by libgba_gb300 in this process so far."""
    return int(lib.gba_launch_count())


def solve(prob: BALProblem, **opts) -> LMResult:
    """gba::solve_bal_gpu through the C ABI: updates prob.cameras / prob.points in place."""
    o = default_options(**opts)
    cap = max(8, o.max_iterations + 2)
    r, traj, ttime = _result_struct(cap)
    for a, dt in ((prob.cameras, np.float64), (prob.points, np.float64), (prob.obs_camera, np.int32),
                  (prob.obs_point, np.int32), (prob.obs_pixel, np.float64)):
        if a.dtype != dt or not a.flags.c_contiguous:
            raise TypeError("BALProblem arrays must be contiguous float64 / int32")
    _check(lib.gba_solve_bal(prob.num_cameras, prob.num_points, prob.num_observations, _d(prob.cameras),
                             _d(prob.points), _i(prob.obs_camera), _i(prob.obs_point), _d(prob.obs_pixel),
                             C.byref(o), C.byref(r)))
    return _to_result(r, traj, ttime, cap)


def solve_raw(num_cameras: int, num_points: int, num_observations: int, cams: int, pts: int, oc: int, op: int,
              px: int, **opts) -> LMResult:
    """gba_solve_bal on raw host addresses (e.g. pinned torch tensors' data_ptr())."""
    o = default_options(**opts)
    cap = max(8, o.max_iterations + 2)
    r, traj, ttime = _result_struct(cap)
    _check(lib.gba_solve_bal(num_cameras, num_points, num_observations, C.cast(cams, _dp), C.cast(pts, _dp),
                             C.cast(oc, _ip), C.cast(op, _ip), C.cast(px, _dp), C.byref(o), C.byref(r)))
    return _to_result(r, traj, ttime, cap)


class Solver:
    """Device-resident LM state (gba_solver); each method is one LM stage."""

    def __init__(self, prob: BALProblem, form: str = "plain", stream: int | None = None):
        self.prob = prob
        self.form = form
        h = C.c_void_p()
        _check(lib.gba_solver_create(prob.num_cameras, prob.num_points, prob.num_observations, _d(prob.cameras),
                                     _d(prob.points), _i(prob.obs_camera), _i(prob.obs_point), _d(prob.obs_pixel),
                                     FORMS[form], C.c_void_p(stream) if stream else None, C.byref(h)))
        self.h = h

    def close(self) -> None:
        if self.h:
            lib.gba_solver_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def dims(self):
        c, p, e, n = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _check(lib.gba_solver_dims(self.h, C.byref(c), C.byref(p), C.byref(e), C.byref(n)))
        return c.value, p.value, e.value, n.value

    def set_params(self, cams: np.ndarray, pts: np.ndarray) -> None:
        _check(lib.gba_solver_set_params(self.h, _d(np.ascontiguousarray(cams, np.float64)),
                                         _d(np.ascontiguousarray(pts, np.float64))))

    def get_params(self):
        cams, pts = np.empty(9 * self.prob.num_cameras), np.empty(3 * self.prob.num_points)
        _check(lib.gba_solver_get_params(self.h, _d(cams), _d(pts)))
        return cams, pts

    def accumulate(self) -> float:
        v = C.c_double()
        _check(lib.gba_solver_accumulate(self.h, C.byref(v)))
        return v.value

    def damp_invert_v(self, lam: float) -> int:
        v = C.c_ulonglong()
        _check(lib.gba_solver_damp_invert_v(self.h, lam, C.byref(v)))
        return v.value

    def schur_dense(self, lam: float) -> int:
        v = C.c_int()
        _check(lib.gba_solver_schur_dense(self.h, lam, C.byref(v)))
        return v.value

    def schur_pcg(self, lam: float, learned: bool = False, **opts):
        o = default_options(**opts)
        it, steps, rr = C.c_longlong(), C.c_int(), C.c_double()
        _check(lib.gba_solver_schur_pcg(self.h, lam, C.byref(o), int(learned), C.byref(it), C.byref(steps),
                                        C.byref(rr)))
        return it.value, steps.value, rr.value

    def back_substitute(self, lam: float) -> float:
        v = C.c_double()
        _check(lib.gba_solver_back_substitute(self.h, lam, C.byref(v)))
        return v.value

    def trial_cost(self) -> float:
        v = C.c_double()
        _check(lib.gba_solver_trial_cost(self.h, C.byref(v)))
        return v.value

    def accept(self) -> None:
        _check(lib.gba_solver_accept(self.h))

    def counters(self):
        a, n = C.c_ulonglong(), C.c_ulonglong()
        _check(lib.gba_solver_counters(self.h, C.byref(a), C.byref(n)))
        return a.value, n.value

    def load_model(self, path) -> None:
        _check(lib.gba_solver_load_model(self.h, str(path).encode()))

    def run(self, **opts) -> LMResult:
        """Full LM loop on the device-resident problem from the current parameters."""
        opts.setdefault("form", self.form)
        o = default_options(**opts)
        cap = max(8, o.max_iterations + 2)
        r, traj, ttime = _result_struct(cap)
        _check(lib.gba_solver_run(self.h, C.byref(o), C.byref(r)))
        return _to_result(r, traj, ttime, cap)

    def reset_params(self) -> None:
        _check(lib.gba_solver_reset_params(self.h))

    def set_preconditioner(self, mode: str = "judge") -> None:
        """Learned form: "judge" (default), "learned" (always) or "block-jacobi" (never learned)."""
        _check(lib.gba_solver_set_preconditioner(self.h, {"judge": 0, "learned": 1, "block-jacobi": 2}[mode]))

    def set_matvec(self, mode: str = "auto") -> bool:
        """Mixed forms: the FP32 PCG product, "auto", "two-pass", "one-pass" or "query";
        returns whether the one-pass product is in use."""
        v = C.c_int()
        _check(lib.gba_solver_set_matvec(self.h, {"query": -1, "auto": 0, "two-pass": 1, "one-pass": 2}[mode],
                                         C.byref(v)))
        return bool(v.value)

    def set_schur_layout(self, layout: str = "auto") -> None:
        """Plain form: storage of S, "auto", "dense" or "band" (from the next schur_dense on)."""
        _check(lib.gba_solver_set_schur_layout(self.h, SCHUR_LAYOUTS[layout]))

    def schur_band(self):
        """After schur_dense: (ldb, bt, perm) of the band S is stored in; (0, 0, None) when dense."""
        ldb, bt = C.c_int(), C.c_int()
        _check(lib.gba_solver_schur_band(self.h, C.byref(ldb), C.byref(bt), None))
        if ldb.value == 0:
            return 0, 0, None
        perm = np.empty(self.dims()[0], np.int32)
        _check(lib.gba_solver_schur_band(self.h, None, None, perm.ctypes.data_as(_ip)))
        return ldb.value, bt.value, perm

    def judge_info(self):
        """Last judged solve: ((block-Jacobi, learned) PCG iterations, (block-Jacobi, learned) b.x)."""
        it, bx = (C.c_longlong * 2)(), (C.c_double * 2)()
        _check(lib.gba_solver_judge_info(self.h, it, bx))
        return (it[0], it[1]), (bx[0], bx[1])

    def set_loss(self, loss: str = "none", delta: float = 1.0) -> None:
        _check(lib.gba_solver_set_loss(self.h, LOSSES[loss], delta))

    def profile(self, enable: bool = True) -> None:
        _check(lib.gba_solver_profile(self.h, int(enable)))

    def kernel_stats(self, name: str):
        n, ms = C.c_longlong(), C.c_double()
        _check(lib.gba_solver_kernel_stats(self.h, name.encode(), C.byref(n), C.byref(ms)))
        return n.value, ms.value

    def profile_reset(self) -> None:
        _check(lib.gba_solver_profile_reset(self.h))

    def download(self, name: str) -> np.ndarray:
        bid = BUF[name]
        size = C.c_size_t()
        _check(lib.gba_solver_buffer_size(self.h, bid, C.byref(size)))
        dt = _BUF_DTYPE.get(name, np.float64)
        out = np.empty(size.value // np.dtype(dt).itemsize, dt)
        if size.value:
            _check(lib.gba_solver_download(self.h, bid, out.ctypes.data_as(C.c_void_p), size.value))
        return out

    def device_ptr(self, name: str) -> int:
        p = C.c_void_p()
        _check(lib.gba_solver_device_ptr(self.h, BUF[name], C.byref(p)))
        return p.value or 0


# ---- standalone kernels on device addresses (e.g. torch.Tensor.data_ptr()) ----

def batch_chol9_factor_solve(A: int, b: int, x: int, ok: int, n: int, stream: int = 0) -> None:
    _check(lib.gba_batch_chol9_factor_solve(A, b, x, ok, n, stream or None))


def batch_inverse3_spd(A: int, Ainv: int, ok: int, n: int, stream: int = 0) -> None:
    _check(lib.gba_batch_inverse3_spd(A, Ainv, ok, n, stream or None))


def dense_potrf(A: int, n: int, lda: int, info: int, stream: int = 0) -> None:
    _check(lib.gba_dense_potrf(A, n, lda, info, stream or None))


def dense_potrs(L: int, n: int, lda: int, b: int, info: int, stream: int = 0) -> None:
    _check(lib.gba_dense_potrs(L, n, lda, b, info, stream or None))


def band_potrf(AB: int, n: int, ldb: int, bt: int, info: int, stream: int = 0) -> None:
    _check(lib.gba_band_potrf(AB, n, ldb, bt, info, stream or None))


def band_potrs(LB: int, n: int, ldb: int, bt: int, b: int, info: int, stream: int = 0) -> None:
    _check(lib.gba_band_potrs(LB, n, ldb, bt, b, info, stream or None))


def eval_edges(precision: int, cams: int, pts: int, oc: int, op: int, px: int, E: int, r: int, Jc: int = 0,
               Jp: int = 0, stream: int = 0) -> None:
    _check(lib.gba_eval_edges(precision, cams, pts, oc, op, px, E, r, Jc or None, Jp or None, stream or None))


def solver_set_harvest(solver: "Solver", enable: bool = True) -> None:
    _check(lib.gba_solver_set_harvest(solver.h, int(enable)))


def solver_features(solver: "Solver", lam: float, feat_dev: int) -> None:
    """Features of the solver's current S_cc blocks into a device buffer (C x 64 float)."""
    _check(lib.gba_solver_features(solver.h, lam, feat_dev))


class Mlp:
    """The learned coarse-basis network (gba_mlp): per-camera features (64) -> 96 outputs,
    the first 81 of which are the camera's 9 x 9 rows of the coarse basis (row-major)."""

    NUM_PARAMS = int(lib.gba_mlp_num_params())
    N_IN, N_OUT, N_USED_OUT, K = 64, 96, 81, 9

    def __init__(self, seed: int = 0, capacity: int = 4096, path=None):
        h = C.c_void_p()
        if path is not None:
            _check(lib.gba_mlp_load(str(path).encode(), capacity, C.byref(h)))
        else:
            _check(lib.gba_mlp_create(seed, capacity, C.byref(h)))
        self.h = h

    def close(self) -> None:
        if self.h:
            lib.gba_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def save(self, path) -> None:
        _check(lib.gba_mlp_save(self.h, str(path).encode()))

    def params(self) -> np.ndarray:
        out = np.empty(self.NUM_PARAMS, np.float32)
        _check(lib.gba_mlp_get_params(self.h, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        _check(lib.gba_mlp_set_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float))))

    def grads(self) -> np.ndarray:
        out = np.empty(self.NUM_PARAMS, np.float32)
        _check(lib.gba_mlp_get_grads(self.h, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def forward(self, feat_dev: int, batch: int, out_dev: int, stream: int = 0) -> None:
        _check(lib.gba_mlp_forward(self.h, feat_dev, batch, out_dev, stream or None))

    def backward(self, feat_dev: int, d_out_dev: int, batch: int, stream: int = 0) -> None:
        """Parameter gradients from d(loss)/d(outputs) of the last forward on feat_dev."""
        _check(lib.gba_mlp_backward(self.h, feat_dev, d_out_dev, batch, stream or None))

    def adam_step(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8,
                  stream: int = 0) -> None:
        _check(lib.gba_mlp_adam_step(self.h, lr, beta1, beta2, eps, stream or None))
