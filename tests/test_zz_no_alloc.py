"""GPU: gba_cost_noalloc, the reprojection-cost entry point that allocates no
device memory, for callers whose device memory is owned by their own pool or
who must keep cudaMalloc / cudaFree (which synchronise the device) out of a
per-frame loop.

It is checked through the C ABI, on two calls in a row with different
parameters, against
  - the plain (all-FP64) form's cost kernel behind gba_solver_accumulate, which
    computes the same FP64 residuals with the solver's own allocated scratch,
    to 1e-12 relative (the two sum in different orders), and
  - the FP64 CPU oracle's cost (oracle.cost), to 1e-12 relative.
This file is collected last so that a failure here comes after every other
test has run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_cost_noalloc_matches_fp64_cost_on_two_calls(gba, oracle, torch_cuda):
    torch = torch_cuda
    prob = gba.synthetic_custom(12, 5000, 2, 8, 1.4, seed=41)
    prob.obs_pixel[7] = np.nan  # one non-finite residual, counted by all three
    dev = [torch.from_numpy(a.copy()).cuda() for a in prob.arrays()]
    out_sse = torch.zeros(1, dtype=torch.float64, device="cuda")
    out_bad = torch.zeros(1, dtype=torch.int64, device="cuda")
    rng = np.random.default_rng(5)
    cams, pts = prob.cameras.copy(), prob.points.copy()
    with gba.Solver(prob, "plain") as s:
        for call in range(2):
            if call == 1:
                cams = prob.cameras + rng.normal(0, 1e-3, prob.cameras.size)
                pts = prob.points + rng.normal(0, 1e-2, prob.points.size)
                s.set_params(cams, pts)
                dev[0].copy_(torch.from_numpy(cams))
                dev[1].copy_(torch.from_numpy(pts))
            a0 = s.counters()[0]
            ref_solver = s.accumulate()
            assert s.counters()[0] - a0 == 1
            ref_oracle = oracle.cost(prob, cams, pts)
            status = gba.lib.gba_cost_noalloc(*(t.data_ptr() for t in dev), prob.num_observations,
                                              out_sse.data_ptr(), out_bad.data_ptr(), None)
            assert status == 0, gba.lib.gba_last_error().decode()
            torch.cuda.synchronize()
            got = out_sse.item()
            assert abs(got - ref_solver) <= 1e-12 * abs(ref_solver), (call, got, ref_solver)
            assert abs(got - ref_oracle) <= 1e-12 * abs(ref_oracle), (call, got, ref_oracle)
            assert out_bad.item() == 1


def test_cost_noalloc_rejects_sizes_above_its_limit(gba):
    # rejected on the host before any device work
    status = gba.lib.gba_cost_noalloc(C.c_void_p(1), C.c_void_p(1), C.c_void_p(1), C.c_void_p(1), C.c_void_p(1),
                                      67108864 + 1, C.c_void_p(1), None, None)
    assert status == 1
    assert b"limit" in gba.lib.gba_last_error()
