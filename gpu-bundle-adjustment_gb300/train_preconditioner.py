"""Trains the learned coarse-space correction of block-Jacobi PCG on the GPU with
this library's own MLP kernels (gba_mlp_forward / gba_mlp_backward /
gba_mlp_adam_step), from reduced camera systems that the plain FP64 solver
assembles.

  python train_preconditioner.py [--out models/coarse_mlp.bin] [--epochs 300]

Why a coarse space: the Jacobi-preconditioned reduced camera system
B^-1/2 S B^-T/2 (B the 9x9 diagonal blocks) has a handful of eigenvalues far
below the rest: the 7-dimensional similarity gauge of bundle adjustment (only
the LM damping holds it) and a few soft modes. They set block-Jacobi PCG's
iteration count at tight tolerances, and a block-diagonal correction cannot
touch them. The network predicts, per camera, its rows Z_c (9 x 9) of a basis
whose span should contain those eigenvectors; the solver then adds the
balancing two-level correction built from Z (see csrc/mlp.hpp).

Harvest: plain-form LM solves driven stage by stage on the HARVEST problems; at
each inner trial (up to PER_PROBLEM per problem) the dense S is factored on
the device; its factor, the diagonal blocks S_cc, the features and the cameras
are kept, and the M lowest eigenvectors of the Jacobi-preconditioned S are
computed on the host.

Loss per system: the weighted share of those eigenvectors outside span(B^T Z)
(coarse_loss_and_grad, the gradient w.r.t. the network outputs in closed
form); the network's parameter gradients come from the library's backward
kernels. Adam, one system per step. The report (JSON beside the model) gives
the held-out loss and the evaluation solves (block-Jacobi vs learned, inner
PCG iterations at the strict Schur targets).
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
sys.path.insert(0, str(PKG))

K = 9            # coarse basis columns per camera
M_EIG = 9        # lowest eigenvectors per system in the loss
PER_PROBLEM = 12
# (problem, seed, LM iterations); a problem is a workload id or the generator
# parameters (cameras, points, track_min, track_max, alpha, outlier share,
# outlier sigma). The last one has the track and outlier statistics of
# workload 5 at a size whose dense S the host eigensolver handles in seconds.
HARVEST = [
    (2, 2, 20), (2, 12, 20), (2, 22, 20), (2, 32, 20),
    ((400, 120000, 2, 200, 2.2, 0.05, 20.0), 21, 15),
]
# held-out problems: block-Jacobi vs learned solves at the strict Schur targets
EVALUATE = [(2, 42), (4, 4)]


def make_problem(gba, spec, seed):
    if isinstance(spec, int):
        return gba.synthetic(spec, seed)
    C, P, kmin, kmax, alpha, ofrac, osig = spec
    return gba.synthetic_custom(C, P, kmin, kmax, alpha, ofrac, osig, seed)


def units(cams):
    """Row units of the basis: 1, except the focal-length row (f of the camera)."""
    u = np.ones((cams.shape[0], 9))
    u[:, 6] = cams[:, 6]
    return u


def coarse_loss_and_grad(O, cams, Bl, V, w=None):
    """Loss = sum_i w_i (1 - |Q v_i|^2) / sum w, Q the orthogonal projector onto
    span(Zh), Zh_c = B_c^T Z_c, Z_c(i, j) = O_c[9 i + j] * unit_i; V (9C x m)
    orthonormal eigenvectors of the Jacobi-preconditioned S, B_c (lower) the
    Cholesky factors of its diagonal blocks. Returns (loss, dloss/dO (C x
    O.shape[1], zero past column 81), per-vector captured share)."""
    C = O.shape[0]
    m = V.shape[1]
    w = np.ones(m) if w is None else np.asarray(w, np.float64)
    u = units(cams)
    Z = O[:, :9 * K].astype(np.float64).reshape(C, 9, K) * u[:, :, None]
    Zh = np.einsum("cji,cjk->cik", Bl, Z).reshape(9 * C, K)
    G = Zh.T @ Zh
    Ginv = np.linalg.inv(G)
    T = Ginv @ (Zh.T @ V)                      # K x m: coefficients of Q v_i
    PV = Zh @ T
    cap = np.einsum("ij,ij->j", V, PV)
    loss = float(np.sum(w * (1.0 - cap)) / np.sum(w))
    dZh = -2.0 * ((V - PV) * w) @ T.T / np.sum(w)     # 9C x K
    dZ = np.einsum("cij,cjk->cik", Bl, dZh.reshape(C, 9, K))
    dO = np.zeros_like(O, dtype=np.float64)
    dO[:, :9 * K] = (dZ * u[:, :, None]).reshape(C, 9 * K)
    return loss, dO, cap


def jacobi_eigvecs(L, Sdiag, C, m):
    """Lowest m eigenvectors of B^-1 S B^-T, S = L L^T (n x n lower factor), B_c =
    chol(S_cc); returns (eigenvalues, eigenvectors, B (C, 9, 9))."""
    import scipy.linalg as sl

    n = 9 * C
    Bl = np.linalg.cholesky(Sdiag)
    G = np.empty((n, n))
    for c in range(C):
        G[9 * c:9 * c + 9] = sl.solve_triangular(Bl[c], L[9 * c:9 * c + 9], lower=True)
    A = G @ G.T
    ev, V = sl.eigh(A, subset_by_index=[0, m - 1])
    return ev, V, Bl


def harvest(gba, torch, spec, seed: int, iterations: int, lam0: float = 1e-3):
    """Plain-form LM run driven stage by stage; returns systems
    {feat, cams, B, V, ev, lam}."""
    prob = make_problem(gba, spec, seed)
    C = prob.num_cameras
    systems = []
    feat_dev = torch.empty((C, 64), dtype=torch.float32, device="cuda")
    raw = []
    with gba.Solver(prob, "plain") as s:
        s.set_schur_layout("dense")  # the eigenvectors are taken of the dense factor
        gba.solver_set_harvest(s, True)
        sse = s.accumulate()
        lam = lam0
        _, _, _, n_pad = s.dims()
        for _ in range(iterations):
            nu, accepted, rel = 2.0, False, 0.0
            for _trial in range(16):
                if s.damp_invert_v(lam):
                    lam, nu = lam * nu, nu * 2
                    continue
                if s.schur_dense(lam) != 0:
                    lam, nu = lam * nu, nu * 2
                    continue
                gba.solver_features(s, lam, feat_dev.data_ptr())
                torch.cuda.synchronize()
                cams, _ = s.get_params()
                L = s.download("S").reshape(n_pad, n_pad).T[:9 * C, :9 * C]  # column-major -> [row, col]
                raw.append(dict(feat=feat_dev.cpu().numpy().copy(), cams=cams.reshape(C, 9).copy(),
                                Sdiag=s.download("Sdiag").reshape(C, 9, 9).copy(), L=np.tril(L), lam=lam))
                denom = s.back_substitute(lam)
                if not denom > 0:
                    lam, nu = lam * nu, nu * 2
                    continue
                a0 = s.counters()[0]
                tsse = s.trial_cost()
                if s.counters()[0] != a0 or not np.isfinite(tsse):
                    lam, nu = lam * nu, nu * 2
                    continue
                rho = (sse - tsse) / (0.5 * denom)
                if rho > 0 and tsse < sse:
                    s.accept()
                    rel = (sse - tsse) / max(sse, 1.0)
                    sse = tsse
                    lam *= max(1 / 3, 1 - (2 * rho - 1) ** 3)
                    accepted = True
                    break
                lam, nu = lam * nu, nu * 2
            if not accepted or rel < 1e-6:
                break
            s.accumulate()
    keep = np.unique(np.linspace(0, len(raw) - 1, min(PER_PROBLEM, len(raw))).astype(int))
    for i in keep:
        r = raw[i]
        ev, V, Bl = jacobi_eigvecs(r["L"], r["Sdiag"], C, M_EIG)
        systems.append(dict(feat=r["feat"], cams=r["cams"], B=Bl, V=V, ev=ev, lam=r["lam"]))
    return systems


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(PKG / "models" / "coarse_mlp.bin"))
    ap.add_argument("--epochs", type=int, default=300)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args()

    import torch

    import build as gba_build

    gba_build.build()
    import gba_gb300 as gba

    t0 = time.time()
    systems = []
    for spec, seed, iters in HARVEST:
        got = harvest(gba, torch, spec, seed, iters)
        systems += [dict(s, problem=str(spec), seed=seed) for s in got]
        print(f"harvested {spec} seed {seed}: {len(got)} systems ({time.time() - t0:.0f} s)", flush=True)
    rng = np.random.default_rng(args.seed)
    perm = rng.permutation(len(systems))
    n_val = max(1, len(systems) // 8)
    val, tr = [systems[i] for i in perm[:n_val]], [systems[i] for i in perm[n_val:]]
    cap = max(s["feat"].shape[0] for s in systems)
    mlp = gba.Mlp(seed=args.seed, capacity=cap)
    out_dev = torch.empty((cap, gba.Mlp.N_OUT), dtype=torch.float32, device="cuda")
    feats = [torch.from_numpy(s["feat"]).cuda() for s in systems]
    fidx = {id(s): i for i, s in enumerate(systems)}

    def run(sysd, train):
        f = feats[fidx[id(sysd)]]
        C = f.shape[0]
        mlp.forward(f.data_ptr(), C, out_dev.data_ptr())
        O = out_dev[:C].cpu().numpy()
        loss, dO, capt = coarse_loss_and_grad(O, sysd["cams"], sysd["B"], sysd["V"])
        if train:
            d = torch.from_numpy(dO.astype(np.float32)).cuda()
            mlp.backward(f.data_ptr(), d.data_ptr(), C)
        return loss, capt

    history = []
    steps = args.epochs * len(tr)
    step = 0
    for ep in range(args.epochs):
        tot = 0.0
        for i in rng.permutation(len(tr)):
            loss, _ = run(tr[i], True)
            lr = args.lr * 0.5 * (1 + np.cos(np.pi * step / steps))
            mlp.adam_step(lr)
            tot += loss
            step += 1
        if ep % 25 == 0 or ep == args.epochs - 1:
            vl = float(np.mean([run(s, False)[0] for s in val]))
            history.append((ep, tot / len(tr), vl))
            print(f"epoch {ep}: train {tot / len(tr):.4f} held-out {vl:.4f}", flush=True)
    out = Path(args.out)
    out.parent.mkdir(parents=True, exist_ok=True)
    mlp.save(out)
    held_cap = np.mean([run(s, False)[1] for s in val], axis=0)

    evaluation = []
    strict = dict(refine_tol=1e-8, pcg_tol=1e-4, max_iterations=30)
    for spec, seed in EVALUATE:
        prob = make_problem(gba, spec, seed)
        bj = gba.solve(prob.copy(), form="mixed", **strict)
        le = gba.solve(prob.copy(), form="learned", model_path=str(out), **strict)
        evaluation.append({
            "problem": spec, "seed": seed, "cameras": prob.num_cameras, "observations": prob.num_observations,
            "block_jacobi": {"pcg_iterations": bj.pcg_iterations, "final_cost": bj.final_cost,
                             "iterations": bj.iterations, "seconds": bj.total_time_s},
            "learned": {"pcg_iterations": le.pcg_iterations, "final_cost": le.final_cost,
                        "iterations": le.iterations, "seconds": le.total_time_s,
                        "judged_first_solve": {"block_jacobi": le.judge_iters[0], "learned": le.judge_iters[1],
                                               "winner": {1: "learned", 2: "block-Jacobi"}.get(le.learned_choice)}},
        })
        print(json.dumps(evaluation[-1]), flush=True)
    report = {
        "evaluation": evaluation,
        "systems": len(systems), "held_out": n_val, "harvest": HARVEST, "epochs": args.epochs, "lr": args.lr,
        "seconds": time.time() - t0, "held_out_loss": history[-1][2],
        "held_out_captured_share_per_eigenvector": held_cap.tolist(),
        "held_out_eigenvalues_mean": np.mean([s["ev"] for s in val], axis=0).tolist(),
        "history": history,
        "loss": f"share of the {M_EIG} lowest eigenvectors of the Jacobi-preconditioned S outside span(B^T Z)",
    }
    out.with_suffix(".json").write_text(json.dumps(report, indent=1))
    print(json.dumps({k: v for k, v in report.items() if k != "history"}))


if __name__ == "__main__":
    main()
