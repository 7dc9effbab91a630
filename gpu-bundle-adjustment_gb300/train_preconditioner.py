"""Trains the learned block-Jacobi correction on the GPU with this library's own
MLP kernels (gba_mlp_*), from (S_cc, right-hand side, exact step) triples that
the plain FP64 solver generates.

  python train_preconditioner.py [--out models/bj_mlp.bin] [--steps 3000]

Harvest: plain-form LM solves of the 257-camera workload (2) and the
1,000-camera workload (3), seeds as listed in HARVEST; at every inner trial the
damped diagonal blocks S_cc, the Schur right-hand side g and the exact dense
step x* = S^-1 g are kept for every camera (Jacobi-scaled, see mlp.hpp).
Training: Adam on the mean per-camera block-norm step error; 10% of the
triples are held out. The report (JSON beside the model) gives the held-out
loss of the network and of plain block-Jacobi (the network at zero output).
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

# (problem, seed, LM iterations); a problem is a workload id or the generator
# parameters (cameras, points, track_min, track_max, alpha, outlier share,
# outlier sigma). The last two have the track and outlier statistics of
# workload 5 at a size the plain dense solver handles in seconds.
HARVEST = [
    (2, 2, 30), (2, 12, 30), (3, 3, 25), (3, 13, 25),
    ((1000, 300000, 2, 200, 2.2, 0.05, 20.0), 21, 20),
    ((600, 180000, 2, 200, 2.2, 0.05, 20.0), 22, 20),
]
# held-out problems on which the trained network is compared with block-Jacobi
EVALUATE = [(4, 4), ((2000, 600000, 2, 200, 2.2, 0.05, 20.0), 31)]


def make_problem(gba, spec, seed):
    if isinstance(spec, int):
        return gba.synthetic(spec, seed)
    C, P, kmin, kmax, alpha, ofrac, osig = spec
    return gba.synthetic_custom(C, P, kmin, kmax, alpha, ofrac, osig, seed)


def _tri():
    return [(i, j) for i in range(9) for j in range(i + 1)]


TRI = _tri()


def harvest(gba, torch, spec, seed: int, iterations: int, lam0: float = 1e-3):
    """Plain-form LM run driven stage by stage; returns per-camera training triples."""
    prob = make_problem(gba, spec, seed)
    C = prob.num_cameras
    feats, blocks, gs, xs = [], [], [], []
    feat_dev = torch.empty((C, 64), dtype=torch.float32, device="cuda")
    with gba.Solver(prob, "plain") as s:
        gba.solver_set_harvest(s, True)
        sse = s.accumulate()
        lam = lam0
        for _ in range(iterations):
            nu, accepted = 2.0, False
            for _trial in range(16):
                if s.damp_invert_v(lam):
                    lam, nu = lam * nu, nu * 2
                    continue
                if s.schur_dense(lam) != 0:
                    lam, nu = lam * nu, nu * 2
                    continue
                gba.solver_features(s, lam, feat_dev.data_ptr())
                torch.cuda.synchronize()
                feats.append(feat_dev.cpu().numpy().copy())
                blocks.append(s.download("Sdiag").reshape(C, 9, 9))
                gs.append(s.download("rhs")[:9 * C].reshape(C, 9))
                xs.append(s.download("dc").reshape(C, 9))
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
    return np.concatenate(feats), np.concatenate(blocks), np.concatenate(gs), np.concatenate(xs)


def scale(blocks, gs, xs):
    """Jacobi-scaled packed S^, its Cholesky factor, g^ and x^; drops blocks that
    are not numerically SPD."""
    d = np.sqrt(np.maximum(np.einsum("bii->bi", blocks), 1e-300))
    Sh = blocks / (d[:, :, None] * d[:, None, :])
    keep = np.ones(len(blocks), bool)
    Lh = np.zeros_like(Sh)
    for b in range(len(blocks)):
        try:
            Lh[b] = np.linalg.cholesky(Sh[b])
        except np.linalg.LinAlgError:
            keep[b] = False
    ii = np.array([i for i, _ in TRI])
    jj = np.array([j for _, j in TRI])
    pk = lambda M: M[:, ii, jj]  # noqa: E731
    ok = keep & np.isfinite(xs).all(1) & (np.abs(xs).sum(1) > 0)
    return ok, pk(Sh), pk(Lh), gs / d, xs * d


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(PKG / "models" / "bj_mlp.bin"))
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args()

    import torch

    import build as gba_build

    gba_build.build()
    import gba_gb300 as gba

    t0 = time.time()
    F, Sb, G, X = [], [], [], []
    for spec, seed, iters in HARVEST:
        f, s, g, x = harvest(gba, torch, spec, seed, iters)
        F.append(f)
        Sb.append(s)
        G.append(g)
        X.append(x)
        print(f"harvested {spec} seed {seed}: {len(f)} camera samples", flush=True)
    F, Sb, G, X = map(np.concatenate, (F, Sb, G, X))
    ok, Sh, Lh, Gh, Xh = scale(Sb, G, X)
    F, Sh, Lh, Gh, Xh = F[ok], Sh[ok], Lh[ok], Gh[ok], Xh[ok]
    n = len(F)
    rng = np.random.default_rng(args.seed)
    perm = rng.permutation(n)
    n_val = max(1, n // 10)
    val, tr = perm[:n_val], perm[n_val:]
    dev = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dt)  # noqa: E731
    D = {k: dev(v, torch.float64) for k, v in (("S", Sh), ("L", Lh), ("g", Gh), ("x", Xh))}
    D["f"] = dev(F, torch.float32)

    mlp = gba.Mlp(seed=args.seed, capacity=max(args.batch, n_val))

    def batch_ptrs(idx):
        t = torch.from_numpy(idx).to("cuda")
        parts = {k: v.index_select(0, t).contiguous() for k, v in D.items()}
        return parts, [parts[k].data_ptr() for k in ("f", "S", "L", "g", "x")]

    vparts, vptr = batch_ptrs(val)
    v0, vb = mlp.loss_grad(*vptr, len(val))
    history = [(0, v0, vb)]
    for step in range(1, args.steps + 1):
        idx = rng.choice(tr, size=min(args.batch, len(tr)), replace=False)
        parts, ptr = batch_ptrs(idx)
        loss, _ = mlp.loss_grad(*ptr, len(idx))
        lr = args.lr * (0.5 * (1 + np.cos(np.pi * step / args.steps)))  # cosine decay
        mlp.adam_step(lr)
        if step % 250 == 0 or step == args.steps:
            vl, vb = mlp.loss_grad(*vptr, len(val))
            history.append((step, vl, vb))
            print(f"step {step}: train {loss:.4f} held-out {vl:.4f} (block-Jacobi {vb:.4f})", flush=True)
    out = Path(args.out)
    out.parent.mkdir(parents=True, exist_ok=True)
    mlp.save(out)
    evaluation = []
    for spec, seed in EVALUATE:
        prob = make_problem(gba, spec, seed)
        bj = gba.solve(prob.copy(), form="mixed", max_iterations=30)
        le = gba.solve(prob.copy(), form="learned", model_path=str(out), max_iterations=30)
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
        "samples": int(n), "held_out": int(n_val), "harvest": HARVEST, "steps": args.steps, "batch": args.batch,
        "lr": args.lr, "seconds": time.time() - t0,
        "held_out_loss": history[-1][1], "held_out_block_jacobi_loss": history[-1][2],
        "history": history,
        "loss": "mean over cameras of (y - x*)^T S^ (y - x*) / (x*^T S^ x*), y = learned block step",
    }
    out.with_suffix(".json").write_text(json.dumps(report, indent=1))
    print(json.dumps({k: v for k, v in report.items() if k != "history"}))


if __name__ == "__main__":
    main()
