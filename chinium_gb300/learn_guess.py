"""Train and evaluate the learned starting density on water clusters.

  python -m chinium_gb300.learn_guess [--train 2000] [--kmax 8] [--test 200]
                                      [--epochs 200] [--out weights.npz]
  python -m chinium_gb300.learn_guess --eval-only [--test 200] [--precision fp64]

The defaults are the configured study: 2000 training clusters of 2..8 waters,
200 held-out clusters of 2..8 waters (about 13 minutes on one GB300).

1. Seeded clusters (H2O)_k, k ~ U{kmin..kmax}: rigid monomers, random
   orientations, O-O >= 2.6 A (training seed 0, held-out seed 1).
2. Converged PBE/def2-SVP/SG-1 densities from this library's SCF (GPU XC,
   repulsion integrals and J on the GPU).
3. Per-atom-pair samples (local-frame features and density blocks); the MLP
   (3 x 256, SiLU) is trained by the library's tensor-core kernels (Adam,
   FP32-level products from three BF16 planes per operand).
4. Held-out clusters: SCF from the SAP guess vs from the learned density
   (BF16-weight inference), iterations and SCF time to 1e-8 Eh.
Prints one JSON line with the summary; writes the weights to --out.
"""
import argparse
import json
import time

import numpy as np

from . import guess as G
from . import molecules as M
from .scf import run_scf


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=2000)
    ap.add_argument("--test", type=int, default=200)
    ap.add_argument("--kmin", type=int, default=2)
    ap.add_argument("--kmax", type=int, default=8)
    ap.add_argument("--epochs", type=int, default=200)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--functional", default="PBE")
    ap.add_argument("--out", default=G.DEFAULT_WEIGHTS)
    ap.add_argument("--residual", type=int, default=1, help="learn (converged - SAP) blocks")
    ap.add_argument("--test-kmax", type=int, default=0)
    ap.add_argument("--jk", default="engine", choices=["cpu", "engine"])
    ap.add_argument("--eval-only", action="store_true", help="evaluate the weights at --out on held-out clusters")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"],
                    help="XC builds of the held-out SCFs (mixed: incremental tensor-core builds)")
    args = ap.parse_args()
    log = lambda s: print(s, flush=True)
    if args.eval_only:
        model = G.load(args.out)
        rows = evaluate(model, args, log)
        print(json.dumps(dict(weights=args.out, precision=args.precision, **summarize(rows))), flush=True)
        return

    t0 = time.perf_counter()
    train = M.water_clusters(args.train, seed=0, kmin=args.kmin, kmax=args.kmax)
    X, T, Mk = [], [], []
    for i, (Z, xyz) in enumerate(train):
        r = run_scf(Z, xyz, functional=args.functional, guess="sap", jk_device=args.jk)
        if not r.converged:
            continue
        ctx = r.context
        base = G.sap_density(ctx["grid"], ctx["H"], ctx["S"], sum(Z) // 2) if args.residual else 0.0
        x, t, m = G.dataset(Z, xyz, ctx["basis"], r.D[0] - base)
        X.append(x)
        T.append(t)
        Mk.append(m)
        if i % 20 == 0:
            log("train molecule %d / %d (%d atoms, %d iterations)" % (i, len(train), len(Z), r.iterations))
    X, T, Mk = np.concatenate(X), np.concatenate(T), np.concatenate(Mk)
    t_data = time.perf_counter() - t0
    log("samples %d, data %.1f s" % (len(X), t_data))

    model = G.PairMLP(seed=0)
    model.residual = bool(args.residual)
    model.scale = float(np.sqrt((T ** 2 * Mk).sum() / Mk.sum()))
    t1 = time.perf_counter()
    losses = G.train(model, X, T / model.scale, Mk, epochs=args.epochs, lr=args.lr, log=log)
    t_train = time.perf_counter() - t1
    G.save(model, args.out)

    rows = evaluate(model, args, log)
    summary = {
        "train_clusters": len(train), "samples": int(len(X)), "epochs": args.epochs,
        "final_loss": losses[-1], "first_loss": losses[0], "residual": model.residual, "scale": model.scale, "data_s": t_data, "train_s": t_train,
        **summarize(rows)}
    print(json.dumps(summary), flush=True)


def evaluate(model, args, log):
    """Held-out clusters (seed 1): SCF from the SAP guess and from the
    learned density (timed including the guess); the setup (integrals, grid)
    is shared and not timed."""
    test = M.water_clusters(args.test, seed=1, kmin=args.kmin, kmax=args.test_kmax or args.kmax)
    kw = dict(functional=args.functional, jk_device=args.jk, precision=args.precision)
    if args.precision == "mixed":
        kw["anchor"] = "density"
    rows = []
    for Z, xyz in test:
        warm = run_scf(Z, xyz, functional=args.functional, guess="core", max_iter=1, jk_device=args.jk)
        ctx = warm.context
        if args.precision == "mixed":  # tiles and AO planes of the mixed path are setup too
            from ._lib import PRECISION_MIXED
            from .xc import ExchangeCorrelation
            ctx["grid"].build(ExchangeCorrelation().Read(args.functional), [warm.D[0]], precision=PRECISION_MIXED)
        r_sap = run_scf(Z, xyz, guess="sap", context=ctx, **kw)
        tg = time.perf_counter()
        D0 = G.guess_density(model, Z, xyz, ctx, precision=args.precision)
        t_guess = time.perf_counter() - tg
        r_ml = run_scf(Z, xyz, guess=D0, context=ctx, **kw)
        it_time = lambda r: r.wall - r.timings["setup"]
        log("test (%d atoms): SAP %d iterations, learned %d" % (len(Z), r_sap.iterations, r_ml.iterations))
        rows.append(dict(natoms=len(Z), it_sap=r_sap.iterations, it_ml=r_ml.iterations,
                         t_sap=it_time(r_sap), t_ml=it_time(r_ml) + t_guess,
                         dE=r_ml.energy - r_sap.energy, conv=bool(r_sap.converged and r_ml.converged)))
    return rows


def summarize(rows):
    it_sap = np.array([r["it_sap"] for r in rows], dtype=float)
    it_ml = np.array([r["it_ml"] for r in rows], dtype=float)
    return {
        "test_clusters": len(rows),
        "mean_iterations_sap": float(it_sap.mean()),
        "mean_iterations_learned": float(it_ml.mean()),
        "fewer_iterations_fraction": float((it_ml < it_sap).mean()),
        "more_iterations_fraction": float((it_ml > it_sap).mean()),
        "mean_scf_s_sap": float(np.mean([r["t_sap"] for r in rows])),
        "mean_scf_s_learned": float(np.mean([r["t_ml"] for r in rows])),
        "by_waters": {str(k): [float(it_sap[[r["natoms"] == 3 * k for r in rows]].mean()),
                               float(it_ml[[r["natoms"] == 3 * k for r in rows]].mean())]
                      for k in sorted({r["natoms"] // 3 for r in rows})},
        "max_abs_dE": float(np.max(np.abs([r["dE"] for r in rows]))),
        "all_converged": all(r["conv"] for r in rows),
    }


if __name__ == "__main__":
    main()
