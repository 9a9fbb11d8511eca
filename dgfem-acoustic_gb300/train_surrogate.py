"""Builds the spectral surrogate from batched DG runs and evaluates it.

    python dgfem-acoustic_gb300/train_surrogate.py --out DIR

1. Draws 20,000 training (seed 5) and 2,000 held-out (seed 6) parameter rows
   (x, y, f, M, th, p) with the ensemble's distributions.
2. Runs every row through the batched DG path (FP32, 3000 RK4 steps, one
   fixed jittered mesh per order) and turns the observer pressure traces into
   128-bin log-PSD targets (surrogate.dg_spectra).
3. Trains four networks on 18,000 training rows (GPU kernels of csrc/mlp.cu),
   four more without one fold each for out-of-fold errors and the error
   network on those, keeps the remaining 2,000 training rows as the
   calibration split that sets each bound's acceptance threshold, and
   evaluates on the held-out rows: true RMS dB error per query, the queries
   accepted under each bound, and throughput against DG.
4. Writes DIR/surrogate.npz (weights, normalisation, calibration) and
   DIR/report.json.
"""
import argparse
import importlib
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--n-train", type=int, default=20000)
    ap.add_argument("--n-test", type=int, default=2000)
    ap.add_argument("--n-calib", type=int, default=2000)
    ap.add_argument("--train-steps", type=int, default=10000)
    ap.add_argument("--lr", type=float, default=4e-3)
    ap.add_argument("--dg-steps", type=int, default=3000)
    ap.add_argument("--grid", type=int, default=25)
    ap.add_argument("--bound-db", type=float, default=1.0)
    ap.add_argument("--models", type=int, default=4)
    ap.add_argument("--weight-decay", type=float, default=0.1)
    ap.add_argument("--data", default=None,
                    help="an OUT/dataset.npz of an earlier run with the same draws and DG settings: skips the DG runs")
    args = ap.parse_args()
    sys.path.insert(0, ROOT)
    pkg = importlib.import_module("dgfem-acoustic_gb300")
    S = pkg.surrogate
    os.makedirs(args.out, exist_ok=True)
    rep = {"n_train": args.n_train, "n_test": args.n_test, "n_calib": args.n_calib, "dg_steps": args.dg_steps,
           "grid": args.grid, "bound_db": args.bound_db, "models": args.models, "weight_decay": args.weight_decay,
           "train_steps": args.train_steps, "lr": args.lr}

    P_train = S.draw_params(args.n_train, 5)
    P_test = S.draw_params(args.n_test, 6)
    if args.data:
        d = np.load(args.data)
        if not (np.array_equal(d["P_train"], P_train) and np.array_equal(d["P_test"], P_test)
                and int(d["dg_steps"]) == args.dg_steps and int(d["grid"]) == args.grid):
            raise SystemExit("%s holds other draws or DG settings" % args.data)
        Y_train, Y_test = d["Y_train"].astype(np.float64), d["Y_test"].astype(np.float64)
        dg_s_train, dg_s_test = float(d["dg_s_train"]), float(d["dg_s_test"])
        rep["data"] = args.data
    else:
        t0 = time.perf_counter()
        Y_train, dg_s_train = S.dg_spectra(P_train, steps=args.dg_steps, grid=args.grid)
        Y_test, dg_s_test = S.dg_spectra(P_test, steps=args.dg_steps, grid=args.grid)
        rep["dg_generation_s"] = time.perf_counter() - t0
        np.savez_compressed(os.path.join(args.out, "dataset.npz"), P_train=P_train, P_test=P_test,
                            Y_train=Y_train.astype(np.float32), Y_test=Y_test.astype(np.float32),
                            dg_s_train=dg_s_train, dg_s_test=dg_s_test, dg_steps=args.dg_steps, grid=args.grid)
    rep["dg_run_s_train"], rep["dg_run_s_test"] = dg_s_train, dg_s_test
    np.savez_compressed(os.path.join(args.out, "heldout.npz"), params=P_test, targets=Y_test.astype(np.float32))

    nfit = args.n_train - args.n_calib
    t0 = time.perf_counter()
    sur = S.Surrogate.fit(P_train[:nfit], Y_train[:nfit], n_models=args.models, steps=args.train_steps, lr=args.lr,
                          grid=args.grid, dg_steps=args.dg_steps, weight_decay=args.weight_decay)
    rep["train_s"] = time.perf_counter() - t0
    rep["final_train_loss"] = [float(np.mean(l[-200:])) for l in sur.train_losses]
    rep["calibration_median_rms_db"] = sur.calibrate(P_train[nfit:], Y_train[nfit:])
    rep["out_of_fold_median_rms_db"] = float(np.median(sur.oof_rms_db))
    rep["thresholds_db"] = {str(b): sur.threshold(b) for b in (1.0, 2.0, 3.0, 5.0)}
    sur.save(os.path.join(args.out, "surrogate.npz"))

    # held-out evaluation
    mean, est = sur.predict(P_test)
    err = S.rms_db(mean, Y_test)
    acc = est <= sur.threshold(args.bound_db)
    base = S.rms_db(np.broadcast_to(Y_train[:nfit].mean(axis=0), Y_test.shape), Y_test)
    rep["heldout"] = {
        "rms_db_median": float(np.median(err)), "rms_db_p95": float(np.quantile(err, 0.95)),
        "rms_db_max": float(err.max()), "within_bound_fraction": float(np.mean(err <= args.bound_db)),
        "accepted_fraction": float(acc.mean()),
        "accepted_rms_db_max": float(err[acc].max()) if acc.any() else None,
        "accepted_above_bound_fraction": float(np.mean(err[acc] > args.bound_db)) if acc.any() else None,
        "mean_spectrum_baseline_rms_db_median": float(np.median(base)),
    }
    # throughput: surrogate queries (host arrays in and out, both networks)
    sur.predict(P_test[:64])
    t0 = time.perf_counter()
    reps = 20
    for _ in range(reps):
        sur.predict(P_test)
    sur_s = (time.perf_counter() - t0) / reps
    rep["surrogate_queries_per_s"] = args.n_test / sur_s
    rep["dg_queries_per_s"] = args.n_test / dg_s_test
    rep["speedup"] = rep["surrogate_queries_per_s"] / rep["dg_queries_per_s"]
    # the surrogate with its DG fallback at several bounds: the accepted
    # queries, their true error, and the throughput of the combined answer
    # (accepted queries from the network, the others re-run through DG)
    rep["by_bound"] = {}
    for b in (1.0, 2.0, 3.0, 5.0):
        acc_b = est <= sur.threshold(b)
        frac = float(acc_b.mean())
        t_per_q = (1 - frac) / rep["dg_queries_per_s"] + 1 / rep["surrogate_queries_per_s"]
        rep["by_bound"][str(b)] = {
            "accepted_fraction": frac,
            "accepted_rms_db_p95": float(np.quantile(err[acc_b], 0.95)) if acc_b.any() else None,
            "accepted_above_bound_fraction": float(np.mean(err[acc_b] > b)) if acc_b.any() else None,
            "queries_per_s_with_fallback": 1.0 / t_per_q,
            "speedup_over_dg": 1.0 / t_per_q / rep["dg_queries_per_s"]}
    with open(os.path.join(args.out, "report.json"), "w") as f:
        json.dump(rep, f, indent=1)
    print(json.dumps(rep))
    sur.close()


if __name__ == "__main__":
    main()
