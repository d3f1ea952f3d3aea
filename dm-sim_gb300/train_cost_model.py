"""Train the engine's pass-time model on this GPU and save it.

The engine times every pass of its own random circuits (the 29-entry mixed
gate table) under several fusion plans (dmsim_cost_collect), the network is
fitted on the GPU by the library's own forward/backward/Adam kernels
(dmsim_cost_train), and the weights are written where the learned planner
looks for them by default (dm-sim_gb300/model/cost_mlp.bin, or --out).

    python dm-sim_gb300/train_cost_model.py [--sizes 10,12,14,16] [--out PATH]
"""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "python"))

import numpy as np  # noqa: E402

import dmsim_gb300 as E  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", default="10,12,14,16")
    ap.add_argument("--circuits", type=int, default=2)
    ap.add_argument("--gates", type=int, default=60)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", default=os.path.join(HERE, "model", "cost_mlp.bin"))
    args = ap.parse_args()
    feats, ms = [], []
    t0 = time.time()
    for i, n in enumerate(int(x) for x in args.sizes.split(",")):
        # 16 qubits (68.7 GB of FP64 state): shorter circuits, the passes are ~16x slower
        circuits, gates = (args.circuits, args.gates) if n <= 14 else (2, max(8, args.gates // 2))
        for arith in (E.AR_DF64, E.AR_FP64, E.AR_FP32):
            if arith == E.AR_FP64 and n > 14:
                continue  # FP64-pipe dense 4-qubit passes take ~1 s each at 16 qubits; the per-entry model extrapolates
            f, m = E.cost_collect(n, n_circuits=circuits, gates=gates, seed=100 * args.seed + 10 * i + arith,
                                  arith=arith)
            feats.append(f)
            ms.append(m)
    X, Y = np.concatenate(feats), np.concatenate(ms)
    t1 = time.time()
    # hold out every 5th sample to report generalisation
    idx = np.arange(len(Y))
    tr, te = idx[idx % 5 != 0], idx[idx % 5 == 0]
    loss = E.cost_train(X[tr], Y[tr], steps=args.steps, lr=args.lr, seed=args.seed)
    pred = E.cost_predict(X[te])
    err = np.abs(np.log(pred / Y[te]))
    loss_all = E.cost_train(X, Y, steps=args.steps, lr=args.lr, seed=args.seed)
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    E.cost_save(args.out)
    print(json.dumps({"samples": int(len(Y)), "collect_s": round(t1 - t0, 1), "train_s": round(time.time() - t1, 1),
                      "holdout_median_abs_log_err": float(np.median(err)),
                      "holdout_p90_abs_log_err": float(np.percentile(err, 90)),
                      "loss_train_split": [float(loss[0]), float(loss[1])],
                      "loss_all": [float(loss_all[0]), float(loss_all[1])], "out": args.out}))


if __name__ == "__main__":
    main()
