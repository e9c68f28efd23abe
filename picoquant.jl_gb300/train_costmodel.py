"""Train the learned cost model on this GPU and compare the learned planner
with the flop-count planner.

    python picoquant.jl_gb300/train_costmodel.py --pairs 200000 --out costmodel_gb300.npz

Measures ``--pairs`` random pair contractions with the backend's own kernels
in a context of the given ``--precision`` (the one the planner will be used
with; default the exact-accumulation tensor-core mode), trains the MLP on
the GPU, writes the weights, then
for a few circuit workloads executes both the learned planner's choice and the
flop-count planner's choice and prints their measured times (one JSON line
per workload).
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def time_plan(pq, net, steps, out_edges, reps=5):
    import ctypes as C

    import torch

    p = pq.NetworkPlan(net, steps=steps, out_edges=out_edges)
    p.capture()
    be = net.backend
    sp = C.c_void_p()
    be.lib.pq_ctx_stream(be.ctx, C.byref(sp))
    ext = torch.cuda.ExternalStream(sp.value)
    for _ in range(2):
        p.execute()
    be.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    for _ in range(reps):
        p.execute()
    e1.record(ext)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    res = p.result()
    p.close()
    return ms, res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=200_000)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--out", default=str(Path(__file__).resolve().parent / "costmodel_gb300.npz"))
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--budget", type=float, default=600.0, help="seconds allowed for measuring pairs")
    ap.add_argument("--precision", default="ozaki", choices=["c64", "3xtf32", "6xtf32", "ozaki"])
    args = ap.parse_args()
    import __graft_entry__ as g

    pq = g.load_package()
    from pqgb300 import costmodel as CM

    prec = {"c64": pq.PREC_C64, "3xtf32": pq.PREC_3XTF32, "6xtf32": pq.PREC_6XTF32, "ozaki": pq.PREC_OZAKI}
    be = pq.GB300Backend(prec[args.precision])
    t0 = time.perf_counter()
    model, stats = CM.train_cost_model(be, n_pairs=args.pairs, seed=args.seed, epochs=args.epochs,
                                       budget_s=args.budget, log=lambda d: print(json.dumps(d), flush=True))
    stats["seconds"] = time.perf_counter() - t0
    stats["precision"] = args.precision
    model.save(args.out, meta={"stats": json.dumps(stats)})
    print(json.dumps({"trained": stats}), flush=True)

    workloads = [
        ("grid4x5_d12_open_outputs", 4, 5, 12, None),
        ("grid5x5_d12_single_amplitude", 5, 5, 12, "0110100111001010011010011"),
        ("grid4x6_d16_single_amplitude", 4, 6, 16, "011010011100101001101001"),
    ]
    for name, r, c, d, bits in workloads:
        n = r * c
        gates = pq.random_grid_gates(r, c, d, seed=2024)
        net = pq.build_network(n, gates, backend=be, decompose=bits is not None)
        pq.add_input(net, "0" * n)
        out_edges = None
        if bits is not None:
            pq.add_output(net, bits)
            out_edges = []
        chosen, best_flop, cands = CM.learned_plan(net, model, out_edges=out_edges, n_random=16)
        oe = out_edges if out_edges is not None else pq.open_output_edges(net)
        t_l, r_l = time_plan(pq, net, chosen["steps"], oe)
        t_f, r_f = time_plan(pq, net, best_flop["steps"], oe)
        diff = float(np.max(np.abs(np.asarray(r_l) - np.asarray(r_f))))
        print(json.dumps({"workload": name, "learned": chosen["name"], "learned_ms": t_l,
                          "learned_pred_us": chosen["pred_us"], "learned_cmacs": chosen["cmacs"],
                          "flop": best_flop["name"], "flop_ms": t_f, "flop_cmacs": best_flop["cmacs"],
                          "speedup": t_f / t_l, "max_abs_diff_between_plans": diff,
                          "candidates": [(c_["name"], c_["cmacs"], c_.get("pred_us")) for c_ in cands]}),
              flush=True)
    model.close()
    be.close()


if __name__ == "__main__":
    main()
