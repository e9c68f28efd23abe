"""Learned cost model and the learned planner.

* ``random_pair_shapes`` / ``measure_pairs`` — training data: random complex
  pairwise contractions timed by the backend itself (``pq_measure_pairs``).
* ``CostModel`` — MLP (5 features -> 128 -> 128 -> 128 -> 1) trained on the
  GPU by the library's own forward/backward/Adam kernels (``pq_mlp_*``),
  predicting log(microseconds) of one pair; bf16 inference.
* ``learned_plan`` — ranks candidate contraction orders (and slicing sets)
  by predicted time.  The flop-count planner (``planning.best_flop_plan``)
  is the fallback and the judge: the learned choice must stay within a
  factor of the flop-optimal plan's complex multiply-adds, otherwise the
  flop-optimal plan is used.
"""
from __future__ import annotations

import ctypes as C
import time
from pathlib import Path

import numpy as np

from . import _lib as L
from .planning import (NetworkPlan, _leaf_arrays, device_backend, greedy_draws, open_output_edges, plan_cost,
                       sweep_steps, wavefunction_steps)

N_FEATURES = 5
WEIGHTS_FILE = Path(__file__).resolve().parent / "costmodel_gb300.npz"


def model_inputs(feats8):
    """8 step features -> the 5 model inputs: log2|C|, log2 K, log2|A|,
    log2|B|, log2 of the unit-stride run of the larger operand (scaled)."""
    f = np.atleast_2d(np.asarray(feats8, dtype=np.float64))
    run_big = np.where(f[:, 0] >= f[:, 1], f[:, 4], f[:, 5])
    X = np.stack([f[:, 2], f[:, 3], f[:, 0], f[:, 1], run_big], axis=1) / 16.0
    return X.astype(np.float32)


def random_pair_shapes(n, seed=0, max_log2=24, dim_choices=(2, 2, 2, 2, 3, 4, 8, 16, 32, 64), max_cmacs_log2=30):
    """Random pairwise contractions (ranks 2..30, bond dims 2..64) with every
    operand and the result at most 2^max_log2 elements and at most
    2^max_cmacs_log2 complex multiply-adds.  Returns the flat
    (a_ranks, b_ranks, labels, dims) arrays of ``pq_measure_pairs``."""
    rng = np.random.default_rng(seed)
    a_ranks, b_ranks, labels, dims = [], [], [], []
    choices = [int(x) for x in dim_choices]
    l2 = {x: float(np.log2(x)) for x in choices}
    pool = [choices[i] for i in rng.integers(0, len(choices), 64 * n + 64)]
    pi = [0]

    def fill(budget, cap):
        """Extents whose log2 sum stays within ``budget`` (at most ``cap`` modes)."""
        out, s = [], 0.0
        while len(out) < cap:
            d = pool[pi[0]]
            pi[0] += 1
            if s + l2[d] > budget + 1e-9:
                if s + 1.0 > budget + 1e-9:
                    break
                d = 2
            out.append(d)
            s += l2[d]
        return out, s

    u = rng.random((n, 3))
    for i in range(n):
        # log2 budgets: contracted, A-free, B-free, within every limit
        lk = u[i, 0] * min(12.0, max_log2)
        la = u[i, 1] * (max_log2 - lk)
        lb = u[i, 2] * min(max_log2 - lk, max_log2 - la, max_cmacs_log2 - lk - la)
        gk, sk = fill(lk, 8)
        ga, sa = fill(la, 30 - len(gk))
        gb, _ = fill(max(0.0, min(lb, max_cmacs_log2 - sk - sa)), 30 - len(gk))
        if len(gk) + len(ga) < 1:
            ga = [2]
        d = gk + ga + gb
        n_sh, n_a, n_b = len(gk), len(ga), len(gb)
        sh = list(range(n_sh))
        fa = list(range(n_sh, n_sh + n_a))
        fb = list(range(n_sh + n_a, n_sh + n_a + n_b))
        A = sh + fa
        B = sh + fb
        rng.shuffle(A)
        rng.shuffle(B)
        a_ranks.append(len(A))
        b_ranks.append(len(B))
        labels += A + B
        dims += [d[x] for x in A] + [d[x] for x in B]
    return (np.array(a_ranks, np.int32), np.array(b_ranks, np.int32), np.array(labels, np.int32),
            np.array(dims, np.int64))


def measure_pairs(backend, shapes, reps=3, chunk=512, budget_s=None, log=None):
    """Time pairs on the GPU; returns (ms[n'], feats[n', 8]) for the first n'
    pairs measured within ``budget_s`` seconds (all pairs if None)."""
    import time

    a_r, b_r, lab, dims = shapes
    n = len(a_r)
    ms = np.empty(n, np.float32)
    feats = np.empty((n, 8), np.float64)
    lib = L.lib()
    pos = 0
    t0 = time.perf_counter()
    for i0 in range(0, n, chunk):
        if budget_s is not None and time.perf_counter() - t0 > budget_s:
            if log:
                log({"measured": i0, "seconds": time.perf_counter() - t0, "stopped": "time budget"})
            return ms[:i0], feats[:i0]
        if log and i0 % (chunk * 20) == 0:
            log({"measured": i0, "seconds": time.perf_counter() - t0})
        i1 = min(n, i0 + chunk)
        cnt = int(a_r[i0:i1].sum() + b_r[i0:i1].sum())
        m = np.empty(i1 - i0, np.float32)
        f = np.empty((i1 - i0) * 8, np.float64)
        rc = lib.pq_measure_pairs(backend.ctx, i1 - i0, a_r[i0:i1].ctypes.data_as(L.i32p),
                                  b_r[i0:i1].ctypes.data_as(L.i32p),
                                  np.ascontiguousarray(lab[pos:pos + cnt]).ctypes.data_as(L.i32p),
                                  np.ascontiguousarray(dims[pos:pos + cnt]).ctypes.data_as(L.i64p), int(reps),
                                  m.ctypes.data_as(L.f32p), f.ctypes.data_as(L.f64p))
        L.check(rc, backend.ctx, "pq_measure_pairs")
        ms[i0:i1] = m
        feats[i0:i1] = f.reshape(-1, 8)
        pos += cnt
    return ms, feats


class CostModel:
    """The MLP cost model on the backend's device."""

    def __init__(self, backend, hidden=128, layers=3, seed=0):
        self.backend = backend
        self.lib = L.lib()
        h = C.c_void_p()
        L.check(self.lib.pq_mlp_create(backend.ctx, N_FEATURES, hidden, layers, seed, C.byref(h)), backend.ctx,
                "pq_mlp_create")
        self.h = h
        n = C.c_int64()
        L.check(self.lib.pq_mlp_num_params(h, C.byref(n)), backend.ctx, "pq_mlp_num_params")
        self.n_params = n.value
        self.hidden, self.layers = hidden, layers

    def close(self):
        if getattr(self, "h", None):
            self.lib.pq_mlp_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self):
        w = np.empty(self.n_params, np.float32)
        L.check(self.lib.pq_mlp_get_params(self.h, w.ctypes.data_as(L.f32p), w.size), self.backend.ctx,
                "get_params")
        return w

    @params.setter
    def params(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        L.check(self.lib.pq_mlp_set_params(self.h, w.ctypes.data_as(L.f32p), w.size), self.backend.ctx,
                "set_params")

    def gradients(self, X, y):
        X = np.ascontiguousarray(X, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        g = np.empty(self.n_params, np.float32)
        loss = C.c_float()
        L.check(self.lib.pq_mlp_gradients(self.h, X.ctypes.data_as(L.f32p), y.ctypes.data_as(L.f32p), len(y),
                                          g.ctypes.data_as(L.f32p), C.byref(loss)), self.backend.ctx, "gradients")
        return g, loss.value

    def train(self, X, y, epochs=30, batch=1024, lr=1e-3, seed=0):
        X = np.ascontiguousarray(X, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        loss = C.c_float()
        L.check(self.lib.pq_mlp_train(self.h, X.ctypes.data_as(L.f32p), y.ctypes.data_as(L.f32p), len(y),
                                      int(epochs), int(batch), float(lr), int(seed), C.byref(loss)),
                self.backend.ctx, "train")
        return loss.value

    def predict(self, X, bf16=True):
        X = np.ascontiguousarray(X, np.float32)
        out = np.empty(len(X), np.float32)
        if len(X) == 0:
            return out
        L.check(self.lib.pq_mlp_predict(self.h, X.ctypes.data_as(L.f32p), len(X), out.ctypes.data_as(L.f32p),
                                        1 if bf16 else 0), self.backend.ctx, "predict")
        return out

    def predict_us(self, feats8, bf16=True):
        """Predicted microseconds per step from 8-column step features."""
        return np.exp(self.predict(model_inputs(feats8), bf16=bf16).astype(np.float64))

    def save(self, path=WEIGHTS_FILE, meta=None):
        np.savez(path, params=self.params, hidden=self.hidden, layers=self.layers, **(meta or {}))

    @classmethod
    def load(cls, backend, path=WEIGHTS_FILE):
        d = np.load(path)
        m = cls(backend, int(d["hidden"]), int(d["layers"]))
        m.params = d["params"]
        return m


def train_cost_model(backend, n_pairs=200_000, seed=0, epochs=40, reps=3, log=None, budget_s=600.0,
                     max_log2=22, max_cmacs_log2=27):
    """Measure up to ``n_pairs`` random pairs on this GPU (within ``budget_s``
    seconds) and train the model on them (90/10 split).  Returns (model, stats)."""
    import time

    shapes = random_pair_shapes(n_pairs, seed, max_log2=max_log2, max_cmacs_log2=max_cmacs_log2)
    t0 = time.perf_counter()
    ms, feats = measure_pairs(backend, shapes, reps=reps, budget_s=budget_s, log=log)
    t_measure = time.perf_counter() - t0
    X = model_inputs(feats)
    y = np.log(np.maximum(ms.astype(np.float64), 1e-4) * 1e3).astype(np.float32)
    rng = np.random.default_rng(seed)
    idx = rng.permutation(len(y))
    nt = int(0.9 * len(y))
    tr, te = idx[:nt], idx[nt:]
    model = CostModel(backend, seed=seed)
    loss = model.train(X[tr], y[tr], epochs=epochs, batch=1024, lr=1e-3, seed=seed)
    pred = model.predict(X[te], bf16=True)
    rmse = float(np.sqrt(np.mean((pred - y[te]) ** 2)))
    base = float(np.sqrt(np.mean((y[te] - y[tr].mean()) ** 2)))
    stats = {"pairs": len(y), "measure_seconds": t_measure, "train_loss": loss, "test_rmse_log": rmse,
             "test_rmse_mean_predictor": base,
             "median_abs_rel_err": float(np.median(np.abs(np.exp(pred - y[te]) - 1)))}
    if log:
        log(stats)
    return model, stats


# ---------------------------------------------------------------------------
# learned planner
# ---------------------------------------------------------------------------

def candidate_plans(network, out_edges=None, n_random=16, seed=0, n_sweep_random=0):
    """Candidate SSA plans: the qubit sweeps (with ``n_sweep_random``
    randomized sweep orders, the cheapest few kept), the reference's
    full-wavefunction order (for open outputs), plain greedy and
    Boltzmann-greedy draws."""
    if out_edges is None:
        out_edges = open_output_edges(network)
    nodes, ranks, flat, dims, label_of = _leaf_arrays(network, out_edges)
    outl = [label_of[e] for e in out_edges]
    out = []
    # the sweep and native greedy planners return their own cost and largest
    # intermediate (the same label rule as plan_cost)
    for i, (s, c, m) in enumerate(sweep_steps(network, nodes, outl, label_of, ranks, flat, dims, all_orders=True,
                                              random_orders=n_sweep_random, seed=seed,
                                              cost_backend=device_backend(network))):
        out.append({"name": f"sweep{i}", "steps": s, "cmacs": c, "max_elems": m})
    if not out_edges or all(network.edges[e].src is not None for e in network.input_qubits):
        try:
            s = wavefunction_steps(network, nodes)
            cost, mx = plan_cost(ranks, flat, dims, s, outl)
            out.append({"name": "wavefunction", "steps": s, "cmacs": cost, "max_elems": mx})
        except KeyError:
            pass
    if n_random > 0:
        for i, (s, c, m) in enumerate(greedy_draws(ranks, flat, dims, outl, n_random, 1.0, 1.0, seed)):
            out.append({"name": f"greedy{i}", "steps": s, "cmacs": c, "max_elems": m})
    return out, out_edges


def learned_plan(network, model, out_edges=None, n_random=16, seed=0, flop_factor=8.0, max_elems=2**30,
                 slice_targets=(), max_sliced=10, batch=1024, timings=None, n_sweep_random=0):
    """Rank candidate plans -- and, with ``slice_targets``, candidate slicing
    sets of each (the slice chooser at each target, log2 elements, for plans
    whose largest intermediate exceeds the largest target) -- by the model's
    predicted time per amplitude.  The flop-count planner judges:
    candidates more than ``flop_factor`` times the minimum complex
    multiply-adds (or above ``max_elems`` without slicing) are rejected, and
    the flop-optimal plan is the fallback.  Returns (chosen, flop-optimal
    plan, all candidates); each candidate carries ``pred_us`` and, when
    slicing sets were ranked, its best ``sliced`` edge list.  ``timings``, a
    dict, receives the seconds spent generating and ranking candidates."""
    t0 = time.perf_counter()
    cands, out_edges = candidate_plans(network, out_edges, n_random, seed, n_sweep_random)
    t1 = time.perf_counter()
    best_flop = min(cands, key=lambda c: (c["cmacs"], c["max_elems"]))
    for c in cands:
        if c["cmacs"] > flop_factor * best_flop["cmacs"] or (c["max_elems"] > max_elems and not slice_targets):
            c["pred_us"] = float("inf")
            continue
        p = NetworkPlan(network, steps=c["steps"], out_edges=out_edges)
        if not slice_targets:
            c["pred_us"] = float(model.predict_us(p.features()).sum())
        else:
            best = (float("inf"), None)
            options = [[]] if c["max_elems"] <= max_elems else []
            # slicing a plan whose intermediates already fit the largest
            # target only adds work, so slicing sets are ranked when needed
            if c["max_elems"] > 2.0 ** max(slice_targets):
                for t in slice_targets:
                    sl = p.choose_slices(max_sliced=max_sliced, log2_target=float(t))
                    if sl not in options:
                        options.append(sl)
            for sl in options:
                feats, reps = p.sliced_features(sl, batch)
                t_us = float((model.predict_us(feats) * reps).sum())
                if t_us < best[0]:
                    best = (t_us, sl)
            c["pred_us"], c["sliced"] = best
        p.close()
    chosen = min(cands, key=lambda c: c["pred_us"])
    if not np.isfinite(chosen["pred_us"]):
        chosen = best_flop
    if timings is not None:
        timings["candidates_s"] = t1 - t0
        timings["ranking_s"] = time.perf_counter() - t1
    return chosen, best_flop, cands
