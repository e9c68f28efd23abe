"""Benchmark: amplitudes/s of tensor-network contraction on one GB300.

Default workload (the configuration the headline metric is quoted on): one
single amplitude of a 6x6-qubit random grid circuit of depth 16 (Haar SU(2)
layers + CZ on four alternating edge patterns, CZ split into bond-2 virtual
edges), contracted along the qubit-sweep order the learned cost model ranks
first (the flop-count planner judging) with 10 bond-2 edges sliced -> 1024
identical-shape slices, batched per launch and summed on the device in FP64
(Neumaier), exact-accumulation tensor cores for the large pairs.  A step = all
1024 slices of one amplitude.

Also (--workload): grid4x5_d12_amps (1024 amplitudes of a 4x5 depth-12
circuit), grid7x7_d14_learned (learned plan selection, end to end),
uneven512 (512 circuits x 64 amplitudes), grid6x6_d16_accuracy (several
amplitudes against the plain FP64 path), pair (one pairwise contraction, for
kernel profiling).

Rank 0 prints one JSON line.  `--impl reference` times the FP64 CPU
restatement (numpy tensordot -> BLAS zgemm, all host cores) on a bounded
sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "amplitudes/s on 1 GB300: mixed-prec+learned plan vs plain FP64 @ rel err≤1e-6"
PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"


def load_peaks():
    try:
        return json.loads(PEAKS_FILE.read_text()), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------

# randomized qubit-sweep orders joining the sweep candidates of the 6x6
# depth-16 plans (every arm: mixed precision, plain FP64, CPU sample), seeded;
# planning is outside the timed region
SWEEP_RANDOM = 64


def build_sliced(pq, precision, rows=6, cols=6, depth=16, n_sliced=10, seed=2026, rank=0, target=28.0,
                 planner="learned", steps=None, tuning="off", storage="c64"):
    """The sliced single-amplitude workload on a new backend of ``precision``:
    network, plan (``steps`` if given, else the named planner's choice) and
    the sliced bonds chosen for a 2^target-element intermediate limit.
    ``tuning="cache"``: the autotuner's table for this GPU is loaded (the
    plan's classes it lacks tuned and the cache written back) and the plan
    compiled under it.  ``storage="c128"`` stores every tensor as complex128
    (the mixed modes otherwise store large tensors as complex64)."""
    n = rows * cols
    gates = pq.random_grid_gates(rows, cols, depth, seed=seed)
    bits = pq.random_bitstrings(n, 1, seed=seed + 1 + rank)[0]
    be = pq.GB300Backend(precision, small_elems=(1 << 62) if storage == "c128" else None)
    net = pq.build_network(n, gates, decompose=True, backend=be)
    pq.add_input(net, "0" * n)
    pq.add_output(net, bits)
    t0 = time.perf_counter()
    from pqgb300 import costmodel as CM

    if steps is not None:
        nodes, ranks, flat, dims, label_of = pq.planning._leaf_arrays(net, [])
        cm, mx = pq.planning.plan_cost(ranks, flat, dims, steps, [])
        name = "given"
    elif planner == "learned" and CM.WEIGHTS_FILE.exists():
        model = CM.CostModel.load(be)
        chosen, best_flop, cands = CM.learned_plan(net, model, out_edges=[], n_random=4, n_sweep_random=SWEEP_RANDOM)
        model.close()
        steps, cm, mx, name = chosen["steps"], chosen["cmacs"], chosen["max_elems"], "learned:" + chosen["name"]
    else:
        steps, cm, mx, name = pq.planning.best_flop_plan(net, out_edges=[], candidates=("sweep",),
                                                         sweep_random=SWEEP_RANDOM)
    plan = pq.NetworkPlan(net, steps=steps, out_edges=[])
    sliced = plan.choose_slices(max_sliced=n_sliced, log2_target=target)
    t_plan = time.perf_counter() - t0
    tune_info = None
    if tuning == "cache":
        from pqgb300 import autotune as AT

        t1 = time.perf_counter()
        loaded = AT.Tuner(be).load()
        tuner, new = AT.ensure_tuned(be, [plan])
        plan.close()
        plan = pq.NetworkPlan(net, steps=steps, out_edges=[])  # compiled under the tuned table
        tune_info = {"classes": len(tuner.entries), "cache_loaded": loaded, "tuned_now": new,
                     "seconds": time.perf_counter() - t1, "cache": AT.cache_path().name,
                     "changed": [{"key": k, "choice": AT.choice_name(e["choice"]),
                                  "default": AT.choice_name(e["default"]), "ms": e["ms"]}
                                 for k, e in tuner.entries.items() if e["choice"] != e["default"]]}
    return dict(be=be, net=net, plan=plan, sliced=sliced, gates=gates, bits=bits, cmacs=cm, max_elems=mx,
                planner=name, t_plan=t_plan, n=n, rows=rows, cols=cols, depth=depth, seed=seed,
                bits_seed=seed + 1 + rank, tuning=tune_info)


# The 6x6 depth-16 plan the GB300 arm contracts, recorded for the CPU
# reference arm (which must not load the product library to plan): written
# by `python bench.py --write-plan oracle/plans/grid6x6_d16_sliced.json`.
PLAN_FILE = ROOT / "oracle" / "plans" / "grid6x6_d16_sliced.json"


def plan_record(w):
    """The sliced workload's plan in a library-independent form: the
    circuit's generator seeds, the leaves (node names and their index names
    in node order), the SSA steps over them and the sliced bonds."""
    net, plan = w["net"], w["plan"]
    return {"workload": f"grid{w['rows']}x{w['cols']}_depth{w['depth']}_sliced_single_amplitude",
            "rows": w["rows"], "cols": w["cols"], "depth": w["depth"], "circuit_seed": w["seed"],
            "bitstring_seed": w["bits_seed"], "bitstring": w["bits"], "planner": w["planner"],
            "log2_cmacs": float(np.log2(w["cmacs"])), "log2_max_elems": float(np.log2(w["max_elems"])),
            "leaves": list(plan.leaves), "leaf_indices": [list(net.nodes[x].indices) for x in plan.leaves],
            "steps": [int(x) for x in plan.steps], "sliced": list(w["sliced"])}


def oracle_network(O, rec):
    """The record's network built by the oracle's own circuit generator and
    graph code; its leaves must be the record's (same node and index names in
    the same order), so the record's SSA steps apply to it."""
    rows, cols = rec["rows"], rec["cols"]
    n = rows * cols
    gates = O.random_grid_gates(rows, cols, rec["depth"], seed=rec["circuit_seed"])
    net = O.build_network(n, gates, decompose=True, backend=O.OracleBackend())
    O.add_input(net, "0" * n)
    O.add_output(net, rec["bitstring"])
    names = list(net.nodes.keys())
    if names != rec["leaves"] or [list(net.nodes[x].indices) for x in names] != rec["leaf_indices"]:
        raise RuntimeError("the oracle's network does not have the plan's leaves")
    return net


def oracle_amplitude(O, rec):
    """The record's amplitude contracted by the FP64 oracle (numpy tensordot
    -> BLAS zgemm) along the record's steps, unsliced; returns (amplitude,
    seconds of the contraction itself)."""
    net = oracle_network(O, rec)
    t0 = time.perf_counter()
    r = O.contract_along_steps(net, rec["steps"])
    dt = time.perf_counter() - t0
    return complex(np.asarray(r).reshape(-1)[0]), dt


def host_threads():
    """BLAS threads of the host arm: OPENBLAS_NUM_THREADS / OMP_NUM_THREADS
    when set, else every core (OpenBLAS's default)."""
    for v in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS"):
        if os.environ.get(v, "").isdigit():
            return int(os.environ[v])
    return os.cpu_count()


def leaf_host_data(pq, w, dtype):
    """Host copies of every leaf (what a caller uploads each end-to-end step)."""
    be, plan, net = w["be"], w["plan"], w["net"]
    out = []
    for nl in plan.leaves:
        lab = net.nodes[nl].data_label
        out.append((lab, np.asfortranarray(be.load_tensor_data(lab)).astype(dtype)))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="grid6x6_d16_sliced",
                    choices=["grid6x6_d16_sliced", "grid6x6_d16_accuracy", "grid4x5_d12_amps", "grid7x7_d14_learned",
                             "uneven512", "pair", "svd"],
                    help="grid7x7_d14_learned: learned plan selection over sweep orders and 256 seeded greedy "
                         "orders for a 7x7 depth-14 single amplitude, end to end; pair: one pairwise contraction "
                         "of the dominant shape (M x K c64 boundary times K x N c128 gate-column tensor), for "
                         "kernel profiling; svd: bond splits (decompose_tensor) on the host and on the device")
    ap.add_argument("--candidates", type=int, default=256, help="seeded random-greedy orders ranked by the model")
    ap.add_argument("--circuits", type=int, default=512, help="circuits of the uneven512 workload")
    ap.add_argument("--amplitudes", type=int, default=8, help="amplitudes of the grid6x6_d16_accuracy workload")
    ap.add_argument("--check", type=int, default=8, help="uneven512 circuits also run in complex128 for the error")
    ap.add_argument("--sv-budget-gb", type=float, default=64.0,
                    help="uneven512: state bytes resident at once in the grouped state-vector batch")
    ap.add_argument("--pair", default="1048576x256x256", help="M x N x K of the pair workload")
    ap.add_argument("--svd-sizes", default="16x16,64x64,128x128,256x256,1024x64",
                    help="m x n matrix sizes of the svd workload")
    ap.add_argument("--pair-order", default="mk", choices=["mk", "km"],
                    help="memory order of the pair's A: contiguous along M (mk) or along K (km)")
    ap.add_argument("--rows", type=int, default=6, help="grid rows of the sliced workload (smaller for ncu)")
    ap.add_argument("--cols", type=int, default=6)
    ap.add_argument("--depth", type=int, default=16)
    ap.add_argument("--precision", default="auto",
                    choices=["auto", "c64", "3xtf32", "6xtf32", "ozaki", "ozaki4", "3xbf16", "c128"])
    ap.add_argument("--storage", default="c64", choices=["c64", "c128"],
                    help="storage of large tensors in the mixed-precision modes (c128: every tensor complex128)")
    ap.add_argument("--batch", type=int, default=0, help="slices per launch (0: sized from memory)")
    ap.add_argument("--ref-budget", type=float, default=150.0,
                    help="seconds of whole-amplitude CPU steps the reference arm times (at least one step)")
    ap.add_argument("--oracle", default="full", choices=["full", "skip"],
                    help="contract the headline amplitude with the FP64 oracle too (rel_err_vs_oracle, cpu_baseline)")
    ap.add_argument("--write-plan", default="", help="write the sliced workload's plan record to this JSON file")
    ap.add_argument("--tuning", default="cache", choices=["cache", "off"],
                    help="cache: the autotuner's per-class kernel choices (cache for this GPU and kernels, missing "
                         "classes of the plan tuned first, outside the timed region); off: the fixed rules")
    ap.add_argument("--slice-target", type=float, default=28.0,
                    help="log2 elements allowed per slice intermediate when choosing sliced bonds")
    ap.add_argument("--fp64", default="full", choices=["full", "skip"],
                    help="also run the plain complex-FP64 GPU path on the same amplitude and plan")
    ap.add_argument("--fp64-steps", type=int, default=3, help="timed runs of the plain complex-FP64 path")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return 0
        return run_reference(args)
    if args.workload == "pair":
        return run_pair(args)
    if args.workload == "grid7x7_d14_learned":
        return run_learned(args)
    if args.workload == "uneven512":
        return run_uneven(args)
    if args.workload == "grid6x6_d16_accuracy":
        return run_accuracy(args)
    if args.workload == "svd":
        return run_svd(args)
    return run_gb300(args, world, rank)


def run_svd(args):
    """Bond splits (decompose_tensor!, src/layer1.jl:146-184) of random
    complex m x n tensors: per size and context precision, the time of one
    split on the host (download, LAPACK in FP64, upload) and on the device
    (pq_decompose_tensor, one-sided Jacobi), the median of --steps timed
    splits after --warmup, with the device's sweep count and the largest
    difference of the singular values (squared column norms of the left
    factor) between the two, relative to the largest."""
    import time

    import __graft_entry__ as g

    pq = g.load_package()
    rng = np.random.default_rng(0)
    for prec_name, prec in (("c64", pq.PREC_C64), ("c128", pq.PREC_C128)):
        for size in args.svd_sizes.split(","):
            m, n = (int(x) for x in size.lower().split("x"))
            T = rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))
            rec = {"workload": "svd", "precision": prec_name, "m": m, "n": n}
            sig = {}
            for mode in ("host", "device"):
                be = pq.GB300Backend(prec, svd=mode)
                ts = []
                for it in range(args.warmup + args.steps):
                    be.save_tensor_data("t", T)
                    be.sync()
                    t0 = time.perf_counter()
                    chi = be.decompose_tensor("t", [1], [2], left_label="b", right_label="c")
                    be.sync()
                    if it >= args.warmup:
                        ts.append(time.perf_counter() - t0)
                B = np.asarray(be.load_tensor_data("b")).reshape(m, chi, order="F")
                sig[mode] = np.sum(np.abs(B) ** 2, axis=0)
                rec[f"{mode}_ms"] = float(np.median(ts)) * 1e3
                rec["chi"] = chi
                if mode == "device":
                    rec["sweeps"] = be.last_svd_sweeps
                be.close()
            rec["sigma_rel_diff"] = float(np.max(np.abs(sig["host"] - sig["device"])) / np.max(sig["host"]))
            print(json.dumps(rec), flush=True)
    return 0


def run_accuracy(args):
    """Error distribution of the headline configuration: ``--amplitudes``
    single amplitudes of the 6x6 depth-16 circuit (bitstrings of ranks
    0, 1, ...: the headline's is rank 0), each computed in ``--precision``
    with the learned plan and in the plain complex-FP64 path with the
    flop-count plan; reports every relative error and their rms and max."""
    import __graft_entry__ as g

    pq = g.load_package()
    prec_name = args.precision if args.precision != "auto" else "ozaki"
    prec = {"c64": pq.PREC_C64, "3xtf32": pq.PREC_3XTF32, "6xtf32": pq.PREC_6XTF32, "ozaki": pq.PREC_OZAKI,
            "3xbf16": pq.PREC_3XBF16, "c128": pq.PREC_C128, "ozaki4": pq.PREC_OZAKI4}[prec_name]
    errs, scaled, secs = [], [], []
    for r in range(args.amplitudes):
        w = build_sliced(pq, prec, args.rows, args.cols, args.depth, rank=r, target=args.slice_target,
                         storage=args.storage)
        bat = w["plan"].auto_batch(w["sliced"])
        for _ in range(2):  # the second identical run records the CUDA graph
            a = w["plan"].run_sliced(w["sliced"], batch=bat)
        t0 = time.perf_counter()
        a = w["plan"].run_sliced(w["sliced"], batch=bat)
        secs.append(time.perf_counter() - t0)
        w["plan"].close()
        w["be"].close()
        w64 = build_sliced(pq, pq.PREC_C128, args.rows, args.cols, args.depth, rank=r, target=args.slice_target,
                           planner="flop")
        a64 = w64["plan"].run_sliced(w64["sliced"], batch=w64["plan"].auto_batch(w64["sliced"]))
        w64["plan"].close()
        w64["be"].close()
        errs.append(abs(a - a64) / abs(a64))
        scaled.append(abs(a - a64) / 2.0 ** (-(args.rows * args.cols) / 2))
    line = {"workload": f"grid{args.rows}x{args.cols}_depth{args.depth}_sliced_accuracy", "precision": prec_name,
            "metric": "relative amplitude error vs the plain complex-FP64 GPU path", "amplitudes": len(errs),
            "rel_errors": errs, "rms": float(np.sqrt(np.mean(np.square(errs)))), "max": float(np.max(errs)),
            "max_err_over_2^-n/2": float(np.max(scaled)), "target": 1e-6, "storage": args.storage,
            "ms_per_amplitude": [1e3 * x for x in secs],
            "timing": "third run of each amplitude (graph replay, host clock, result read back)",
            "plans": "learned plan (mixed) vs flop-count plan (FP64)", "data": "synthetic (seeded random circuit)"}
    print(json.dumps(line))
    return 0


AMP_INDEX = "__amplitudes__"


def batched_outputs(pq, net, bitstrings):
    """Output tensors for a batch of bitstrings: qubit q's output becomes a
    2 x B matrix whose column b is the basis vector of bitstring b's bit, and
    all of them share one extra index, so a single contraction leaves the B
    amplitudes as a vector over that index (a hyper index of the plan)."""
    from pqgb300 import network as NW

    B = len(bitstrings)
    for i in range(net.number_qubits):
        pos = net.qubit_ordering[i]
        index = net.output_qubits[pos - 1]
        data = np.zeros((2, B), dtype=np.complex128)
        for b, s in enumerate(bitstrings):
            data[1 if s[i] == "1" else 0, b] = 1.0
        label = NW.new_label(net, "node")
        net.nodes[label] = NW.Node([index, AMP_INDEX], [2, B], label)
        net.node_layers[label] = -1
        NW.save_tensor_data(net, label, data)
        net.edges[index].dst = label


def run_uneven(args):
    """Batched uneven workload: ``--circuits`` seeded random grid circuits
    (qubits uniform in 12..30, grid factorised from the count, depth uniform
    in 8..24), 64 random-bitstring amplitudes each.  Per circuit the cheaper
    of two strategies by a roofline estimate: the state vector (gates fused
    into blocks of at most four qubits) or the qubit-sweep tensor-network
    order with the 64 output bitstrings as one batch index.  All state-vector
    circuits run as one grouped batch (``StateVectorBatch``: circuits packed
    by size into chunks under a memory budget, launch s applying every
    circuit's s-th block, the whole batch one CUDA graph); each sweep circuit
    is a compiled plan captured as a CUDA graph.  Compilation and capture
    happen once (reported); a step replays everything and reads all
    amplitudes back.  The first ``--check`` circuits are also run in
    complex128, and a seeded sample of up to 16 circuits of at most 20 qubits
    is checked against the FP64 oracle's state vector."""
    import __graft_entry__ as g

    pq = g.load_package()
    from pqgb300 import circuits as CI
    from pqgb300 import planning as PL
    from pqgb300.svbatch import StateVectorBatch

    prec_name = args.precision if args.precision != "auto" else "ozaki"
    prec = {"c64": pq.PREC_C64, "3xtf32": pq.PREC_3XTF32, "6xtf32": pq.PREC_6XTF32, "ozaki": pq.PREC_OZAKI,
            "3xbf16": pq.PREC_3XBF16, "c128": pq.PREC_C128, "ozaki4": pq.PREC_OZAKI4}[prec_name]
    rng = np.random.default_rng(2026)
    specs = [(int(rng.integers(12, 31)), int(rng.integers(8, 25))) for _ in range(args.circuits)]
    t0 = time.perf_counter()
    plans = []
    for i, (n, d) in enumerate(specs):
        r, c = CI.grid_shape(n)
        gates = pq.random_grid_gates(r, c, d, seed=10_000 + i)
        fused = CI.fuse_gates(gates, 4)
        bits = pq.random_bitstrings(n, 64, seed=20_000 + i)
        t_sv = (2.0 ** n) * 16 * len(fused) / 6e12 + len(fused) * 4e-6
        host = _HostStore()
        hn = pq.build_network(n, gates, decompose=True, backend=host)
        pq.add_input(hn, "0" * n)
        batched_outputs(pq, hn, bits)
        nodes, ranks, flat, dims, label_of = PL._leaf_arrays(hn, [AMP_INDEX])
        sw, cm, mx = PL.sweep_steps(hn, nodes, [label_of[AMP_INDEX]], label_of, ranks, flat, dims)
        t_sw = cm * 8 / 40e12 + len(sw) // 2 * 4e-6 if mx * 8 < 2 ** 34 else float("inf")
        if t_sv <= t_sw:
            plans.append(dict(kind="statevector", n=n, d=d, r=r, c=c, i=i, fused=fused, gates=gates, bits=bits))
        else:
            plans.append(dict(kind="sweep", n=n, d=d, r=r, c=c, i=i, gates=gates, bits=bits, steps=sw))
    t_plan = time.perf_counter() - t0
    sv_ids = [k for k, p in enumerate(plans) if p["kind"] == "statevector"]
    sw_ids = [k for k, p in enumerate(plans) if p["kind"] == "sweep"]

    def sweep_network(be, ci, p):
        from pqgb300 import network as NW

        net = NW.TensorNetworkCircuit(p["n"], be)
        net.counters["node"] = ci * 10_000_000  # distinct tensor names per circuit on one backend
        for U, qs in p["gates"]:
            NW.add_gate(net, CI.operator_to_tensor(U), qs, decompose=True)
        pq.add_input(net, "0" * p["n"])
        batched_outputs(pq, net, p["bits"])
        return net

    def compile_all(be, ids_sv, ids_sw, budget):
        sb = StateVectorBatch(be, [(plans[k]["n"], plans[k]["fused"], plans[k]["bits"]) for k in ids_sv],
                              state_budget_bytes=budget) if ids_sv else None
        sweeps = []
        for k in ids_sw:
            net = sweep_network(be, k, plans[k])
            plan = pq.NetworkPlan(net, steps=plans[k]["steps"], out_edges=[AMP_INDEX])
            out = plan.capture()
            sweeps.append((k, plan, out))
        return (sb, list(ids_sv)), sweeps

    split = {"statevector_s": [], "sweeps_s": []}

    def run_all(be, sbk, sweeps):
        amps = {}
        sb, keys = sbk
        t_a = time.perf_counter()
        if sb is not None:
            for k, a in zip(keys, sb.execute()):
                amps[k] = a
        t_b = time.perf_counter()
        for k, plan, out in sweeps:
            plan.execute(out)
            amps[k] = np.asarray(be.load_tensor_data(out)).reshape(-1)
        split["statevector_s"].append(t_b - t_a)
        split["sweeps_s"].append(time.perf_counter() - t_b)
        return amps

    budget = int(args.sv_budget_gb * (1 << 30))
    be = pq.GB300Backend(prec)
    t1 = time.perf_counter()
    sbk, sweeps = compile_all(be, sv_ids, sw_ids, budget)
    sb = sbk[0]
    t_compile = time.perf_counter() - t1
    t1 = time.perf_counter()
    amps = run_all(be, sbk, sweeps)  # first pass records the state-vector graph
    t_first = time.perf_counter() - t1
    be.sync()
    launches0 = be.launch_count()
    ts = []
    for _ in range(max(1, args.steps)):
        t1 = time.perf_counter()
        amps = run_all(be, sbk, sweeps)
        be.sync()
        ts.append(time.perf_counter() - t1)
    launches = (be.launch_count() - launches0) / max(1, args.steps)
    sb_info = sb.info() if sb is not None else {}
    n_t = max(1, args.steps)
    t_sv = float(np.mean(split["statevector_s"][-n_t:]))
    t_swp = float(np.mean(split["sweeps_s"][-n_t:]))
    if sb is not None:
        peaks, peaks_kind = load_peaks()
        sb_info.update({"seconds_per_step": t_sv, "algorithmic_bytes": sb.algorithmic_bytes,
                        "achieved_gbs": sb.algorithmic_bytes / t_sv / 1e9,
                        "frac_of_hbm": sb.algorithmic_bytes / t_sv / 1e9 / peaks["hbm_gbs"],
                        "hbm_peak_source": f"{peaks_kind} hbm copy"})
    if sb is not None:
        sb.close()
    for _, plan, _ in sweeps:
        plan.close()
    be.close()
    # complex128 on the first --check circuits, same strategies
    k = min(args.check, len(plans))
    chk = list(range(k))
    chk_sv = [x for x in chk if plans[x]["kind"] == "statevector"]
    chk_sw = [x for x in chk if plans[x]["kind"] == "sweep"]
    # (the state-vector circuits as per-circuit complex128 plans: the grouped
    # batch itself always keeps complex64 states)
    be64 = pq.GB300Backend(pq.PREC_C128)
    _, sweeps64 = compile_all(be64, [], chk_sw, budget)
    ref64 = run_all(be64, (None, []), sweeps64)
    for _, plan, _ in sweeps64:
        plan.close()
    for x in chk_sv:
        from pqgb300 import network as NW

        p = plans[x]
        net = NW.TensorNetworkCircuit(p["n"], be64)
        net.counters["node"] = (len(plans) + x) * 10_000_000
        for U, qs in p["fused"]:
            NW.add_gate(net, CI.operator_to_tensor(U), qs, decompose=False)
        pq.add_input(net, "0" * p["n"])
        plan = pq.NetworkPlan(net, steps=PL.statevector_steps(net))
        res = plan.capture()
        ref64[x] = be64.gather(res, PL.bitstrings_to_index(p["bits"]))
        be64.delete_tensor(res)
        plan.close()
    be64.close()
    errs = [float(np.max(np.abs(amps[x] - ref64[x])) / np.sqrt(np.mean(np.abs(ref64[x]) ** 2))) for x in chk]
    # the FP64 oracle's state vector of the original gates, on a seeded sample
    oracle_errs = []
    if args.oracle == "full":
        sys.path.insert(0, str(ROOT / "oracle"))
        import tn_oracle as O  # the checker

        small = [x for x in range(len(plans)) if plans[x]["n"] <= 20]
        sample = sorted(np.random.default_rng(7).choice(small, size=min(16, len(small)), replace=False).tolist())
        for x in sample:
            p = plans[x]
            sv = O.statevector(p["n"], O.random_grid_gates(p["r"], p["c"], p["d"], seed=10_000 + p["i"]))
            ref = sv[[O.amplitude_index(b) for b in p["bits"]]]
            oracle_errs.append({"circuit": x, "qubits": p["n"], "depth": p["d"], "strategy": p["kind"],
                                "max_err_over_max_amp": float(np.max(np.abs(amps[x] - ref)) / np.max(np.abs(sv)))})
    secs = sum(ts) / len(ts)
    line = {"workload": f"uneven{args.circuits}_random_grid_circuits_64_amplitudes", "precision": prec_name,
            "metric": "amplitudes/s (all circuits, 64 amplitudes each; compiled once, every step replays the "
                      "captured graphs and reads all amplitudes back)",
            "value": 64 * len(plans) / secs, "unit": "amplitudes/s", "higher_is_better": True,
            "seconds_per_step": secs, "steps": len(ts), "circuits": len(plans),
            "qubits_range": [min(p["n"] for p in plans), max(p["n"] for p in plans)],
            "depth_range": [min(p["d"] for p in plans), max(p["d"] for p in plans)],
            "strategies": {"statevector_grouped": len(sv_ids), "sweep_batched": len(sw_ids)},
            "statevector_batch": {**sb_info, "state_budget_gb": args.sv_budget_gb,
                                  "storage": "complex64 states, FP32 block products"},
            "kernel_launches_per_step": launches, "sweep_circuits_seconds_per_step": t_swp,
            "host_planning_s": t_plan, "compile_and_upload_s": t_compile, "first_pass_s": t_first,
            "first_pass_amplitudes_per_s": 64 * len(plans) / (t_compile + t_first),
            "checked_circuits": k, "max_err_over_rms_amplitude_vs_c128": max(errs) if errs else None,
            "oracle_sample": oracle_errs,
            "oracle_max_err_over_max_amp": max(e["max_err_over_max_amp"] for e in oracle_errs) if oracle_errs
            else None,
            "grouping": "state-vector circuits: one grouped launch per block index over every circuit of a chunk, "
                        "the whole batch one CUDA graph; sweep circuits: one captured graph each",
            "data": "synthetic (seeded random circuits)"}
    print(json.dumps(line))
    return 0


def run_learned(args, rows=7, cols=7, depth=14):
    """Learned plan selection for a 7x7 depth-14 random circuit (49 qubits),
    one amplitude: candidate orders (the qubit sweeps, the full-wavefunction
    order and ``--candidates`` seeded random-greedy draws) and, for each, its
    slicing sets ranked by the cost model, the flop-count planner judging; the
    end-to-end time from the network to the amplitude (planning included) and
    the amplitudes of the learned and the flop-count plans and of the plain
    complex-FP64 path."""
    import torch

    import __graft_entry__ as g

    pq = g.load_package()
    from pqgb300 import costmodel as CM

    prec_name = args.precision if args.precision != "auto" else "ozaki"
    prec = {"c64": pq.PREC_C64, "3xtf32": pq.PREC_3XTF32, "6xtf32": pq.PREC_6XTF32, "ozaki": pq.PREC_OZAKI,
            "3xbf16": pq.PREC_3XBF16, "c128": pq.PREC_C128, "ozaki4": pq.PREC_OZAKI4}[prec_name]
    n = rows * cols
    gates = pq.random_grid_gates(rows, cols, depth, seed=2026)
    bits = pq.random_bitstrings(n, 1, seed=2027)[0]
    target = args.slice_target  # slice only what does not fit 2^target elements

    def network(be):
        net = pq.build_network(n, gates, decompose=True, backend=be)
        pq.add_input(net, "0" * n)
        pq.add_output(net, bits)
        return net

    def amplitude(plan, sliced):
        if sliced:
            return plan.run_sliced(sliced, batch=plan.auto_batch(sliced))
        plan.execute()
        return complex(np.asarray(plan.result()).reshape(-1)[0])

    be = pq.GB300Backend(prec)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    net = network(be)
    t_net = time.perf_counter() - t0
    model = CM.CostModel.load(be)
    # orders and slicing sets ranked together (unsliced, and the slice
    # chooser at 2^target, 2^(target-2), 2^(target-4) elements)
    phases = {}
    chosen, best_flop, cands = CM.learned_plan(net, model, out_edges=[], n_random=args.candidates,
                                               slice_targets=(target, target - 2, target - 4), batch=1024,
                                               timings=phases)
    model.close()
    t2 = time.perf_counter()
    plan = pq.NetworkPlan(net, steps=chosen["steps"], out_edges=[])
    sliced = chosen.get("sliced", [])
    t_plan = time.perf_counter() - t0
    phases = {"network_s": t_net, **phases, "compile_plan_s": time.perf_counter() - t2}
    amp = amplitude(plan, sliced)
    t_e2e = time.perf_counter() - t0
    # steady state: the same plan again, inputs resident
    for _ in range(max(0, args.warmup - 1)):
        amplitude(plan, sliced)
    be.sync()
    ts = []
    for _ in range(args.steps):
        t1 = time.perf_counter()
        amplitude(plan, sliced)
        ts.append(time.perf_counter() - t1)
    # the flop-count planner's choice, same precision, timed the same way
    # (warm, then --steps runs), interleaved with the learned plan's
    pf = pq.NetworkPlan(net, steps=best_flop["steps"], out_edges=[])
    sf = pf.choose_slices(max_sliced=10, log2_target=target)
    amp_f = None
    for _ in range(max(1, args.warmup - 1)):
        amp_f = amplitude(pf, sf)
    be.sync()
    tf, tl = [], []
    for _ in range(args.steps):
        t1 = time.perf_counter()
        amp_f = amplitude(pf, sf)
        tf.append(time.perf_counter() - t1)
        t1 = time.perf_counter()
        amplitude(plan, sliced)
        tl.append(time.perf_counter() - t1)
    t_flop = float(np.median(tf)) if tf else None
    t_learned = float(np.median(tl)) if tl else None
    pf.close()
    plan.close()
    be.close()
    # the FP64 oracle's contraction of the same amplitude along the learned plan
    oracle = None
    if args.oracle == "full":
        sys.path.insert(0, str(ROOT / "oracle"))
        import tn_oracle as O  # the checker

        nodes = list(net.nodes)
        rec = {"rows": rows, "cols": cols, "depth": depth, "circuit_seed": 2026, "bitstring": bits,
               "leaves": nodes, "leaf_indices": [list(net.nodes[x].indices) for x in nodes], "steps": chosen["steps"]}
        amp_o, t_o = oracle_amplitude(O, rec)
        oracle = {"amplitude": [amp_o.real, amp_o.imag], "seconds": t_o, "threads": host_threads(),
                  "rel_err": abs(amp - amp_o) / abs(amp_o)}
    # the plain complex-FP64 path on the flop-count plan
    be64 = pq.GB300Backend(pq.PREC_C128)
    net64 = network(be64)
    p64 = pq.NetworkPlan(net64, steps=best_flop["steps"], out_edges=[])
    s64 = p64.choose_slices(max_sliced=10, log2_target=target)
    t1 = time.perf_counter()
    amp64 = amplitude(p64, s64)
    t64 = time.perf_counter() - t1
    p64.close()
    be64.close()
    ranked = sorted((c for c in cands if np.isfinite(c.get("pred_us", np.inf))), key=lambda c: c["pred_us"])
    line = {"workload": f"grid{rows}x{cols}_depth{depth}_learned_plan_single_amplitude", "qubits": n,
            "depth": depth, "precision": prec_name,
            "metric": "end-to-end seconds to one amplitude (network -> plan -> amplitude)",
            "value": t_e2e, "unit": "s", "higher_is_better": False,
            "planning_s": t_plan, "planning_phases_s": phases, "steady_amplitudes_per_s": len(ts) / sum(ts) if ts else None,
            "learned_plan": {"name": chosen["name"], "log2_cmacs": float(np.log2(chosen["cmacs"])),
                             "pred_us": chosen["pred_us"]},
            "flop_plan": {"name": best_flop["name"], "log2_cmacs": float(np.log2(best_flop["cmacs"])),
                          "seconds": t_flop, "sliced_bonds": len(sf)},
            "learned_plan_seconds": t_learned,
            "learned_gain_over_flop_plan": (t_flop / t_learned) if (t_flop and t_learned) else None,
            "timing": "median of --steps warm runs per plan, interleaved (host clock, result read back)",
            "oracle": oracle, "rel_err_vs_oracle": oracle["rel_err"] if oracle else None,
            "candidates": len(cands), "candidates_within_flop_judge": len(ranked),
            "model_ranking_top5": [(c["name"], c["pred_us"], len(c.get("sliced", []))) for c in ranked[:5]],
            "sliced_bonds": len(sliced), "slice_target_log2": target,
            "amplitude": [amp.real, amp.imag],
            "rel_diff_learned_vs_flop_plan": abs(amp - amp_f) / abs(amp_f),
            "rel_err_vs_fp64": abs(amp - amp64) / abs(amp64), "plain_fp64_seconds": t64,
            "data": "synthetic (seeded random circuit)"}
    print(json.dumps(line))
    return 0


def run_pair(args):
    """Time one pairwise contraction C[m, n] = sum_k A[m, k] B[k, n] of the
    6x6 depth-16 plan's dominant shape (a 2^28-element complex64 boundary
    tensor absorbing a 2^16-element complex128 gate-column tensor: M = 2^20,
    N = K = 256) through a compiled two-leaf plan, inputs resident; reports
    the algorithmic rate 8 M N K / time and the error against FP64 on a row
    sample."""
    import ctypes as C

    import torch

    import __graft_entry__ as g

    pq = g.load_package()
    from pqgb300 import _lib as L

    M, N, K = (int(x) for x in args.pair.lower().split("x"))
    prec = {"c64": pq.PREC_C64, "3xtf32": pq.PREC_3XTF32, "6xtf32": pq.PREC_6XTF32, "ozaki": pq.PREC_OZAKI,
            "3xbf16": pq.PREC_3XBF16, "c128": pq.PREC_C128, "ozaki4": pq.PREC_OZAKI4}[args.precision if args.precision != "auto" else "ozaki"]
    be = pq.GB300Backend(prec)
    rng = np.random.default_rng(0)
    A = (rng.standard_normal((M, K)) + 1j * rng.standard_normal((M, K))).astype(np.complex64)
    B = rng.standard_normal((K, N)) + 1j * rng.standard_normal((K, N))
    km = args.pair_order == "km"
    be.save_tensor_data("a", A.T if km else A)  # stored column-major: (K, M) has K contiguous
    be.save_tensor_data("b", B)
    h = C.c_void_p()
    L.check(be.lib.pq_plan_create(be.ctx, 2, L.arr(C.c_int32, [2, 2]),
                                  L.arr(C.c_int32, [1, 0, 1, 2] if km else [0, 1, 1, 2]), 3,
                                  L.arr(C.c_int64, [M, K, N]), 1, L.arr(C.c_int32, [0, 1]), 2,
                                  L.arr(C.c_int32, [0, 2]), C.byref(h)), be.ctx, "plan_create")
    ids = L.arr(C.c_int64, [be.id_of("a"), be.id_of("b")])
    out = be.id_of("c")
    sp = C.c_void_p()
    be.lib.pq_ctx_stream(be.ctx, C.byref(sp))
    ext = torch.cuda.ExternalStream(sp.value)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(max(3, args.warmup)):
        L.check(be.lib.pq_plan_execute(h, ids, out), be.ctx, "execute")
    be.sync()
    times = []
    n0 = be.launch_count()
    for _ in range(args.steps):
        with torch.cuda.stream(ext):
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        L.check(be.lib.pq_plan_execute(h, ids, out), be.ctx, "execute")
        e1.record(ext)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    launches = be.launch_count() - n0
    got = be.load_tensor_data("c")
    rows = rng.choice(M, size=min(M, 2048), replace=False)
    ref = A[rows].astype(np.complex128) @ B
    err = float(np.max(np.abs(got[rows] - ref)) / np.max(np.abs(ref)))
    be.lib.pq_plan_destroy(h)
    be.close()
    ms = sum(times) / len(times)
    print(json.dumps({"workload": "pair", "pair": {"M": M, "N": N, "K": K, "a_order": args.pair_order},
                      "precision": args.precision,
                      "ms_per_contraction": ms, "algorithmic_tflops": 8.0 * M * N * K / ms / 1e9,
                      "gpu_launches_per_contraction": launches / max(1, args.steps),
                      "max_abs_err_over_max_abs_vs_fp64": err, "l2": "flushed between steps (256 MiB write)"}))
    return 0


def run_reference(args):
    """The CPU reference arm: the FP64 oracle (numpy restatement of the
    reference's contraction semantics, tensordot -> BLAS zgemm on every host
    core) timed on the same workload.  It imports neither the product
    package nor its library: the 6x6 depth-16 amplitude is contracted along
    the plan recorded in ``PLAN_FILE`` (the GB300 arm's plan), the network
    built by the oracle's own generator.  A step is one whole amplitude
    (about a minute on 16 cores), so the arm times as many steps as fit
    ``--ref-budget`` seconds (at least one, at most ``--steps``); CPU runs
    need no warm-up."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import tn_oracle as O  # the FP64 CPU restatement (reference arm)

    cores = host_threads()
    base = {"impl": "reference", "metric": METRIC, "unit": "amplitudes/s", "n_gpus": args.gpus,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic"}
    if args.workload == "grid6x6_d16_sliced":
        rows, cols, depth = args.rows, args.cols, args.depth
        if not PLAN_FILE.exists() or (rows, cols, depth) != (6, 6, 16):
            print(json.dumps({"impl": "reference", "unavailable": f"no recorded plan for grid{rows}x{cols} depth "
                                                                  f"{depth} ({PLAN_FILE.name} covers 6x6 depth 16)"}))
            return 0
        rec = json.loads(PLAN_FILE.read_text())
        times, amp = [], None
        t_start = time.perf_counter()
        while len(times) < max(1, args.steps):
            amp, dt = oracle_amplitude(O, rec)
            times.append(dt)
            if time.perf_counter() - t_start + dt > args.ref_budget:
                break
        val = len(times) / sum(times)
        sample = (f"timed: {len(times)} whole amplitude(s) of the 6x6 depth-16 circuit, each contracted unsliced "
                  f"by the FP64 oracle (numpy tensordot -> BLAS zgemm, {cores} threads) along the GB300 arm's plan "
                  f"({rec['planner']}, 2^{rec['log2_cmacs']:.2f} complex MACs, read from {PLAN_FILE.name}); "
                  f"{np.mean(times):.1f} s per amplitude")
        extra = {"amplitude": [amp.real, amp.imag], "steps_requested": args.steps,
                 "plan_sha": plan_sha(rec["steps"])}
    else:
        rows, cols, depth = 4, 5, 12
        val, sample = _cpu_sample_amps(O, rows, cols, depth)
        times, extra = [1024 / val], {}
    line = {**base, "value": val, "steps": len(times), "warmup": 0, "ms_per_step": 1e3 * float(np.mean(times)),
            "config": workload_config(args, rows, cols, depth),
            "cpu_baseline": {"value": val, "unit": "amplitudes/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": val, "unit": "amplitudes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    line.update(extra)
    print(json.dumps(line))
    return 0


def plan_sha(steps):
    import hashlib

    return hashlib.sha256(",".join(str(int(x)) for x in steps).encode()).hexdigest()[:16]


def workload_config(args, rows, cols, depth):
    if args.workload == "grid6x6_d16_sliced":
        return {"workload": f"grid{rows}x{cols}_depth{depth}_sliced_single_amplitude", "qubits": rows * cols,
                "depth": depth, "sliced_bonds": 10, "slices": 1024, "batch": args.batch,
                "plan": "learned cost model over qubit-sweep orders (flop-count planner judges); the plain FP64 "
                        "GPU path, the FP64 oracle and the CPU reference arm contract the same plan",
                "l2": "flushed between steps (256 MiB write)"}
    return {"workload": f"grid{rows}x{cols}_depth{depth}_1024_amplitudes", "qubits": rows * cols, "depth": depth,
            "amplitudes_per_step": 1024,
            "plan": "flop-count planner over the circuit fused into blocks of up to four qubits (open outputs + "
                    "gather)",
            "l2": "flushed between steps (256 MiB write)"}


class _HostStore:
    """Minimal host tensor store for building the CPU-baseline network."""

    def __init__(self):
        from pqgb300.backend import Metrics

        self.tensors = {}
        self.metrics = Metrics()

    def save_tensor_data(self, label, data):
        self.tensors[label] = np.asarray(data, dtype=np.complex128)

    def shape(self, label):
        return self.tensors[label].shape


def _cpu_sample_amps(O, rows=4, cols=5, depth=12):
    """1024 amplitudes of the 4x5 depth-12 circuit from the oracle's FP64
    state vector (one tensordot per gate), timed."""
    n = rows * cols
    gates = O.random_grid_gates(rows, cols, depth, seed=2024)
    t0 = time.perf_counter()
    sv = O.statevector(n, gates)
    bits = O.random_bitstrings(n, 1024, seed=7)
    _ = sv[[O.amplitude_index(b) for b in bits]]
    dt = time.perf_counter() - t0
    return 1024 / dt, "timed: all 1024 amplitudes via the oracle's FP64 numpy state vector (tensordot per gate)"


def run_gb300(args, world, rank):
    import torch

    import __graft_entry__ as g

    pq = g.load_package()
    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    dev = torch.cuda.current_device()
    peaks, peaks_kind = load_peaks()
    prec_map = {"c64": pq.PREC_C64, "3xtf32": pq.PREC_3XTF32, "6xtf32": pq.PREC_6XTF32, "ozaki": pq.PREC_OZAKI,
                "3xbf16": pq.PREC_3XBF16, "c128": pq.PREC_C128, "ozaki4": pq.PREC_OZAKI4}
    prec_name = args.precision if args.precision != "auto" else "ozaki"
    precision = prec_map[prec_name]

    if args.workload == "grid6x6_d16_sliced":
        rows, cols, depth = args.rows, args.cols, args.depth
        w = build_sliced(pq, precision, rows, cols, depth, rank=rank, target=args.slice_target,
                         tuning=args.tuning if precision != pq.PREC_C128 else "off", storage=args.storage)
        be, plan, sliced = w["be"], w["plan"], w["sliced"]
        if args.batch <= 0:
            args.batch = plan.auto_batch(sliced)

        def step():
            return plan.run_sliced(sliced, batch=args.batch)

        amps_per_step = 1
    else:
        from pqgb300 import circuits as CI

        rows, cols, depth = 4, 5, 12
        n = rows * cols
        gates = pq.random_grid_gates(rows, cols, depth, seed=2024)
        be = pq.GB300Backend(precision)
        # the circuit as blocks of up to four qubits (exact): one pass over the
        # state per block in a state-vector order
        net = pq.build_network(n, CI.fuse_gates(gates, 4), backend=be)
        pq.add_input(net, "0" * n)
        steps_, cm, mx, name = pq.planning.best_flop_plan(
            net, trials=4, candidates=("sweep", "greedy", "wavefunction", "statevector"))
        plan = pq.NetworkPlan(net, steps=steps_)
        plan.capture()
        bits = pq.random_bitstrings(n, 1024, seed=7)
        w = dict(be=be, net=net, plan=plan, cmacs=cm, max_elems=mx, planner=name, bits=bits)

        def step():
            return plan.amplitudes(bits)

        amps_per_step = 1024

    import ctypes as C

    sp = C.c_void_p()
    be.lib.pq_ctx_stream(be.ctx, C.byref(sp))
    ext = torch.cuda.ExternalStream(sp.value)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    for _ in range(max(3, args.warmup)):
        step()
    be.sync()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(dev)
    clocks.start()
    launches0 = be.launch_count()
    times = []
    result = None
    for _ in range(args.steps):
        with torch.cuda.stream(ext):
            flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        result = step()
        e1.record(ext)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    launches = be.launch_count() - launches0
    clk = clocks.stop()
    t_total = sum(times) / 1e3
    if dist:
        t = torch.tensor([t_total], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_total = float(t.item())
        dist.barrier()
    value = world * amps_per_step * args.steps / t_total

    # ---- end to end: host leaf upload + contraction + result download -----
    e2e = None
    if args.workload == "grid6x6_d16_sliced":
        host = leaf_host_data(pq, w, np.complex128 if precision == pq.PREC_C128 else np.complex64)
        h2d = sum(a.nbytes for _, a in host)
        prepared = be.prepare_tensors(host)  # the argument arrays, built once (the host buffers are reused)

        def e2e_step():
            be.save_prepared(prepared)  # every leaf's current values: one staging copy + one device scatter
            return plan.run_sliced(sliced, batch=args.batch)

        e2e_step()
        ts = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            e2e_step()
            ts.append(time.perf_counter() - t0)
        e2e = {"value": world / (sum(ts) / len(ts)), "unit": "amplitudes/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": 16}
    else:
        def e2e_step():
            return plan.amplitudes(w["bits"])

        ts = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            e2e_step()
            ts.append(time.perf_counter() - t0)
        e2e = {"value": world * 1024 / (sum(ts) / len(ts)), "unit": "amplitudes/s",
               "h2d_bytes_per_step": 1024 * 8, "d2h_bytes_per_step": 1024 * 16}

    line = None
    if rank == 0:
        line = report(args, pq, w, be, plan, rows, cols, depth, value, t_total, times, launches, clk, e2e, peaks,
                      peaks_kind, prec_name, precision, result, world)
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def report(args, pq, w, be, plan, rows, cols, depth, value, t_total, times, launches, clk, e2e, peaks, peaks_kind,
           prec_name, precision, result, world):
    import torch

    sys.path.insert(0, str(ROOT / "oracle"))
    import tn_oracle as O  # the FP64 oracle: the checker and the timed cpu_baseline leg only

    import ctypes as C

    extra = {}
    roof = None
    cpu = None
    ms_step = 1e3 * t_total / args.steps
    sp = C.c_void_p()
    be.lib.pq_ctx_stream(be.ctx, C.byref(sp))
    ext = torch.cuda.ExternalStream(sp.value)
    if args.workload == "grid6x6_d16_sliced":
        sliced = w["sliced"]
        ms, batched, feats = plan.profile_sliced(sliced, batch=args.batch)
        roof, kinfo, overall = roofline_from_profile(ms, batched, feats, peaks, peaks_kind,
                                                     2 ** len(sliced) // args.batch, prec_name, ms_step)
        extra["kernel_classes"] = kinfo
        extra["roofline_all_steps"] = overall
        rec = plan_record(w)
        ref_rec = json.loads(PLAN_FILE.read_text()) if PLAN_FILE.exists() else None
        if args.write_plan:
            Path(args.write_plan).parent.mkdir(parents=True, exist_ok=True)
            Path(args.write_plan).write_text(json.dumps(rec))
        extra["amplitude"] = [float(np.real(result)), float(np.imag(result))]
        extra["tuning"] = w.get("tuning")
        extra["plan"] = {"planner": w["planner"], "cmacs_unsliced": w["cmacs"], "max_elems_unsliced": w["max_elems"],
                         "sliced_bonds": len(sliced), "planning_s": w["t_plan"], "plan_sha": plan_sha(rec["steps"]),
                         "same_plan_as_reference_arm": bool(ref_rec is not None and ref_rec["steps"] == rec["steps"]
                                                            and ref_rec["leaves"] == rec["leaves"])}
        # the flop-count planner's own pick (the method without the learned
        # model) on the same backend and tuned table, timed like the headline
        fsteps, fcm, fmx, fname = pq.planning.best_flop_plan(w["net"], out_edges=[], candidates=("sweep",),
                                                              sweep_random=SWEEP_RANDOM)
        flop = {"planner": "flop:" + fname, "log2_cmacs": float(np.log2(fcm)),
                "same_as_learned": list(fsteps) == list(plan.steps)}
        if not flop["same_as_learned"]:
            pf = pq.NetworkPlan(w["net"], steps=fsteps, out_edges=[])
            sf = pf.choose_slices(max_sliced=len(sliced), log2_target=args.slice_target)
            bf = pf.auto_batch(sf)
            for _ in range(2):
                pf.run_sliced(sf, batch=bf)

            def timed(fn):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(ext)
                fn()
                e1.record(ext)
                e1.synchronize()
                return e0.elapsed_time(e1)

            tfl, tle = [], []
            for _ in range(max(3, args.fp64_steps)):  # interleaved, no L2 flush for either
                tfl.append(timed(lambda: pf.run_sliced(sf, batch=bf)))
                tle.append(timed(lambda: plan.run_sliced(sliced, batch=args.batch)))
            pf.close()
            flop["ms_per_amplitude"] = float(np.median(tfl))
            flop["learned_ms_per_amplitude"] = float(np.median(tle))
            extra["learned_gain_over_flop_plan"] = flop["ms_per_amplitude"] / flop["learned_ms_per_amplitude"]
        extra["flop_plan"] = flop
        # the plain complex-FP64 CUDA path on the same amplitude along the same
        # plan, timed warm with CUDA events on its context's stream
        a64 = None
        if args.fp64 == "full":
            w64 = build_sliced(pq, pq.PREC_C128, rows, cols, depth, target=args.slice_target, steps=plan.steps)
            p64, s64 = w64["plan"], w64["sliced"]
            b64 = p64.auto_batch(s64)
            sp = C.c_void_p()
            w64["be"].lib.pq_ctx_stream(w64["be"].ctx, C.byref(sp))
            ext64 = torch.cuda.ExternalStream(sp.value)
            for _ in range(2):  # warm-up; the second identical call records the CUDA graph
                a64 = p64.run_sliced(s64, batch=b64)
            ts64 = []
            for _ in range(max(3, args.fp64_steps)):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(ext64)
                a64 = p64.run_sliced(s64, batch=b64)
                e1.record(ext64)
                e1.synchronize()
                ts64.append(e0.elapsed_time(e1))
            extra["plain_fp64_gpu"] = {
                "value": len(ts64) / (sum(ts64) / 1e3), "unit": "amplitudes/s", "steps": len(ts64),
                "sliced_bonds": len(s64), "batch": b64,
                "sample": "the same amplitude along the same plan, all slices, complex128 storage and FP64 kernels; "
                          "2 warm-up runs, then CUDA events on the context's stream"}
            extra["speedup_vs_plain_fp64"] = value / extra["plain_fp64_gpu"]["value"]
            extra["rel_err_vs_fp64"] = abs(result - a64) / abs(a64)
            p64.close()
            w64["be"].close()
        # the FP64 oracle's contraction of the same amplitude along the same
        # plan (its own network build, numpy on the host): the parity check,
        # and the timed CPU baseline
        if args.oracle == "full":
            amp_o, t_o = oracle_amplitude(O, rec)
            extra["oracle"] = {"amplitude": [amp_o.real, amp_o.imag], "seconds": t_o, "threads": host_threads()}
            extra["rel_err_vs_oracle"] = abs(result - amp_o) / abs(amp_o)
            # relative to the amplitude scale 2^(-n/2) (amplitudes of random
            # circuits are Porter-Thomas distributed around it)
            extra["err_vs_oracle_over_2^-n/2"] = abs(result - amp_o) / 2.0 ** (-rows * cols / 2)
            if a64 is not None:
                extra["plain_fp64_gpu"]["rel_err_vs_oracle"] = abs(a64 - amp_o) / abs(amp_o)
            cpu = {"value": 1.0 / t_o, "unit": "amplitudes/s", "cores": host_threads(), "kind": "port",
                   "sample": f"timed: the whole amplitude contracted unsliced by the FP64 oracle (numpy tensordot -> "
                             f"BLAS zgemm, {host_threads()} threads) along the same plan, once ({t_o:.1f} s)"}
    else:
        extra["plan"] = {"planner": w["planner"], "cmacs": w["cmacs"], "max_elems": w["max_elems"]}
        ms = w["plan"].profile()
        feats = w["plan"].features()
        roof, kinfo, overall = roofline_from_profile(ms, np.zeros(len(ms), bool), feats, peaks, peaks_kind, 1,
                                                     prec_name, ms_step)
        extra["kernel_classes"] = kinfo
        extra["roofline_all_steps"] = overall
        # the fidelity check: the open-output result is the whole 2^20 state,
        # whose squared norm (FP64, on the device) is 1 for a unitary circuit
        n2 = be.norm2(w["plan"].execute())
        extra["state_fidelity_check"] = {"norm2": n2, "abs_norm2_minus_1": abs(n2 - 1.0),
                                         "how": "pq_tensor_norm2: FP64 compensated sum of |psi|^2 on the device"}
        v, desc = _cpu_sample_amps(O, rows, cols, depth)
        cpu = {"value": v, "unit": "amplitudes/s", "cores": host_threads(), "kind": "port", "sample": desc}
    line = {
        "metric": METRIC, "value": value, "unit": "amplitudes/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": {"c64": "c64", "3xtf32": "c64(3xtf32)", "6xtf32": "c64(6xtf32)",
                                                           "ozaki": "c64(ozaki-bf16)", "3xbf16": "c64(3xbf16)",
                                                           "c128": "c128", "ozaki4": "c64(ozaki4-bf16)"}[prec_name]
        if args.storage == "c64" else f"c128({prec_name})",
        "data": "synthetic (seeded random circuits)", "config": workload_config(args, rows, cols, depth),
        "precision": prec_name, "e2e": e2e, "gpu_launches": int(launches), "clocks": clk, "roofline": roof,
        "cpu_baseline": cpu,
    }
    line.update(extra)
    return line


# Tensor-core operations per algorithmic flop of a complex multiply-add:
# 3xTF32 issues 3 split products of each of 4 real products, 6xTF32 6; the
# exact-accumulation scheme 15 slice pairs of 4 real products.
TENSOR_OPS_PER_FLOP = {"3xtf32": 3.0, "6xtf32": 6.0, "ozaki": 15.0}
# DRAM bytes of one exact-accumulation contraction step (row-exponent pass +
# GEMM) over its algorithmic bytes (|A| + |B| + |C| once), from an ncu
# capture of the dominant pair at a quarter height (M = 2^18, N = K = 256):
# the GEMM moves 1.032 GB against 1.025 GB algorithmic, and the exponent pass
# reads A (0.537 GB) once more.
OZ_CLASS_TRAFFIC_RATIO = (1.032 + 0.537) / 1.025
OZ_CLASS_TRAFFIC_SOURCE = ("k_oz_exp + k_oz_gemm DRAM bytes of the dominant pair at M = 2^18 (ncu), as a ratio "
                           "to algorithmic bytes, scaled to this class's average algorithmic bytes per launch")


# Nominal SIMT compute ceilings of a GB300 (not measured): FP32 = 152 SMs x
# 128 lanes x 2 flop x 2.07 GHz; FP64 at GB300's reduced rate.  Only the
# compute side of the SIMT kernel classes uses them; those classes are
# memory-bound at the circuit shapes here (K <= 16 per gate).
SIMT_TFLOPS = {"fp32": 152 * 128 * 2 * 2.07e9 / 1e12, "fp64": 1.25}


def roofline_from_profile(ms, batched, feats, peaks, peaks_kind, nchunks, prec_name=None, wall_ms=None):
    """Per-step lower bounds t_p = max(B_p / BW, F_p / P) (B_p = algorithmic
    bytes, each operand read once and the result written once at its storage
    size; F_p = 8 |C| K real flops; P = the measured bf16 peak for the
    tensor-core class, the nominal SIMT rate otherwise) against the measured
    per-step device times.  Returns (roofline of the dominant kernel class by
    device time, per-class summary, all-step summary).  The dominant class's
    ``bound`` is the side with the larger summed lower bound; ``achieved`` is
    its algorithmic bytes (or flops) over its measured time."""
    names = {0: "generic", 1: "gemm_simt", 2: "tcgen05", 3: "copy", 4: "skinny"}
    bw = peaks.get("hbm_gbs") * 1e9
    p_tc = peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops")) * 1e12
    p_simt = SIMT_TFLOPS["fp64" if prec_name == "c128" else "fp32"] * 1e12
    info = {}
    for t, b, f in zip(ms, batched, feats):
        k = int(f[6])
        d = info.setdefault(names.get(k, str(k)), {"ms_per_run": 0.0, "launches_per_run": 0, "flops": 0.0,
                                                    "bytes": 0.0, "hbm_bound_ms": 0.0, "compute_bound_ms": 0.0,
                                                    "lower_bound_ms": 0.0})
        rep = nchunks if b else 1
        F = 8.0 * 2 ** f[2] * 2 ** f[3] * rep
        B = f[7] * rep
        th, tcmp = 1e3 * B / bw, 1e3 * F / (p_tc if k == 2 else p_simt)
        d["ms_per_run"] += t * rep
        d["launches_per_run"] += rep
        d["flops"] += F
        d["bytes"] += B
        d["hbm_bound_ms"] += th
        d["compute_bound_ms"] += tcmp
        d["lower_bound_ms"] += max(th, tcmp)
    tot = sum(d["ms_per_run"] for d in info.values()) or 1.0
    for d in info.values():
        d["share"] = d["ms_per_run"] / tot
        d["lower_bound_frac"] = d["lower_bound_ms"] / d["ms_per_run"] if d["ms_per_run"] else None
    lb = sum(d["lower_bound_ms"] for d in info.values())
    overall = {"lower_bound_ms": lb, "device_ms": tot, "wall_ms": wall_ms,
               "frac_of_wall": lb / wall_ms if wall_ms else None,
               "rule": "sum over steps of max(B_p / measured HBM copy, F_p / P) over the measured time"}
    dom = max(info, key=lambda k: info[k]["ms_per_run"])
    d = info[dom]
    secs = d["ms_per_run"] / 1e3
    common = {"kernel": dom, "per_launch_ms": d["ms_per_run"] / d["launches_per_run"],
              "launches_per_run": d["launches_per_run"], "lower_bound_frac": d["lower_bound_frac"]}
    if d["hbm_bound_ms"] >= d["compute_bound_ms"]:
        ach = d["bytes"] / secs / 1e9
        roof = {"bound": "hbm", "achieved": ach, "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                "frac": ach / peaks.get("hbm_gbs"), "traffic": None, "peak_source": f"{peaks_kind} hbm copy",
                **common}
    elif dom == "tcgen05":
        ach = d["flops"] / secs / 1e12
        roof = {"bound": "tensor", "achieved": ach, "peak": p_tc / 1e12, "unit": "TFLOP/s", "frac": ach * 1e12 / p_tc,
                "traffic": None, "peak_source": f"{peaks_kind} bf16 sustained", **common}
    else:
        ach = d["flops"] / secs / 1e12
        roof = {"bound": "simt", "achieved": ach, "peak": p_simt / 1e12, "unit": "TFLOP/s",
                "frac": ach * 1e12 / p_simt, "traffic": None, "peak_source": "nominal SIMT", **common}
    if dom == "tcgen05":
        roof["kernel"] = "tcgen05 contraction steps (GEMM plus its scale / slice pre-passes)"
        roof["algorithmic_tflops"] = d["flops"] / secs / 1e12
        if prec_name in TENSOR_OPS_PER_FLOP:
            r = TENSOR_OPS_PER_FLOP[prec_name]
            roof.update({"tensor_ops_per_algorithmic_flop": r, "tensor_work_tflops": roof["algorithmic_tflops"] * r,
                         "tensor_work_frac": roof["algorithmic_tflops"] * r * 1e12 / p_tc})
        if prec_name == "ozaki":
            roof["traffic"] = d["bytes"] / d["launches_per_run"] * OZ_CLASS_TRAFFIC_RATIO
            roof["traffic_unit"] = "bytes per launch"
            roof["traffic_source"] = OZ_CLASS_TRAFFIC_SOURCE
    return roof, info, overall


if __name__ == "__main__":
    sys.exit(main())
