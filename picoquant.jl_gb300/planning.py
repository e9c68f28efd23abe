"""Whole-plan execution and planning on the GB300 backend.

* ``bgreedy`` / ``bgreedy_contraction`` — the flop-count planner
  (src/layer2/bgreedy_contraction.jl:17-66, 140-145) run natively in the
  library (``pq_plan_greedy``).
* ``NetworkPlan`` — a pair plan compiled once into kernel descriptors and an
  arena (``pq_plan_create``), executed from a CUDA graph, in slices with an
  FP64 compensated sum, or as many amplitudes of one circuit.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .contraction import _finish, contract_network
from .network import save_output


def _leaf_arrays(network, out_edges):
    """Leaves (current nodes, in ``network.nodes`` order) as integer-labelled
    arrays: returns (node_labels, ranks, flat_labels, label_dims, label_of)."""
    label_of: dict[str, int] = {}
    dims: list[int] = []
    be = network.backend
    nodes = list(network.nodes.keys())
    ranks, flat = [], []
    for nl in nodes:
        node = network.nodes[nl]
        shp = be.shape(node.data_label) if hasattr(be, "shape") else tuple(node.dims)
        if len(shp) != len(node.indices):
            raise ValueError(f"node {nl}: tensor rank {len(shp)} != {len(node.indices)} indices")
        ranks.append(len(node.indices))
        for idx, d in zip(node.indices, shp):
            if idx not in label_of:
                label_of[idx] = len(dims)
                dims.append(int(d))
            elif dims[label_of[idx]] != int(d):
                raise ValueError(f"index {idx} has extents {dims[label_of[idx]]} and {d}")
            flat.append(label_of[idx])
    for e in out_edges:
        if e not in label_of:
            raise ValueError(f"output index {e} is not on any node")
    return nodes, ranks, flat, dims, label_of


def open_output_edges(network):
    """The output wire labels in qubit order (as full_wavefunction_contraction!
    orders its result, src/layer2.jl:180), restricted to edges still open."""
    outs = [network.output_qubits[q - 1] for q in network.qubit_ordering]
    return [e for e in outs if network.edges[e].dst is None]


def greedy_steps(ranks, flat, dims, out_labels, alpha=1.0, tau=1.0, trials=10, seed=0):
    """Run the native Boltzmann-greedy planner; returns (steps, cmacs, max_elems)."""
    lib = L.lib()
    n = len(ranks)
    steps = (C.c_int32 * max(1, 2 * (n - 1)))()
    cm = C.c_double()
    mx = C.c_int64()
    rc = lib.pq_plan_greedy(n, L.arr(C.c_int32, ranks), L.arr(C.c_int32, flat), len(dims),
                            L.arr(C.c_int64, dims), len(out_labels), L.arr(C.c_int32, out_labels), float(alpha),
                            float(tau), int(trials), int(seed) & ((1 << 64) - 1), steps, C.byref(cm), C.byref(mx))
    L.check(rc, None, "pq_plan_greedy")
    return [int(x) for x in steps[: 2 * (n - 1)]], cm.value, mx.value


def greedy_draws(ranks, flat, dims, out_labels, n_draws, alpha=1.0, tau=1.0, seed=0, threads=0):
    """``n_draws`` independent native planner draws (draw 0 plain greedy, the
    others Boltzmann-sampled with ``tau``), run on host threads; returns a
    list of (steps, cmacs, max_elems)."""
    lib = L.lib()
    n = len(ranks)
    per = max(0, 2 * (n - 1))
    steps = (C.c_int32 * max(1, per * n_draws))()
    cm = (C.c_double * n_draws)()
    mx = (C.c_int64 * n_draws)()
    rc = lib.pq_plan_greedy_many(n, L.arr(C.c_int32, ranks), L.arr(C.c_int32, flat), len(dims),
                                 L.arr(C.c_int64, dims), len(out_labels), L.arr(C.c_int32, out_labels),
                                 float(alpha), float(tau), int(n_draws), int(seed) & ((1 << 64) - 1), int(threads),
                                 steps, cm, mx)
    L.check(rc, None, "pq_plan_greedy_many")
    flat_steps = [int(x) for x in steps[: per * n_draws]]
    return [(flat_steps[d * per:(d + 1) * per], cm[d], mx[d]) for d in range(n_draws)]


def steps_to_pairs(network, steps, leaves=None):
    """SSA steps -> pair plan of node labels as contract_pair! will name them
    (results are node_<counter+1>, node_<counter+2>, ...)."""
    leaves = leaves if leaves is not None else list(network.nodes.keys())
    names = list(leaves)
    base = network.counters["node"]
    plan = []
    for i in range(len(steps) // 2):
        plan.append([names[steps[2 * i]], names[steps[2 * i + 1]]])
        names.append(f"node_{base + i + 1}")
    return plan


def pairs_to_steps(network, plan, leaves=None):
    """Pair plan of node labels -> SSA steps over ``leaves``."""
    leaves = leaves if leaves is not None else list(network.nodes.keys())
    pos = {lab: i for i, lab in enumerate(leaves)}
    base = network.counters["node"]
    steps = []
    for i, (a, b) in enumerate(plan):
        steps += [pos[a], pos[b]]
        pos[f"node_{base + i + 1}"] = len(leaves) + i
    return steps


def bgreedy(network, alpha=1.0, tau=1.0, N=10, seed=0):
    """src/layer2/bgreedy_contraction.jl:163-176: best of N Boltzmann-greedy
    plans by cost.  Returns (pair plan, complex multiply-adds)."""
    outs = [e for e, v in network.edges.items() if v.src is None or v.dst is None]
    nodes, ranks, flat, dims, label_of = _leaf_arrays(network, outs)
    out_labels = [label_of[e] for e in outs if e in label_of]
    steps, cost, _ = greedy_steps(ranks, flat, dims, out_labels, alpha, tau, N, seed)
    return steps_to_pairs(network, steps, nodes), cost


def bgreedy_contraction(network, alpha=1.0, tau=1.0, N=10, output_shape="", seed=0):
    """src/layer2/bgreedy_contraction.jl:250-255."""
    plan, _ = bgreedy(network, alpha, tau, N, seed)
    return contract_network(network, plan, output_shape)


class NetworkPlan:
    """A compiled contraction of a network's current nodes.

    ``steps`` are SSA pairs over the leaves (node order of the network at
    construction); ``out_edges`` is the mode order of the result (default: the
    open output wires in qubit order).  The leaves' tensors stay in the backend
    and are not consumed, so the plan can be executed repeatedly.
    """

    def __init__(self, network, steps=None, out_edges=None, planner="greedy", trials=16, seed=0, alpha=1.0,
                 tau=1.0):
        self.network = network
        self.backend = network.backend
        self.lib = L.lib()
        if out_edges is None:
            out_edges = open_output_edges(network)
        self.out_edges = list(out_edges)
        nodes, ranks, flat, dims, label_of = _leaf_arrays(network, self.out_edges)
        self.leaves = nodes
        self.ranks, self.flat, self.dims, self.label_of = ranks, flat, dims, label_of
        self.out_labels = [label_of[e] for e in self.out_edges]
        if steps is None:
            if planner == "greedy":
                steps, _, _ = greedy_steps(ranks, flat, dims, self.out_labels, alpha, tau, trials, seed)
            elif planner == "wavefunction":
                steps = wavefunction_steps(network, nodes)
            else:
                raise ValueError(f"unknown planner {planner}")
        self.steps = list(steps)
        h = C.c_void_p()
        rc = self.lib.pq_plan_create(self.backend.ctx, len(ranks), L.arr(C.c_int32, ranks), L.arr(C.c_int32, flat),
                                     len(dims), L.arr(C.c_int64, dims), len(self.steps) // 2,
                                     L.arr(C.c_int32, self.steps), len(self.out_labels),
                                     L.arr(C.c_int32, self.out_labels), C.byref(h))
        L.check(rc, self.backend.ctx, "pq_plan_create")
        self.h = h
        self.leaf_ids = L.arr(C.c_int64, [self.backend.id_of(network.nodes[n].data_label) for n in nodes])
        self.out_label = "__plan_result__"

    def close(self):
        if getattr(self, "h", None):
            self.lib.pq_plan_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        cm = C.c_double()
        mx, ar, la = C.c_int64(), C.c_int64(), C.c_int64()
        L.check(self.lib.pq_plan_info(self.h, C.byref(cm), C.byref(mx), C.byref(ar), C.byref(la)),
                self.backend.ctx, "plan_info")
        return {"cmacs": cm.value, "max_elems": mx.value, "arena_bytes": ar.value, "launches": la.value,
                "steps": len(self.steps) // 2}

    def execute(self, out_label=None):
        """Run the plan; the result is stored under ``out_label`` (asynchronous)."""
        out = out_label or self.out_label
        L.check(self.lib.pq_plan_execute(self.h, self.leaf_ids, self.backend.id_of(out)), self.backend.ctx,
                "plan_execute")
        return out

    def capture(self, out_label=None):
        """Capture the plan into a CUDA graph (and run it once)."""
        out = out_label or self.out_label
        L.check(self.lib.pq_plan_capture(self.h, self.leaf_ids, self.backend.id_of(out)), self.backend.ctx,
                "plan_capture")
        return out

    def profile(self):
        """Per-step device time in milliseconds (CUDA events around each step)."""
        n = len(self.steps) // 2
        ms = (C.c_float * max(1, n))()
        L.check(self.lib.pq_plan_profile(self.h, self.leaf_ids, self.backend.id_of(self.out_label), ms),
                self.backend.ctx, "plan_profile")
        return np.array(ms[:n], dtype=np.float64)

    def features(self):
        n = len(self.steps) // 2
        f = (C.c_double * max(1, 8 * n))()
        L.check(self.lib.pq_plan_step_features(self.h, f), self.backend.ctx, "plan_step_features")
        return np.array(f[: 8 * n], dtype=np.float64).reshape(n, 8)

    def result(self, out_label=None):
        return self.backend.load_tensor_data(out_label or self.out_label)

    def amplitudes(self, bitstrings, dtype=np.complex128):
        """Execute and read the amplitudes of ``bitstrings`` (character i is the
        output of qubit ``qubit_ordering[i]``) from the open-output result."""
        out = self.execute()
        idx = bitstrings_to_index(bitstrings)
        return self.backend.gather(out, idx, dtype)

    def run_sliced(self, sliced_edges, batch=64, begin=0, end=None, reset=True):
        """Contract all slices over ``sliced_edges`` (each fixed to one value per
        slice) and return the FP64 compensated sum of the slice results."""
        lab = [self.label_of[e] for e in sliced_edges]
        total = 1
        for x in lab:
            total *= self.dims[x]
        end = total if end is None else end
        rc = self.lib.pq_plan_run_sliced(self.h, self.leaf_ids, len(lab), L.arr(C.c_int32, lab), int(begin),
                                         int(end), int(batch), 1 if reset else 0)
        L.check(rc, self.backend.ctx, "plan_run_sliced")
        n = 1
        for x in self.out_labels:
            n *= self.dims[x]
        out = np.empty(2 * n, dtype=np.float64)
        rc = self.lib.pq_sliced_result(self.h, out.ctypes.data_as(L.f64p), n)
        L.check(rc, self.backend.ctx, "sliced_result")
        res = out[0::2] + 1j * out[1::2]
        if not self.out_labels:
            return res[0]
        return res.reshape([self.dims[x] for x in self.out_labels], order="F")

    def profile_sliced(self, sliced_edges, batch=64):
        """Per-step device time (ms) of sliced execution for one batch of
        slices, whether each step runs per batch, and per-step features."""
        lab = [self.label_of[e] for e in sliced_edges]
        n = len(self.steps) // 2
        ms = (C.c_float * max(1, n))()
        bat = (C.c_int32 * max(1, n))()
        f = (C.c_double * max(1, 8 * n))()
        rc = self.lib.pq_plan_profile_sliced(self.h, self.leaf_ids, len(lab), L.arr(C.c_int32, lab), int(batch),
                                             ms, bat, f)
        L.check(rc, self.backend.ctx, "plan_profile_sliced")
        return (np.array(ms[:n], dtype=np.float64), np.array(bat[:n], dtype=bool),
                np.array(f[: 8 * n], dtype=np.float64).reshape(n, 8))

    def sliced_sizes(self, sliced_edges):
        """Per step: (log2 elements of the result for one slice, whether the
        step runs per slice)."""
        S = {self.label_of[e] for e in sliced_edges}
        labs, dep, pos = [], [], 0
        for r in self.ranks:
            l = self.flat[pos:pos + r]
            pos += r
            labs.append(l)
            dep.append(bool(set(l) & S))
        cnt: dict[int, int] = {}
        for l in labs:
            for x in l:
                cnt[x] = cnt.get(x, 0) + 1
        for x in self.out_labels:
            cnt[x] = cnt.get(x, 0) + 1
        out = []
        for i in range(len(self.steps) // 2):
            a, b = self.steps[2 * i], self.steps[2 * i + 1]
            for x in labs[a] + labs[b]:
                cnt[x] -= 1
            keep = [x for x in dict.fromkeys(labs[a] + labs[b]) if cnt[x] > 0]
            for x in keep:
                cnt[x] += 1
            labs.append(keep)
            dep.append(dep[a] or dep[b])
            out.append((sum(np.log2(self.dims[x]) for x in keep if x not in S), dep[-1]))
        return out

    def sliced_features(self, sliced_edges, batch):
        """Step features of the sliced execution (the cost model's inputs) and
        how often each step runs per amplitude: the sliced labels are fixed,
        steps that depend on a sliced leaf carry the batch of ``batch``
        slices as an extra mode and run once per batch, the others once.
        The unit-stride runs come from the unsliced plan."""
        base = self.features()
        S = {self.label_of[e] for e in sliced_edges}
        total = 1
        for x in S:
            total *= self.dims[x]
        nbatch = -(-total // batch) if S else 1
        lb = float(np.log2(batch)) if S else 0.0
        l2 = [float(np.log2(d)) for d in self.dims]
        labs, dep, pos = [], [], 0
        for r in self.ranks:
            ll = self.flat[pos:pos + r]
            pos += r
            labs.append(ll)
            dep.append(bool(set(ll) & S))
        cnt: dict[int, int] = {}
        for ll in labs:
            for x in ll:
                cnt[x] = cnt.get(x, 0) + 1
        for x in self.out_labels:
            cnt[x] = cnt.get(x, 0) + 1
        feats = np.array(base, dtype=np.float64)
        reps = np.ones(len(self.steps) // 2)
        for i in range(len(self.steps) // 2):
            a, b = self.steps[2 * i], self.steps[2 * i + 1]
            for x in labs[a] + labs[b]:
                cnt[x] -= 1
            union = list(dict.fromkeys(labs[a] + labs[b]))
            keep = [x for x in union if cnt[x] > 0]
            for x in keep:
                cnt[x] += 1
            labs.append(keep)
            dep.append(dep[a] or dep[b])
            size = lambda ls: sum(l2[x] for x in ls if x not in S)
            feats[i, 0] = size(labs[a]) + (lb if dep[a] else 0.0)
            feats[i, 1] = size(labs[b]) + (lb if dep[b] else 0.0)
            feats[i, 2] = size(keep) + (lb if dep[-1] else 0.0)
            feats[i, 3] = sum(l2[x] for x in union if x not in keep and x not in S)
            reps[i] = nbatch if dep[-1] else 1
        return feats, reps

    def auto_batch(self, sliced_edges, budget_bytes=32 << 30, max_batch=1024):
        """Largest power-of-two batch of slices whose per-slice intermediates
        (three live at a time, at most) fit in ``budget_bytes``."""
        elem = 16 if self.backend.precision == L.PREC_C128 else 8
        big = max([s for s, b in self.sliced_sizes(sliced_edges) if b] or [0.0])
        total = 1
        for e in sliced_edges:
            total *= self.dims[self.label_of[e]]
        b = 1
        while b * 2 <= min(max_batch, total) and 3 * elem * (2 ** big) * b * 2 <= budget_bytes:
            b *= 2
        return b

    def choose_slices(self, max_sliced=10, log2_target=0.0):
        """Labels (edge names) the slice chooser picks for this plan."""
        out = (C.c_int32 * max(1, max_sliced))()
        n = C.c_int()
        rc = self.lib.pq_plan_choose_slices(len(self.ranks), L.arr(C.c_int32, self.ranks),
                                            L.arr(C.c_int32, self.flat), len(self.dims),
                                            L.arr(C.c_int64, self.dims), len(self.steps) // 2,
                                            L.arr(C.c_int32, self.steps), len(self.out_labels),
                                            L.arr(C.c_int32, self.out_labels), int(max_sliced), float(log2_target),
                                            out, C.byref(n))
        L.check(rc, None, "pq_plan_choose_slices")
        inv = {v: k for k, v in self.label_of.items()}
        return [inv[out[i]] for i in range(n.value)]


def slice_range(total, rank, world):
    """Contiguous, balanced share [begin, end) of ``total`` slices for rank
    ``rank`` of ``world`` (the multi-GPU split of a sliced contraction: each
    rank runs ``NetworkPlan.run_sliced(..., begin, end)`` and one reduction
    of the partial sums finishes the amplitude, as the reference's
    examples/dist_slicing_example.jl:30 reduces partition results)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(int(total), int(world))
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def bitstrings_to_index(bitstrings):
    """Column-major linear index of each bitstring (character i -> bit i)."""
    out = np.empty(len(bitstrings), dtype=np.int64)
    for j, b in enumerate(bitstrings):
        v = 0
        for i, ch in enumerate(b):
            if ch == "1":
                v |= 1 << i
        out[j] = v
    return out


def plan_cost(ranks, flat, dims, steps, out_labels):
    """Complex multiply-adds and largest intermediate (elements) of SSA steps,
    with the label rule of the executor (a label is summed once no other live
    tensor and no output carries it); computed natively (``pq_plan_cost``)."""
    lib = L.lib()
    cm, mx = C.c_double(), C.c_double()
    i32 = [np.ascontiguousarray(np.asarray(v, dtype=np.int64).reshape(-1), dtype=np.int32)
           if len(v) else np.zeros(1, np.int32) for v in (ranks, flat, steps, out_labels)]
    d64 = np.ascontiguousarray(np.asarray(dims, dtype=np.int64).reshape(-1)) if len(dims) else np.zeros(1, np.int64)
    p32 = [a.ctypes.data_as(L.i32p) for a in i32]
    rc = lib.pq_plan_cost(len(ranks), p32[0], p32[1], len(dims), d64.ctypes.data_as(L.i64p), len(steps) // 2, p32[2],
                          len(out_labels), p32[3], C.byref(cm), C.byref(mx))
    L.check(rc, None, "pq_plan_cost")
    return cm.value, mx.value


def device_backend(network):
    """The network's backend when it has a device context (candidate plans
    are then scored on the device), else None."""
    be = network.backend
    return be if getattr(be, "ctx", None) is not None and hasattr(be, "lib") else None


def plan_cost_batch(backend, ranks, flat, dims, step_lists, out_labels):
    """(cmacs, max_elems) of many SSA plans of the same leaves, scored on the
    backend's device in one launch (``pq_plan_cost_batch``: one warp per
    plan, the executor's label rule); the values of ``plan_cost``."""
    lib = L.lib()
    n = len(step_lists)
    if n == 0:
        return []
    ns = len(step_lists[0]) // 2
    if any(len(st) != 2 * ns for st in step_lists):
        raise ValueError("plans of one network have the same number of steps")
    st = np.ascontiguousarray(np.asarray(step_lists, dtype=np.int32).reshape(-1) if ns else np.zeros(1, np.int32))
    a32 = [np.ascontiguousarray(np.asarray(v, dtype=np.int64).reshape(-1), dtype=np.int32)
           if len(v) else np.zeros(1, np.int32) for v in (ranks, flat, out_labels)]
    d64 = np.ascontiguousarray(np.asarray(dims, dtype=np.int64).reshape(-1)) if len(dims) else np.zeros(1, np.int64)
    cm = np.empty(n, np.float64)
    mx = np.empty(n, np.float64)
    rc = lib.pq_plan_cost_batch(backend.ctx, len(ranks), a32[0].ctypes.data_as(L.i32p), a32[1].ctypes.data_as(L.i32p),
                                len(dims), d64.ctypes.data_as(L.i64p), ns, n, st.ctypes.data_as(L.i32p),
                                len(out_labels), a32[2].ctypes.data_as(L.i32p), cm.ctypes.data_as(L.f64p),
                                mx.ctypes.data_as(L.f64p))
    L.check(rc, backend.ctx, "pq_plan_cost_batch")
    return list(zip(cm.tolist(), mx.tolist()))


def _node_qubit(network, node_label):
    for idx in network.nodes[node_label].indices:
        e = network.edges.get(idx)
        if e is not None and not e.virtual and e.qubit is not None:
            return e.qubit
    return None


def sweep_steps(network, leaves=None, out_labels=None, label_of=None, ranks=None, flat=None, dims=None,
                all_orders=False, random_orders=0, keep_random=4, seed=0, cost_backend=None):
    """Qubit-sweep plan: contract each qubit's tensors along time into one
    tensor, then absorb qubits one at a time into a growing boundary.

    Several qubit orders are tried (natural and reversed order, and greedy
    smallest-boundary orders started from a few qubits); with
    ``random_orders``, that many seeded randomized boundary-greedy orders too
    (a random start, each next qubit drawn with weight 2^(-boundary / T) over
    the frontier, T cycling through 0.3, 0.7, 1.5 in log2 elements), of which
    the ``keep_random`` cheapest are kept.  The cheapest by complex
    multiply-adds is returned as (steps, cmacs, max_elems), or every kept
    order's triple when ``all_orders``.  With ``cost_backend`` (a backend with
    a device context) the candidates are scored together on the device
    (``plan_cost_batch``).
    """
    leaves = leaves if leaves is not None else list(network.nodes.keys())
    groups: dict[int, list] = {}
    for i, nl in enumerate(leaves):
        q = _node_qubit(network, nl)
        groups.setdefault(q if q is not None else 0, []).append(i)
    qs = sorted(groups)
    pos = 0
    labs = []
    for r in ranks:
        labs.append(list(flat[pos:pos + r]))
        pos += r
    outset = set(out_labels)
    # chain contraction inside each group (in leaf order = circuit order)
    base_steps = []
    nxt = len(leaves)
    group_val = {}
    cnt: dict[int, int] = {}
    for l in labs:
        for x in l:
            cnt[x] = cnt.get(x, 0) + 1
    glabels = {}
    for q in qs:
        members = groups[q]
        v = members[0]
        for m in members[1:]:
            base_steps += [v, m]
            v = nxt
            nxt += 1
        group_val[q] = v
        ls = set()
        for m in members:
            ls.update(labs[m])
        glabels[q] = ls
    # labels internal to a group disappear; the group tensor keeps labels that
    # leave the group or are outputs
    ngroups: dict[int, int] = {}
    for q in qs:
        for x in glabels[q]:
            ngroups[x] = ngroups.get(x, 0) + 1
    ext = {q: {x for x in glabels[q] if ngroups[x] > 1 or x in outset} for q in qs}
    l2 = [float(np.log2(d)) for d in dims]
    owners: dict[int, list] = {}
    for q in qs:
        for x in ext[q]:
            owners.setdefault(x, []).append(q)
    adj = {q: set() for q in qs}
    for x, ow in owners.items():
        for q in ow:
            adj[q].update(p for p in ow if p != q)

    def greedy_order(start, rng=None, temp=1.0):
        # the boundary after absorbing a set of groups: the labels of absorbed
        # groups still held by an unabsorbed group or open; rem[x] counts the
        # unabsorbed groups holding x, so one candidate's boundary is the
        # current one plus a change over its own labels
        rem = {x: len(ow) for x, ow in owners.items()}
        bnd: set = set()
        cur = 0.0

        def absorb(c):
            nonlocal cur
            for x in ext[c]:
                rem[x] -= 1
                if x in bnd:
                    if rem[x] == 0 and x not in outset:
                        bnd.discard(x)
                        cur -= l2[x]
                elif rem[x] > 0 or x in outset:
                    bnd.add(x)
                    cur += l2[x]

        def after(c):
            d = 0.0
            for x in ext[c]:
                if x in bnd:
                    if rem[x] == 1 and x not in outset:
                        d -= l2[x]
                elif rem[x] > 1 or x in outset:
                    d += l2[x]
            return cur + d

        order = [start]
        absorbed = {start}
        absorb(start)
        front = set(adj[start])
        while len(order) < len(qs):
            cands = front - absorbed
            if not cands:
                cands = set(qs) - absorbed
            best, bl = None, None
            if rng is None:
                for c in sorted(cands):
                    b = after(c)
                    if bl is None or b < bl - 1e-9:
                        best, bl = c, b
            else:
                cs = sorted(cands)
                b = np.array([after(c) for c in cs])
                w = np.exp2(-(b - b.min()) / temp)
                best = cs[int(rng.choice(len(cs), p=w / w.sum()))]
            order.append(best)
            absorbed.add(best)
            absorb(best)
            front |= adj[best]
        return order

    orders = [list(qs), list(reversed(qs))]
    nq = len(qs)
    starts = [qs[0], qs[-1], qs[nq // 2], qs[nq // 4], qs[(3 * nq) // 4]]
    for s in dict.fromkeys(starts):
        orders.append(greedy_order(s))
    def order_steps(order):
        steps = list(base_steps)
        n2 = nxt
        v = group_val[order[0]]
        for q in order[1:]:
            steps += [v, group_val[q]]
            v = n2
            n2 += 1
        return steps

    def costs(step_lists):
        # every candidate's (cmacs, max_elems): one device batch when a
        # backend context is given, else one native host pass each
        if cost_backend is not None and len(step_lists) > 1:
            return plan_cost_batch(cost_backend, ranks, flat, dims, step_lists, out_labels)
        return [plan_cost(ranks, flat, dims, st, out_labels) for st in step_lists]

    step_lists = [order_steps(order) for order in orders]
    found = [(st, *cm) for st, cm in zip(step_lists, costs(step_lists))]
    if random_orders > 0:
        rng = np.random.default_rng(seed)
        temps = (0.3, 0.7, 1.5)
        seen = {tuple(o) for o in orders}
        extra_steps = []
        for i in range(random_orders):
            o = greedy_order(qs[int(rng.integers(nq))], rng, temps[i % len(temps)])
            if tuple(o) in seen:
                continue
            seen.add(tuple(o))
            extra_steps.append(order_steps(o))
        extra = [(st, *cm) for st, cm in zip(extra_steps, costs(extra_steps))]
        extra.sort(key=lambda t: (t[1], t[2]))
        found += extra[:keep_random]
    if all_orders:
        return found
    return min(found, key=lambda t: (t[1], t[2]))


def best_flop_plan(network, out_edges=None, trials=16, seed=0, candidates=("sweep", "greedy", "wavefunction"),
                   sweep_random=0):
    """The flop-count planner: the cheapest (complex multiply-adds) of the
    candidate plans ("sweep", "greedy", "wavefunction" and the gate-by-gate
    "statevector" order); ``sweep_random`` randomized qubit-sweep orders join
    the sweep candidates (``sweep_steps``).  Returns (steps, cmacs, max_elems,
    name)."""
    if out_edges is None:
        out_edges = open_output_edges(network)
    nodes, ranks, flat, dims, label_of = _leaf_arrays(network, out_edges)
    outl = [label_of[e] for e in out_edges]
    found = []
    if "greedy" in candidates:
        s, c, m = greedy_steps(ranks, flat, dims, outl, 1.0, 1.0, trials, seed)
        found.append((s, *plan_cost(ranks, flat, dims, s, outl), "greedy"))
    if "sweep" in candidates:
        s, c, m = sweep_steps(network, nodes, outl, label_of, ranks, flat, dims, random_orders=sweep_random,
                              seed=seed, cost_backend=device_backend(network))
        found.append((s, c, m, "sweep"))
    if "wavefunction" in candidates and all(network.edges[e].src is not None for e in network.input_qubits):
        try:
            s = wavefunction_steps(network, nodes)
            found.append((s, *plan_cost(ranks, flat, dims, s, outl), "wavefunction"))
        except KeyError:
            pass
    if "statevector" in candidates and all(network.edges[e].src is not None for e in network.input_qubits):
        s = statevector_steps(network, nodes)
        found.append((s, *plan_cost(ranks, flat, dims, s, outl), "statevector"))
    return min(found, key=lambda t: (t[1], t[2]))


def statevector_steps(network, leaves=None):
    """SSA steps of a gate-by-gate state-vector order: the input vectors
    folded into the state, then every gate node applied to the state in
    creation (circuit) order, then the output vectors if any.  Unlike the
    reference's layer order it never contracts a layer's gates together
    first, so no intermediate exceeds the state's size."""
    leaves = leaves if leaves is not None else list(network.nodes.keys())
    pos = {lab: i for i, lab in enumerate(leaves)}
    inputs = [pos[network.edges[e].src] for e in network.input_qubits]
    steps = []
    wf = inputs[0]
    nxt = len(leaves)
    for w in inputs[1:]:
        steps += [wf, w]
        wf = nxt
        nxt += 1
    in_set = set(inputs)
    outs = [i for i, lab in enumerate(leaves) if network.node_layers.get(lab) == -1]
    for i, lab in enumerate(leaves):
        if i in in_set or i in outs:
            continue
        steps += [wf, i]
        wf = nxt
        nxt += 1
    for o in outs:
        steps += [wf, o]
        wf = nxt
        nxt += 1
    return steps


def wavefunction_steps(network, leaves=None):
    """SSA steps of the reference's default full-wavefunction order
    (src/layer2.jl:132-173): inputs folded left to right, then per layer the
    layer's nodes contracted together and applied to the wavefunction."""
    leaves = leaves if leaves is not None else list(network.nodes.keys())
    pos = {lab: i for i, lab in enumerate(leaves)}
    nxt = [len(leaves)]
    steps = []

    def pair(a, b):
        steps.extend([a, b])
        r = nxt[0]
        nxt[0] += 1
        return r

    inputs = [pos[network.edges[e].src] for e in network.input_qubits]
    wf = inputs[0]
    for w in inputs[1:]:
        wf = pair(wf, w)
    groups: dict[int, list] = {}
    for k, v in network.node_layers.items():
        if k in pos:
            groups.setdefault(v, []).append(k)
    order = [k for k in sorted(groups) if k > 0]
    if -1 in groups:
        order.append(-1)
    for layer in order:
        nodes = [pos[x] for x in groups[layer]]
        n = nodes[0]
        for n2 in nodes[1:]:
            n = pair(n, n2)
        wf = pair(wf, n)
    return steps
