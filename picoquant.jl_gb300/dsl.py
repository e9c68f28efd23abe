"""The DSL: the reference's text wire format for whole contraction plans.

``DSLBackend`` (src/backends/dsl.jl:14-214) records the backend calls of a
network contraction as DSL lines instead of executing them;
``execute_dsl_file`` (src/layer1.jl:211-330) replays a DSL script on any
backend (the GB300 backend by default); ``compile_dsl`` turns a script made
only of ``tensor`` / ``ncon`` / ``del`` / ``save`` lines -- what
``contract_network`` records -- into one compiled plan, which can be captured
as a CUDA graph and run again without re-reading the script.

Line formats (kept alike so scripts move between the two implementations):

    tensor <label> <dataset>
    ncon <C> <A> <i,j,..> <B> <k,l,..>        (+n contracted, -n open; C's modes in
                                              symdiff(ia, ib) order, src/layer1.jl:89)
    del <label>
    save <label> <file> <group>
    reshape <label> <a,b;c;..>                (1-based axis groups)
    permute <label> <a,b,..>                  (1-based)
    decompose <A> <B> <i,..> <C> <j,..> {"threshold":t, "max_rank":r}
    view <view> <node> <bond_idx> <lo,..,hi>

Tensor data: the reference stores it in HDF5 (HDF5.jl); no HDF5 library is
available to this package, so datasets are numpy arrays in a ``.npz`` file
(or a mapping passed directly), keyed by dataset name, column-major.
"""
from __future__ import annotations

import ctypes as C
import json
import os

import numpy as np

from . import _lib as L
from .backend import Metrics


def _ints(s):
    return [int(x) for x in s.split(",") if x != ""]


class DSLBackend:
    """src/backends/dsl.jl:14-214: every backend call appends a DSL line;
    tensor data go to ``self.data`` (written to ``tensor_data`` as .npz by
    ``flush``).  ``decompose_tensor`` returns 0 like the reference (the bond
    extent is known only when the script runs)."""

    def __init__(self, dsl="contract_network.tl", tensor_data="tensor_data.npz", output="", overwrite=False):
        self.dsl_filename = dsl
        self.tensor_data_filename = tensor_data
        self.output_data_filename = output or tensor_data
        self.metrics = Metrics()
        self.data: dict[str, np.ndarray] = {}
        self.outputs: dict[str, np.ndarray] = {}
        if overwrite or not os.path.exists(dsl):
            open(dsl, "w").close()

    def push(self, instruction):
        with open(self.dsl_filename, "a") as f:
            f.write(instruction + "\n")

    def flush(self):
        np.savez(self.tensor_data_filename, **self.data)

    def shape(self, label):
        return np.asarray(self.data[str(label)]).shape

    def save_tensor_data(self, label, data):
        label = str(label)
        self.data[label] = np.asarray(data, dtype=np.complex128)
        self.push(f"tensor {label} {label}")

    def load_tensor_data(self, label):
        label = str(label)
        if label == "result":
            return self.outputs.get(label)
        return self.data.get(label)

    def contract_tensors(self, A, ia, B, ib, C):
        self.push(f"ncon {C} {A} {','.join(map(str, ia))} {B} {','.join(map(str, ib))}")
        self.push(f"del {A}")
        self.push(f"del {B}")

    def save_output(self, node, name="result"):
        self.push(f"save {node} {self.output_data_filename} {name}")

    def reshape_tensor(self, tensor, groups):
        self.push(f"reshape {tensor} " + ";".join(",".join(map(str, g)) for g in groups))

    def permute_tensor(self, tensor, axes):
        self.push(f"permute {tensor} " + ",".join(map(str, axes)))

    def decompose_tensor(self, tensor, left_positions, right_positions, threshold=1e-13, max_rank=0,
                         left_label=None, right_label=None):
        self.push(f"decompose {tensor} {left_label} {','.join(map(str, left_positions))} {right_label} "
                  f"{','.join(map(str, right_positions))} " + json.dumps({"threshold": threshold,
                                                                          "max_rank": max_rank}))
        return 0

    def delete_tensor(self, tensor):
        self.push(f"del {tensor}")

    def view_tensor(self, view_node, node, bond_idx, bond_range):
        if isinstance(bond_range, range):
            vals = list(bond_range)
        else:
            lo, hi = bond_range
            vals = list(range(lo, hi + 1))
        self.push(f"view {view_node} {node} {bond_idx} {','.join(map(str, vals))}")


def _read_data(tensor_data):
    if isinstance(tensor_data, (str, os.PathLike)):
        with np.load(tensor_data) as z:
            return {k: z[k] for k in z.files}
    return dict(tensor_data)


def _lines(dsl):
    if isinstance(dsl, (str, os.PathLike)) and os.path.exists(dsl):
        with open(dsl) as f:
            text = f.read()
    else:
        text = str(dsl)
    return [ln.split() for ln in text.splitlines() if ln.strip()]


def execute_dsl_file(dsl_filename="contract_network.tl", tensor_data="tensor_data.npz", backend=None,
                     output_data_filename=""):
    """src/layer1.jl:211-315: run every line of a DSL script on ``backend``
    (default: a complex128 GB300 backend, the reference's
    ``Array{ComplexF64}``); returns the saved outputs {group: array} (also
    written to ``output_data_filename`` as .npz when one is given)."""
    own = backend is None
    if own:
        from .backend import GB300Backend

        backend = GB300Backend(L.PREC_C128)
    data = _read_data(tensor_data)
    outputs = {}
    try:
        for cmd in _lines(dsl_filename):
            op = cmd[0]
            if op == "ncon":
                c_l, a_l, a_i, b_l, b_i = cmd[1:6]
                backend.contract_tensors(a_l, _ints(a_i), b_l, _ints(b_i), c_l)
            elif op == "del":
                backend.delete_tensor(cmd[1])
            elif op == "tensor":
                backend.save_tensor_data(cmd[1], data[cmd[2]])
            elif op == "save":
                outputs[cmd[3]] = backend.load_tensor_data(cmd[1])
            elif op == "reshape":
                groups = [_ints(g) for g in cmd[2].split(";")]
                backend.reshape_tensor(cmd[1], groups)
            elif op == "permute":
                backend.permute_tensor(cmd[1], _ints(cmd[2]))
            elif op == "decompose":
                a_l, b_l, b_i, c_l, c_i = cmd[1:6]
                opts = json.loads("".join(cmd[6:])) if len(cmd) > 6 else {}
                backend.decompose_tensor(a_l, _ints(b_i), _ints(c_i), threshold=opts.get("threshold", 1e-13),
                                         max_rank=opts.get("max_rank", 0), left_label=b_l, right_label=c_l)
            elif op == "view":
                vals = _ints(cmd[4])
                backend.view_tensor(cmd[1], cmd[2], int(cmd[3]), (min(vals), max(vals)))
            else:
                raise ValueError(f"unknown DSL command {op!r}")
    finally:
        if own:
            backend.close()
    if output_data_filename:
        np.savez(output_data_filename, **{k: np.asarray(v) for k, v in outputs.items()})
    return outputs


class DSLPlan:
    """A script of ``tensor`` / ``ncon`` / ``del`` / ``save`` lines compiled
    to one plan on a GB300 backend: the leaves are the script's tensors (kept,
    not consumed), the SSA steps its ncon lines, the result the tensor of the
    last ``save`` in its mode order.  ``run()`` executes it (``capture=True``
    first records it as a CUDA graph) and returns the saved array."""

    def __init__(self, lines, data, backend):
        self.backend = backend
        self.lib = L.lib()
        leaf_of: dict[str, int] = {}   # DSL label -> SSA value
        leaves: list[str] = []
        modes: dict[int, list[int]] = {}  # SSA value -> mode position ids
        parent: list[int] = []            # union-find over mode positions
        extent: list[int] = []

        def new_pos(d):
            parent.append(len(parent))
            extent.append(int(d))
            return len(parent) - 1

        def find(x):
            while parent[x] != x:
                parent[x] = parent[parent[x]]
                x = parent[x]
            return x

        steps: list[int] = []
        saved = None
        for cmd in lines:
            if cmd[0] not in ("tensor", "ncon", "del", "save"):
                raise ValueError(f"compile_dsl: {cmd[0]!r} lines are not compiled (run the script with "
                                 "execute_dsl_file)")
        pending = lines
        ds = {}  # leaf label -> dataset name
        for cmd in pending:
            if cmd[0] == "tensor":
                leaves.append(cmd[1])
                leaf_of[cmd[1]] = len(leaves) - 1
                ds[cmd[1]] = cmd[2]
        for i, lab in enumerate(leaves):
            modes[i] = [new_pos(d) for d in np.asarray(data[ds[lab]]).shape]
        nxt = len(leaves)
        live = dict(leaf_of)
        for cmd in pending:
            if cmd[0] == "ncon":
                c_l, a_l, a_i, b_l, b_i = cmd[1:6]
                va, vb = live.pop(a_l), live.pop(b_l)
                ia, ib = _ints(a_i), _ints(b_i)
                ma, mb = modes[va], modes[vb]
                if len(ia) != len(ma) or len(ib) != len(mb):
                    raise ValueError(f"compile_dsl: rank mismatch in ncon {c_l}")
                for x, pa in zip(ia, ma):
                    if x > 0:
                        pb = mb[ib.index(x)]
                        if extent[pa] != extent[pb]:
                            raise ValueError(f"compile_dsl: extent mismatch on ncon index {x}")
                        parent[find(pa)] = find(pb)
                # result modes in symdiff(ia, ib) order (src/layer1.jl:89): A's open
                # modes in A order, then B's
                steps += [va, vb]
                modes[nxt] = [p for x, p in zip(ia, ma) if x < 0] + [p for x, p in zip(ib, mb) if x < 0]
                live[c_l] = nxt
                nxt += 1
            elif cmd[0] == "del":
                live.pop(cmd[1], None)
            elif cmd[0] == "save":
                saved = (live[cmd[1]], cmd[3])
        if saved is None or saved[0] != nxt - 1:
            raise ValueError("compile_dsl: the script must save the result of its last ncon")
        # integer labels: one per class of mode positions joined by ncon
        roots: dict[int, int] = {}
        dims: list[int] = []

        def label(p):
            r = find(p)
            if r not in roots:
                roots[r] = len(dims)
                dims.append(extent[r])
            return roots[r]

        self.ranks = [len(modes[i]) for i in range(len(leaves))]
        self.flat = [label(p) for i in range(len(leaves)) for p in modes[i]]
        self.out_labels = [label(p) for p in modes[nxt - 1]]
        self.dims, self.steps, self.group = dims, steps, saved[1]
        self.leaf_labels = leaves
        for lab in leaves:
            backend.save_tensor_data(lab, data[ds[lab]])
        h = C.c_void_p()
        rc = self.lib.pq_plan_create(backend.ctx, len(self.ranks), L.arr(C.c_int32, self.ranks),
                                     L.arr(C.c_int32, self.flat), len(dims), L.arr(C.c_int64, dims),
                                     len(steps) // 2, L.arr(C.c_int32, steps), len(self.out_labels),
                                     L.arr(C.c_int32, self.out_labels), C.byref(h))
        L.check(rc, backend.ctx, "pq_plan_create")
        self.h = h
        self.leaf_ids = L.arr(C.c_int64, [backend.id_of(lab) for lab in leaves])
        self.out = "__dsl_result__"

    def run(self, capture=False):
        fn = self.lib.pq_plan_capture if capture else self.lib.pq_plan_execute
        L.check(fn(self.h, self.leaf_ids, self.backend.id_of(self.out)), self.backend.ctx, "dsl plan")
        return self.backend.load_tensor_data(self.out)

    def close(self):
        if getattr(self, "h", None):
            self.lib.pq_plan_destroy(self.h)
            self.h = None


def compile_dsl(dsl_filename, tensor_data, backend):
    """Compile a tensor/ncon/del/save DSL script to a ``DSLPlan``."""
    return DSLPlan(_lines(dsl_filename), _read_data(tensor_data), backend)
