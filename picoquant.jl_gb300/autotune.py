"""Autotuner: the fastest kernel choice per tuning class, measured on this GPU.

The reference has no counterpart: its array library picks kernels
internally (TensorOperations -> BLAS / cuTENSOR, src/layer1.jl:85-92).  Here
the library's fixed rules (``analyse_pair`` in pq_analyse.cpp, the tile
width and orientation rules of the exact-accumulation class in pq_oz.cu)
are the defaults, and this module times the alternatives.

A tuning class (``pq_pair_tuning``) is a pair's precision mode, the
ceil-log2 of its M (A-side free), N (B-side free), K (contracted) and batch
extents, and whether A's / B's unit-stride mode is contracted.  For each class
met by the pairs given (for instance every step of a compiled plan), every
eligible choice -- kernel class, and for the exact-accumulation tensor-core
class a tile width of 16 to 128 columns and an orientation -- is timed by the
library's own harness (``pq_measure_pairs``, CUDA events, random operands of
the pair's shape), the default included: one quick pass over all choices,
then ``reps`` timed runs of the three fastest and the default.  The fastest
replaces the default only when it is at least 5 % faster (closer timings are
noise, and a change of kernel class can change the rounding); the choice is
installed in the context (``pq_ctx_set_tuning``), which every later contraction, plan
compile and measurement on it consults, and the table is persisted as JSON
keyed by the GPU's name and a hash of the kernel sources (a cache written for
other kernels or another GPU is ignored).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import re
from pathlib import Path

import numpy as np

from . import _lib as L
from .costmodel import measure_pairs

PKG_DIR = Path(__file__).resolve().parent
CACHE_DIR = PKG_DIR / "tuning"
KCLASS = {0: "generic", 1: "gemm_simt", 2: "tcgen05", 4: "skinny"}


def source_hash() -> str:
    """Hash of the kernel and ABI sources: a tuned table is valid for them only."""
    h = hashlib.sha256()
    files = sorted(p for p in (PKG_DIR / "csrc").iterdir() if p.suffix in (".cu", ".cuh", ".cpp", ".h"))
    for p in files + [PKG_DIR.parent / "include" / "pqgb300.h"]:
        h.update(p.name.encode())
        h.update(p.read_bytes())
    return h.hexdigest()[:16]


def device_name(device: int = 0) -> str:
    buf = C.create_string_buffer(256)
    L.check(L.lib().pq_device_name(int(device), buf, 256), None, "pq_device_name")
    return buf.value.decode()


def cache_path(device: int = 0) -> Path:
    return CACHE_DIR / (re.sub(r"[^A-Za-z0-9]+", "_", device_name(device)).strip("_") + ".json")


def choice_name(c) -> str:
    k, tn, o = (int(x) for x in c)
    s = KCLASS.get(k, str(k))
    if k == 2 and (tn or o):
        s += f"/tn{tn or 'auto'}/{'as_given' if o == 1 else 'swapped' if o == 2 else 'auto'}"
    return s


def plan_pairs(plan):
    """Operand labels and extents of every step of a compiled plan, as
    (a_labels, a_dims, b_labels, b_dims), following the executor's label
    rule; steps that keep a shared (hyper) label are left out (the harness
    sums every shared label)."""
    labs, pos = [], 0
    for r in plan.ranks:
        labs.append(list(plan.flat[pos:pos + r]))
        pos += r
    cnt: dict[int, int] = {}
    for lab in labs:
        for x in lab:
            cnt[x] = cnt.get(x, 0) + 1
    for x in plan.out_labels:
        cnt[x] = cnt.get(x, 0) + 1
    out = []
    for i in range(len(plan.steps) // 2):
        la, lb = labs[plan.steps[2 * i]], labs[plan.steps[2 * i + 1]]
        for x in la + lb:
            cnt[x] -= 1
        keep = [x for x in dict.fromkeys(la + lb) if cnt[x] > 0]
        for x in keep:
            cnt[x] += 1
        labs.append(keep)
        if not any(x in lb and x in keep for x in la):
            out.append((la, [plan.dims[x] for x in la], lb, [plan.dims[x] for x in lb]))
    return out


class Tuner:
    """Per-class tuned choices for one backend context (see the module doc)."""

    def __init__(self, backend, margin=0.05):
        self.be = backend
        self.margin = margin  # a choice must beat the default by this fraction to replace it
        self.entries: dict[int, dict] = {}

    # ---- library calls ------------------------------------------------------
    def classify(self, la, da, lb, db):
        """(tuning key, eligible choices with the default first) of C = A x B."""
        lab = np.ascontiguousarray(list(la) + list(lb), dtype=np.int32)
        dims = np.ascontiguousarray(list(da) + list(db), dtype=np.int64)
        key = C.c_uint64()
        ch = (C.c_int32 * 96)()
        n = C.c_int()
        rc = self.be.lib.pq_pair_tuning(self.be.ctx, len(la), len(lb), lab.ctypes.data_as(L.i32p),
                                        dims.ctypes.data_as(L.i64p), C.byref(key), 32, ch, C.byref(n))
        L.check(rc, self.be.ctx, "pq_pair_tuning")
        return int(key.value), [tuple(ch[3 * i:3 * i + 3]) for i in range(min(n.value, 32))]

    def install(self, extra=None):
        """Install the tuned table (plus ``extra`` {key: choice}) in the context."""
        table = {k: tuple(e["choice"]) for k, e in self.entries.items()}
        if extra:
            table.update(extra)
        keys = (C.c_uint64 * max(1, len(table)))(*table.keys())
        ch = L.arr(C.c_int32, [x for c in table.values() for x in c])
        L.check(self.be.lib.pq_ctx_set_tuning(self.be.ctx, len(table), keys, ch), self.be.ctx, "pq_ctx_set_tuning")

    def _time(self, key, choice, shape, reps):
        self.install({key: choice})
        ms, _ = measure_pairs(self.be, shape, reps=reps)
        return float(ms[0])

    # ---- tuning ---------------------------------------------------------------
    def tune_pair(self, la, da, lb, db, reps=5, force=False):
        """Tune the class of one pair (random operands of its shape); returns
        its key.  Classes already in the table are skipped unless ``force``."""
        key, cands = self.classify(la, da, lb, db)
        if (key in self.entries and not force) or len(cands) <= 1:
            return key
        shape = (np.array([len(la)], np.int32), np.array([len(lb)], np.int32),
                 np.array(list(la) + list(lb), np.int32), np.array(list(da) + list(db), np.int64))
        quick = {c: self._time(key, c, shape, 1) for c in cands}
        best = sorted(quick, key=quick.get)[:3]
        if cands[0] not in best:
            best.append(cands[0])  # the default is always re-timed
        timed = {c: self._time(key, c, shape, reps) for c in best}
        win = min(timed, key=timed.get)
        if timed[win] > (1.0 - self.margin) * timed[cands[0]]:
            win = cands[0]  # within the timing noise: keep the fixed rule's choice
        self.entries[key] = {"choice": list(win), "default": list(cands[0]),
                             "ms": {choice_name(c): t for c, t in timed.items()},
                             "shape": {"a": [int(x) for x in da], "b": [int(x) for x in db],
                                       "a_labels": [int(x) for x in la], "b_labels": [int(x) for x in lb]}}
        self.install()
        return key

    def tune_plan(self, plan, reps=5, min_cmacs=2 ** 20):
        """Tune the classes of a plan's steps of at least ``min_cmacs`` complex
        multiply-adds (smaller steps are launch-bound); returns the keys."""
        keys = []
        for la, da, lb, db in plan_pairs(plan):
            size = {}
            for x, d in list(zip(la, da)) + list(zip(lb, db)):
                size[x] = d
            if float(np.prod([float(d) for d in size.values()])) < min_cmacs:
                continue
            keys.append(self.tune_pair(la, da, lb, db, reps=reps))
        self.install()
        return keys

    # ---- persistence ------------------------------------------------------------
    def to_dict(self):
        return {"gpu": device_name(self.be.device), "source_hash": source_hash(), "precision": self.be.precision,
                "entries": {str(k): v for k, v in self.entries.items()}}

    def save(self, path=None):
        path = Path(path) if path else cache_path(self.be.device)
        data = {}
        if path.exists():
            try:
                data = json.loads(path.read_text())
            except ValueError:
                data = {}
        if data.get("gpu") != device_name(self.be.device) or data.get("source_hash") != source_hash():
            data = {"gpu": device_name(self.be.device), "source_hash": source_hash(), "tables": {}}
        data.setdefault("tables", {})[str(self.be.precision)] = {str(k): v for k, v in self.entries.items()}
        path.parent.mkdir(parents=True, exist_ok=True)
        path.write_text(json.dumps(data, indent=1, sort_keys=True))
        return path

    def load(self, path=None):
        """Read this context's precision's table from the cache when it was
        written on this GPU for these kernel sources; returns whether it was."""
        path = Path(path) if path else cache_path(self.be.device)
        if not path.exists():
            return False
        try:
            data = json.loads(path.read_text())
        except ValueError:
            return False
        if data.get("gpu") != device_name(self.be.device) or data.get("source_hash") != source_hash():
            return False
        table = data.get("tables", {}).get(str(self.be.precision))
        if table is None:
            return False
        self.entries = {int(k): v for k, v in table.items()}
        self.install()
        return True


def ensure_tuned(backend, plans=(), reps=5, path=None, save=True):
    """Load the cache for this GPU and kernels, tune what the given plans
    need and it lacks, install the table in ``backend`` and (``save``) write
    the cache back.  Returns (tuner, whether anything new was tuned)."""
    t = Tuner(backend)
    t.load(path)
    before = set(t.entries)
    for p in plans:
        t.tune_plan(p, reps=reps)
    new = set(t.entries) != before
    if new and save:
        t.save(path)
    t.install()
    return t, new
