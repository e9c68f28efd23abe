"""GB300Backend: the backend method table of PicoQuant over the C ABI.

Mirrors the reference's `AbstractBackend` interface (src/backends.jl:3) as
implemented by `InteractiveBackend{T}` (src/backends/interactive.jl:10-172):
save/load/contract/save_output/reshape/permute/decompose/delete/view plus the
`metrics` field updated by `contract_pair!` (src/layer2.jl:373).  Tensors live
on the GPU inside the library's context; node Symbols map to int64 ids.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L


@dataclass
class Metrics:
    """src/backends.jl:8-20."""

    max_tensor_size: int = 0
    total_space_allocated: int = 0
    flops: int = 0


def record_compute_costs(backend, open_dims, contracted_dims):
    """src/backends.jl:30-41: space += prod(open); flops += prod(open)*prod(contracted)."""
    space = 1
    for d in open_dims:
        space *= int(d)
    record_memory_costs(backend, space)
    k = 1
    for d in contracted_dims:
        k *= int(d)
    backend.metrics.flops += space * k
    return space * k, space


def record_memory_costs(backend, mem):
    """src/backends.jl:50-57."""
    backend.metrics.total_space_allocated += mem
    if mem > backend.metrics.max_tensor_size:
        backend.metrics.max_tensor_size = mem


_PREC_NAMES = {L.PREC_C128: "c128", L.PREC_C64: "c64", L.PREC_3XTF32: "3xtf32", L.PREC_3XBF16: "3xbf16",
               L.PREC_6XTF32: "6xtf32", L.PREC_OZAKI: "ozaki", L.PREC_OZAKI4: "ozaki4"}


class GB300Backend:
    """Device-resident tensor store + contraction kernels on one GB300.

    ``precision`` selects storage and arithmetic (the role of the element type
    ``T`` of ``InteractiveBackend{T}``): PREC_C128 (ComplexF64, FP64 math),
    PREC_C64 (ComplexF32 storage and FP32 math for large tensors),
    PREC_3XTF32 / PREC_6XTF32 (as PREC_C64, with split-precision TF32
    tensor-core products for large pairs), PREC_OZAKI (as PREC_C64, with
    exact-accumulation bf16-slice tensor-core products for large pairs),
    PREC_3XBF16 (accepted, runs as PREC_C64).  In the complex64 modes tensors of at most
    ``small_elems`` elements (default 65536) stay complex128: gate tensors and
    small intermediates cost nothing in time, and rounding them would dominate
    the error of the final amplitudes.
    """

    def __init__(self, precision: int = L.PREC_C64, device: int = 0, small_elems: int | None = None,
                 svd: str = "host"):
        if svd not in ("host", "device"):
            raise ValueError(f"svd must be 'host' or 'device', not {svd!r}")
        self.svd = svd
        self.lib = L.lib()
        h = C.c_void_p()
        rc = self.lib.pq_ctx_create(device, precision, C.byref(h))
        if rc != L.PQ_OK:
            raise L.PQError(rc, f"pq_ctx_create(device={device}, precision={precision}) failed")
        self.ctx = h
        self.precision = precision
        self.device = device
        if small_elems is not None:
            self._check(self.lib.pq_ctx_set_small_elems(self.ctx, int(small_elems)), "set_small_elems")
        self.metrics = Metrics()
        self._ids: dict[str, int] = {}
        self._next = 1

    # ---- lifetime -----------------------------------------------------------
    def close(self):
        if self.ctx:
            self.lib.pq_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass

    @property
    def precision_name(self):
        return _PREC_NAMES[self.precision]

    def _check(self, rc, what):
        L.check(rc, self.ctx, what)

    def tuning_size(self) -> int:
        """Entries of the context's autotuned table (``autotune``)."""
        n = C.c_int()
        self._check(self.lib.pq_ctx_tuning_size(self.ctx, C.byref(n)), "tuning_size")
        return n.value

    def id_of(self, label) -> int:
        key = str(label)
        i = self._ids.get(key)
        if i is None:
            i = self._next
            self._next += 1
            self._ids[key] = i
        return i

    def sync(self):
        self._check(self.lib.pq_ctx_sync(self.ctx), "sync")

    def launch_count(self) -> int:
        v = C.c_int64()
        self._check(self.lib.pq_ctx_launch_count(self.ctx, C.byref(v)), "launch_count")
        return v.value

    def mem_in_use(self) -> int:
        v = C.c_int64()
        self._check(self.lib.pq_ctx_mem_in_use(self.ctx, C.byref(v)), "mem_in_use")
        return v.value

    def set_mem_cap(self, nbytes: int):
        self._check(self.lib.pq_ctx_set_mem_cap(self.ctx, int(nbytes)), "set_mem_cap")

    # ---- backend method table ---------------------------------------------
    def save_tensor_data(self, label, data):
        """src/backends/interactive.jl:32-36."""
        a = np.asarray(data)
        shape = a.shape  # (asfortranarray turns a 0-d array into shape (1,))
        if a.dtype == np.complex64:
            a = np.asfortranarray(a)
            dt = L.PQ_C64
        else:
            a = np.asfortranarray(a, dtype=np.complex128)
            dt = L.PQ_C128
        dims = L.arr(C.c_int64, shape)
        rc = self.lib.pq_save_tensor_data(self.ctx, self.id_of(label), len(shape), dims,
                                          a.ctypes.data_as(C.c_void_p), dt)
        self._check(rc, f"save_tensor_data({label})")

    def save_tensors(self, items):
        """Upload several (label, array) pairs in one batch (``pq_save_tensors``:
        one staging copy and one device scatter instead of one copy each)."""
        items = list(items)
        if not items:
            return
        arrs, ids, ranks, dims, dts = [], [], [], [], []
        for label, data in items:
            a = np.asarray(data)
            shape = a.shape
            if a.dtype == np.complex64:
                a = np.asfortranarray(a)
                dts.append(L.PQ_C64)
            else:
                a = np.asfortranarray(a, dtype=np.complex128)
                dts.append(L.PQ_C128)
            arrs.append(a)
            ids.append(self.id_of(label))
            ranks.append(len(shape))
            dims.extend(shape)
        ptrs = (C.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
        rc = self.lib.pq_save_tensors(self.ctx, len(arrs), L.arr(C.c_int64, ids), L.arr(C.c_int32, ranks),
                                      L.arr(C.c_int64, dims or [0]), ptrs, L.arr(C.c_int32, dts))
        self._check(rc, "save_tensors")

    def prepare_tensors(self, items):
        """The argument arrays of ``save_tensors`` for a fixed list of (label,
        host array) pairs, built once, for a caller that uploads the same
        tensors again and again (new values written into the same arrays,
        e.g. the gates of a parameterised circuit before every contraction).
        Every array must be Fortran-ordered complex64 or complex128 and stay
        alive, with its shape, while the result is in use; ``save_prepared``
        then uploads the arrays' current contents with one library call."""
        items = list(items)
        ids, ranks, dims, dts, keep = [], [], [], [], []
        for label, a in items:
            if not isinstance(a, np.ndarray) or a.dtype not in (np.complex64, np.complex128) or not (
                    a.flags.f_contiguous or a.ndim <= 1):
                raise ValueError(f"prepare_tensors({label}): needs a Fortran-ordered complex64/complex128 array")
            keep.append(a)
            ids.append(self.id_of(label))
            ranks.append(a.ndim)
            dims.extend(a.shape)
            dts.append(L.PQ_C64 if a.dtype == np.complex64 else L.PQ_C128)
        n = len(keep)
        return (n, L.arr(C.c_int64, ids or [0]), L.arr(C.c_int32, ranks or [0]), L.arr(C.c_int64, dims or [0]),
                (C.c_void_p * max(1, n))(*[a.ctypes.data for a in keep]), L.arr(C.c_int32, dts or [0]), keep)

    def save_prepared(self, prepared):
        """Upload the current contents of the arrays of ``prepare_tensors``
        (``pq_save_tensors``: one staging copy and one device scatter)."""
        n, ids, ranks, dims, ptrs, dts, _ = prepared
        if n:
            self._check(self.lib.pq_save_tensors(self.ctx, n, ids, ranks, dims, ptrs, dts), "save_tensors")

    def norm2(self, label) -> float:
        """Squared 2-norm of a tensor, accumulated in FP64 on the device
        (``pq_tensor_norm2``): the fidelity check of a state vector."""
        v = C.c_double(0.0)
        self._check(self.lib.pq_tensor_norm2(self.ctx, self.id_of(label), C.byref(v)), f"tensor_norm2({label})")
        return v.value

    def has_tensor(self, label) -> bool:
        key = str(label)
        return key in self._ids and bool(self.lib.pq_has_tensor(self.ctx, self._ids[key]))

    def shape(self, label):
        r = C.c_int()
        dims = (C.c_int64 * L.PQ_MAX_RANK)()
        self._check(self.lib.pq_tensor_shape(self.ctx, self.id_of(label), C.byref(r), dims), f"shape({label})")
        return tuple(dims[i] for i in range(r.value))

    def load_tensor_data(self, label, dtype=np.complex128):
        """src/backends/interactive.jl:44-49: the tensor as a host array, or None."""
        if not self.has_tensor(label):
            return None
        shp = self.shape(label)
        n = int(np.prod(shp)) if shp else 1
        out = np.empty(n, dtype=dtype)
        dt = L.PQ_C64 if np.dtype(dtype) == np.complex64 else L.PQ_C128
        rc = self.lib.pq_load_tensor_data(self.ctx, self.id_of(label), out.ctypes.data_as(C.c_void_p), n, dt)
        self._check(rc, f"load_tensor_data({label})")
        if not shp:
            return out[0]
        return out.reshape(shp, order="F")

    def contract_tensors(self, A, ia, B, ib, Cl):
        """src/backends/interactive.jl:60-75 (A and B are consumed)."""
        la = L.arr(C.c_int32, ia)
        lb = L.arr(C.c_int32, ib)
        rc = self.lib.pq_contract_tensors(self.ctx, self.id_of(A), la, len(ia), self.id_of(B), lb, len(ib),
                                          self.id_of(Cl))
        self._check(rc, f"contract_tensors({A}, {B} -> {Cl})")

    def save_output(self, node, name="result"):
        """src/backends/interactive.jl:84-88."""
        self._check(self.lib.pq_save_output(self.ctx, self.id_of(node), self.id_of(name)), "save_output")

    def reshape_tensor(self, tensor, groups):
        """src/backends/interactive.jl:97-100 (groups of 1-based axes)."""
        sizes = [len(g) for g in groups]
        axes = [int(x) for g in groups for x in g]
        rc = self.lib.pq_reshape_tensor(self.ctx, self.id_of(tensor), len(groups), L.arr(C.c_int32, sizes),
                                        L.arr(C.c_int32, axes))
        self._check(rc, f"reshape_tensor({tensor})")

    def permute_tensor(self, tensor, axes):
        """src/backends/interactive.jl:105-108 (1-based permutation)."""
        rc = self.lib.pq_permute_tensor(self.ctx, self.id_of(tensor), L.arr(C.c_int32, axes), len(axes))
        self._check(rc, f"permute_tensor({tensor})")

    def delete_tensor(self, tensor):
        """src/backends/interactive.jl:159-161."""
        if str(tensor) in self._ids:
            self._check(self.lib.pq_delete_tensor(self.ctx, self._ids[str(tensor)]), "delete_tensor")

    def view_tensor(self, view_node, node, bond_idx, bond_range):
        """src/backends/interactive.jl:169-172; bond_range is a 1-based
        inclusive (lo, hi) pair or a ``range`` of 1-based values."""
        if isinstance(bond_range, range):
            lo, hi = bond_range.start, bond_range.stop - 1
        else:
            lo, hi = bond_range
        rc = self.lib.pq_view_tensor(self.ctx, self.id_of(view_node), self.id_of(node), int(bond_idx), int(lo),
                                     int(hi))
        self._check(rc, f"view_tensor({node})")

    def decompose_tensor(self, tensor, left_positions, right_positions, threshold=1e-13, max_rank=0,
                         left_label=None, right_label=None):
        """src/backends/interactive.jl:124-151 -> src/layer1.jl:146-184.

        The SVD split is not on the contraction path.  With ``svd="host"``
        (the default) the tensor is downloaded, split by LAPACK in FP64 and
        the two factors uploaded; with ``svd="device"`` it is split in place
        by the library's one-sided Jacobi SVD (FP64, one CTA; the smaller
        side of the split at most 256).  Returns the new bond extent.
        """
        if self.svd == "device":
            lp = np.ascontiguousarray(left_positions, dtype=np.int32)
            rp = np.ascontiguousarray(right_positions, dtype=np.int32)
            chi, sweeps = C.c_int(0), C.c_int(0)
            rc = self.lib.pq_decompose_tensor(self.ctx, self.id_of(tensor), lp.size, lp.ctypes.data_as(L.i32p),
                                              rp.size, rp.ctypes.data_as(L.i32p), float(threshold), int(max_rank),
                                              self.id_of(left_label), self.id_of(right_label), C.byref(chi),
                                              C.byref(sweeps))
            self._check(rc, f"decompose_tensor({tensor})")
            self.last_svd_sweeps = sweeps.value
            return chi.value
        data = self.load_tensor_data(tensor)
        B, Cm, chi = decompose_array(data, left_positions, right_positions, threshold, max_rank,
                                     eps_dtype=np.float32 if self.precision != L.PREC_C128 else np.float64)
        self.save_tensor_data(left_label, B)
        self.save_tensor_data(right_label, Cm)
        self.delete_tensor(tensor)
        return chi

    # ---- bulk helpers -------------------------------------------------------
    def gather(self, label, linear_indices, dtype=np.complex128):
        idx = np.ascontiguousarray(linear_indices, dtype=np.int64)
        out = np.empty(idx.size, dtype=dtype)
        dt = L.PQ_C64 if np.dtype(dtype) == np.complex64 else L.PQ_C128
        rc = self.lib.pq_gather_elements(self.ctx, self.id_of(label), idx.ctypes.data_as(L.i64p), idx.size,
                                         out.ctypes.data_as(C.c_void_p), dt)
        self._check(rc, "gather")
        return out


def decompose_array(tensor, left_positions, right_positions, threshold=1e-13, max_rank=0, eps_dtype=np.float64):
    """src/layer1.jl:146-184: SVD across (left | right) positions (1-based)."""
    dims = tensor.shape
    ld = [dims[x - 1] for x in left_positions]
    rd = [dims[x - 1] for x in right_positions]
    A = np.transpose(tensor, [x - 1 for x in list(left_positions) + list(right_positions)])
    A = np.reshape(A, (int(np.prod(ld)), int(np.prod(rd))), order="F")
    U, S, Vh = np.linalg.svd(A, full_matrices=False)
    threshold = max(threshold, float(np.sqrt(np.finfo(eps_dtype).eps)))
    s_norm = float(np.sqrt(np.sum(S**2)))
    chi = int(np.sum(S / s_norm > threshold)) if s_norm > 0 else 0
    if max_rank > 0:
        chi = min(max_rank, chi)
    sq = np.sqrt(S[:chi])
    B = np.reshape(U[:, :chi] * sq[None, :], tuple(ld) + (chi,), order="F")
    Cm = np.reshape(sq[:, None] * Vh[:chi, :], (chi,) + tuple(rd), order="F")
    return B, Cm, chi
