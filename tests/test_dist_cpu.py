"""Multi-rank slicing on CPU: two gloo ranks each contract a contiguous share
of the slices of a sliced single amplitude (the FP64 oracle stands in for the
device), one all-reduce of the partial sums finishes the amplitude."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _rank(rank, world, port, out):
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    sys.path.insert(0, str(root))
    sys.path.insert(0, str(root / "oracle"))
    import tn_oracle as O

    import __graft_entry__ as g

    pq = g.load_package()
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        host = O.OracleBackend()

        class Store:
            def __getattr__(self, k):
                return getattr(host, k)

            def shape(self, label):
                return host.tensors[label].shape

        be = Store()
        gates = pq.random_grid_gates(3, 3, 6, seed=11)
        bits = "011010011"
        net = pq.build_network(9, gates, decompose=True, backend=be)
        pq.add_input(net, "0" * 9)
        pq.add_output(net, bits)
        nodes, ranks, flat, dims, label_of = pq.planning._leaf_arrays(net, [])
        steps, _, _ = pq.greedy_steps(ranks, flat, dims, [], 1.0, 1.0, 4, 3)
        import ctypes as C

        from pqgb300 import _lib as L

        sl = (C.c_int32 * 4)()
        ns = C.c_int()
        L.check(L.lib().pq_plan_choose_slices(len(ranks), L.arr(C.c_int32, ranks), L.arr(C.c_int32, flat),
                                              len(dims), L.arr(C.c_int64, dims), len(steps) // 2,
                                              L.arr(C.c_int32, steps), 0, L.arr(C.c_int32, [0]), 4, 0.0, sl,
                                              C.byref(ns)), None, "choose_slices")
        sliced = [sl[i] for i in range(ns.value)]
        total = int(np.prod([dims[x] for x in sliced]))
        leaves = [host.tensors[net.nodes[nl].data_label] for nl in nodes]
        labs, pos = [], 0
        for r in ranks:
            labs.append(flat[pos:pos + r])
            pos += r
        b, e = pq.planning.slice_range(total, rank, world)
        part = 0j
        for s in range(b, e):
            lv, ll = O.slice_leaves(leaves, labs, sliced, dims, s)
            part += complex(np.asarray(O.execute_ssa_plan(lv, ll, steps, [])).reshape(-1)[0])
        t = torch.tensor([part.real, part.imag], dtype=torch.float64)
        dist.all_reduce(t)
        if rank == 0:
            full = complex(np.asarray(O.execute_ssa_plan(leaves, labs, steps, [])).reshape(-1)[0])
            out.put((total, e - b, complex(t[0].item(), t[1].item()), full))
    finally:
        dist.destroy_process_group()


def test_slice_range_partition(pq):
    for total, world in ((1024, 2), (1024, 3), (7, 4), (3, 8)):
        parts = [pq.planning.slice_range(total, r, world) for r in range(world)]
        assert parts[0][0] == 0 and parts[-1][1] == total
        assert all(parts[i][1] == parts[i + 1][0] for i in range(world - 1))
        sizes = [e - b for b, e in parts]
        assert max(sizes) - min(sizes) <= 1


def test_two_gloo_ranks_sum_slices():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 2000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    total, mine, amp, full = q.get(timeout=5)
    assert total > 1 and mine < total
    assert abs(amp - full) < 1e-13
