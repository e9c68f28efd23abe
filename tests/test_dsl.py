"""The DSL wire format: the recording backend, the interpreter and the
compiled plan (src/backends/dsl.jl, src/layer1.jl:211-330)."""
import numpy as np
import pytest


def _ghz3_script(pq, tmp_path):
    """src/layer1_tests.jl:11-44: GHZ-3 recorded by the DSL backend."""
    be = pq.DSLBackend(str(tmp_path / "contract_network.tl"), str(tmp_path / "tensor_data.npz"), "", True)
    net = pq.build_network(3, pq.ghz_gates(3), backend=be)
    pq.add_input(net, "000")
    pq.add_output(net, "000")
    plan = pq.random_contraction_plan(net, np.random.default_rng(0))
    pq.contract_network(net, plan)
    be.flush()
    return be, net


def test_dsl_backend_writes_reference_lines(pq, tmp_path):
    be, net = _ghz3_script(pq, tmp_path)
    lines = open(be.dsl_filename).read().splitlines()
    assert lines[0].startswith("tensor node_1 node_1")
    ops = [ln.split()[0] for ln in lines]
    assert set(ops) <= {"tensor", "ncon", "del", "save"}
    ncon = [ln.split() for ln in lines if ln.startswith("ncon")]
    for c in ncon:
        assert len(c) == 6 and all(x.lstrip("-").isdigit() for x in c[3].split(",") + c[5].split(","))
    # every ncon is followed by the deletion of its two operands
    for i, ln in enumerate(lines):
        if ln.startswith("ncon"):
            _, C, A, _, B, _ = ln.split()
            assert lines[i + 1] == f"del {A}" and lines[i + 2] == f"del {B}"
    assert lines[-1].split()[0] == "save" and lines[-1].split()[-1] == "result"
    assert len(net.nodes) == 1


def test_dsl_script_replays_on_the_oracle_backend(pq, O, tmp_path, host_backend):
    be, _ = _ghz3_script(pq, tmp_path)
    out = pq.execute_dsl_file(be.dsl_filename, be.tensor_data_filename, backend=host_backend)
    assert abs(complex(np.asarray(out["result"]).reshape(-1)[0]) - 1 / np.sqrt(2)) < 1e-12


def test_dsl_other_commands_replay(pq, tmp_path, host_backend):
    """reshape / permute / view / decompose lines on a host backend."""
    rng = np.random.default_rng(1)
    A = rng.standard_normal((2, 3, 4)) + 1j * rng.standard_normal((2, 3, 4))
    script = "\n".join(["tensor a a", "permute a 3,1,2", "view v a 2 1,2", "save v out v", "reshape a 1;2,3",
                        "save a out r"])
    out = pq.execute_dsl_file(script, {"a": A}, backend=host_backend)
    np.testing.assert_allclose(out["v"], np.transpose(A, (2, 0, 1))[:, 0:2, :])
    np.testing.assert_allclose(out["r"], np.transpose(A, (2, 0, 1)).reshape((4, 6), order="F"))


@pytest.mark.gpu
def test_dsl_interpreted_and_compiled_on_gpu(pq, O, tmp_path):
    gates = pq.random_grid_gates(2, 3, 4, seed=8)
    rec = pq.DSLBackend(str(tmp_path / "c.tl"), str(tmp_path / "d.npz"), "", True)
    net = pq.build_network(6, gates, backend=rec)
    pq.add_input(net, "0" * 6)
    pq.full_wavefunction_contraction(net, "vector")
    rec.flush()
    ref = O.statevector(6, gates)
    be = pq.GB300Backend(pq.PREC_C128)
    out = pq.execute_dsl_file(rec.dsl_filename, rec.tensor_data_filename, backend=be)
    assert np.max(np.abs(np.asarray(out["result"]).reshape(-1, order="F") - ref)) < 1e-12
    be.close()
    # the ncon part of a single-amplitude script, compiled once and replayed
    rec2 = pq.DSLBackend(str(tmp_path / "a.tl"), str(tmp_path / "a.npz"), "", True)
    net2 = pq.build_network(6, gates, backend=rec2)
    pq.add_input(net2, "0" * 6)
    pq.add_output(net2, "011010")
    pq.contract_network(net2, pq.random_contraction_plan(net2, np.random.default_rng(3)))
    rec2.flush()
    be = pq.GB300Backend(pq.PREC_C128)
    plan = pq.compile_dsl(rec2.dsl_filename, rec2.tensor_data_filename, be)
    amp_ref = ref[O.amplitude_index("011010")]
    for capture in (True, False, False):
        a = complex(np.asarray(plan.run(capture=capture)).reshape(-1)[0])
        assert abs(a - amp_ref) < 1e-12
    plan.close()
    be.close()
