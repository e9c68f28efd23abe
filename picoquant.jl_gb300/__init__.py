"""pqgb300 — PicoQuant's tensor-network contraction path on one GB300.

The API keeps PicoQuant's names (Julia's ``!`` dropped):
``TensorNetworkCircuit``, ``add_gate``, ``add_input``, ``add_output``,
``contract_pair``, ``full_wavefunction_contraction``, ``contract_network``,
``load_tensor_data``, ``bgreedy``, slicing helpers, and ``GB300Backend`` as the
backend (the role of ``InteractiveBackend{T}``).  All numeric work runs in
``libpqgb300.so`` (CUDA, sm_103a); there is no CPU fallback.
"""
from ._lib import (PQ_C64, PQ_C128, PQError, PREC_3XBF16, PREC_3XTF32, PREC_6XTF32, PREC_C64, PREC_C128, PREC_OZAKI,
                   PREC_OZAKI4)
from .backend import GB300Backend, Metrics, decompose_array, record_compute_costs, record_memory_costs
from .dsl import DSLBackend, DSLPlan, compile_dsl, execute_dsl_file
from .mps import (MPSState, calculate_mps_amplitudes, compress_bond, compress_tensor_chain,
                  contract_mps_tensor_network_circuit,
                  contract_tensor_network_circuit_with_compression)
from .circuits import (CX, CZ, SWAP, H, build_network, cphase, ghz_gates, grid_patterns, grid_shape, haar_su2,
                       operator_to_tensor, qft_gates, random_bitstrings, random_grid_gates)
from .contraction import (contract_network, contract_pair, create_ncon_indices, full_wavefunction_contraction,
                          inorder_contraction, merge_common_bonds,
                          multi_index_partition, partition_network_on_virtual_bonds, random_contraction_plan,
                          replace_with_view, slice_tensor_network, sort_indices)
from .network import (Edge, Node, TensorNetworkCircuit, add_gate, add_input, add_output, decompose_gate,
                      delete_tensor, edges, getedge, getnode, inedges, inneighbours, load_tensor_data, neighbours,
                      new_label, outedges, outneighbours, permute_tensor, reshape_tensor, save_output,
                      save_tensor_data, view_tensor, virtualedges, virtualneighbours, network_from_dict, network_from_json, to_dict, to_json)
from .planning import (NetworkPlan, bgreedy, bgreedy_contraction, bitstrings_to_index, greedy_steps,
                       open_output_edges, pairs_to_steps, steps_to_pairs, wavefunction_steps)

__all__ = [k for k in dir() if not k.startswith("_")]
