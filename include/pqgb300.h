/*
 * pqgb300 — GB300 (sm_103a) tensor-network contraction backend, C ABI.
 *
 * This is the drop-in boundary below PicoQuant's backend API: every function
 * here replaces one method of the reference's `AbstractBackend` method table
 * (src/backends.jl:3, forwarded from src/layer3.jl:124-134) or adds the
 * plan-level executor that sits under `contract_network!` /
 * `full_wavefunction_contraction!` (src/layer2.jl:132-195, 250-321).
 *
 * Conventions
 *   - Tensors are dense, column-major (first index fastest), complex:
 *     PQ_C64 = interleaved (re, im) float pairs (Julia ComplexF32),
 *     PQ_C128 = interleaved (re, im) double pairs (Julia ComplexF64).
 *   - Tensor ids are caller-chosen int64 keys (the Julia side maps each
 *     node Symbol to an id).  A rank-0 tensor holds one element.
 *   - Every call returns an int status: 0 = success, < 0 = error.  The
 *     message of the last error on a context is `pq_last_error(ctx)`.
 *     No call exits the process or traps the device; device-side failures
 *     are reported through a status word read at the next synchronising call.
 *   - One context = one CUDA stream on one device.  Calls on a context must
 *     be serialised by the caller; distinct contexts are independent.
 *   - The library owns all device memory.  Host buffers are copied on
 *     put/get and never retained.
 */
#ifndef PQGB300_H
#define PQGB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define PQ_OK               0
#define PQ_ERR_INVALID     -1  /* bad argument, label/dim mismatch, bad plan   */
#define PQ_ERR_NOT_FOUND   -2  /* unknown tensor id                             */
#define PQ_ERR_OOM         -3  /* device allocation failed or cap exceeded      */
#define PQ_ERR_CUDA        -4  /* CUDA runtime error                            */
#define PQ_ERR_DEVICE      -5  /* a kernel reported failure via status word     */
#define PQ_ERR_UNSUPPORTED -6  /* shape/precision not supported                 */

/* ---- element types (host-side data) ------------------------------------ */
#define PQ_C64   1  /* ComplexF32 */
#define PQ_C128  2  /* ComplexF64 */

/* ---- context precision modes ------------------------------------------- *
 * PQ_PREC_C128   : tensors stored as complex128, all arithmetic FP64.
 *                  The plain complex-FP64 CUDA path.
 * PQ_PREC_C64    : large tensors stored as complex64 (small ones, see
 *                  pq_ctx_set_small_elems, as complex128); FP32 SIMT
 *                  arithmetic with Kahan-compensated accumulation.
 * PQ_PREC_3XTF32 : as PQ_PREC_C64, but large GEMM-shaped contractions run on
 *                  the tcgen05 tensor cores: every real product split into
 *                  TF32 hi+lo parts (3 products: hh, hl, lh), FP32 TMEM
 *                  accumulation over 8-deep K chunks folded into
 *                  Kahan-compensated FP32 sums.
 * PQ_PREC_3XBF16 : as PQ_PREC_OZAKI with three bf16 slices (6 slice-pair
 *                  products, about 21 significant bits: pair error ~1e-6, not
 *                  enough for 1e-6 amplitude error); K > 512 runs as
 *                  PQ_PREC_3XTF32.
 * PQ_PREC_6XTF32 : as PQ_PREC_3XTF32 with a hi+mid+lo TF32 split and 6
 *                  products (hh, hm, mh, hl, lh, mm) per real product.
 * PQ_PREC_OZAKI  : as PQ_PREC_C64, but large GEMM-shaped contractions with
 *                  K <= 512 run the Ozaki scheme on the tcgen05 tensor cores:
 *                  rows of A / columns of B scaled by powers of two, cut into
 *                  five 7-bit bf16 slices, the 15 slice products of level
 *                  <= 4 accumulated in FP32 TMEM where levels 0 and 1 are
 *                  exact; the result is rounded once.  Larger K runs as
 *                  PQ_PREC_6XTF32.
 * PQ_PREC_OZAKI4 : as PQ_PREC_OZAKI with four slices: the 10 slice products
 *                  of level <= 3 (residual below 2^-29 of the row / column
 *                  scale), two thirds of the tensor-core work.  With
 *                  complex64 storage its added error is about the size of the
 *                  storage rounding (amplitude errors about twice
 *                  PQ_PREC_OZAKI's); complex128 storage (pq_ctx_set_small_elems
 *                  with a large threshold) removes the storage rounding but
 *                  runs the memory-bound steps in FP64.                     */
#define PQ_PREC_C128    0
#define PQ_PREC_C64     1
#define PQ_PREC_3XTF32  2
#define PQ_PREC_3XBF16  3
#define PQ_PREC_6XTF32  4
#define PQ_PREC_OZAKI   5
#define PQ_PREC_OZAKI4  6

#define PQ_MAX_RANK 56

typedef struct pq_ctx pq_ctx;
typedef struct pq_plan pq_plan;

/* ---- context ------------------------------------------------------------
 * Replaces constructing `InteractiveBackend{T}()` (src/backends/interactive.jl:10-23);
 * `precision` plays the role of the element type parameter T. */
int pq_ctx_create(int device, int precision, pq_ctx** out);
int pq_ctx_destroy(pq_ctx* ctx);
const char* pq_last_error(pq_ctx* ctx);
int pq_ctx_precision(pq_ctx* ctx);
/* Wait for all work on the context's stream; checks the device status word. */
int pq_ctx_sync(pq_ctx* ctx);
/* Cap on device bytes the context may hold (0 = unlimited).  Allocations
 * beyond the cap fail with PQ_ERR_OOM (host-side fault injection). */
int pq_ctx_set_mem_cap(pq_ctx* ctx, int64_t bytes);
int pq_ctx_mem_in_use(pq_ctx* ctx, int64_t* bytes);
/* Precision policy of the complex64 modes: tensors of at most `n` elements
 * are stored (and their contractions accumulated) in complex128, larger ones
 * in complex64 (default n = 65536; 0 stores everything as complex64).
 * Applies to tensors created afterwards. */
int pq_ctx_set_small_elems(pq_ctx* ctx, int64_t n);
/* Number of kernels this context has launched so far. */
int pq_ctx_launch_count(pq_ctx* ctx, int64_t* count);
/* The CUDA stream of the context (a cudaStream_t), for callers that order
 * their own work against it. */
int pq_ctx_stream(pq_ctx* ctx, void** stream);

/* ---- tensor storage ------------------------------------------------------ */
/* src/backends/interactive.jl:32-36 `save_tensor_data` (convert(T, data)).
 * `data` is column-major host memory of `dtype`; converted to the context's
 * storage type on upload.  Replaces an existing tensor with the same id. */
int pq_save_tensor_data(pq_ctx* ctx, int64_t id, int rank, const int64_t* dims,
                        const void* data, int dtype);
/* Upload n tensors in one batch (no reference counterpart: an extension
 * for hosts that re-upload many small tensors per contraction, e.g. every
 * gate of a circuit).  Same semantics per tensor as pq_save_tensor_data
 * (ids[i], ranks[i] extents taken in order from dims_flat, column-major host
 * data[i] of type dtypes[i], stored in the context's storage type); all data
 * go through one pinned staging buffer, one host-to-device copy and one
 * device scatter, and a tensor replaced by one of the same extents keeps its
 * device storage.  The host arrays may be reused as soon as the call
 * returns. */
int pq_save_tensors(pq_ctx* ctx, int n, const int64_t* ids, const int32_t* ranks, const int64_t* dims_flat,
                    const void* const* data, const int32_t* dtypes);
/* src/backends/interactive.jl:44-49 `load_tensor_data`.  Copies the tensor to
 * host memory as `dtype` (dst must hold `n_elems` elements, n_elems >= size).
 * Returns PQ_ERR_NOT_FOUND when the id is absent (the reference returns
 * `nothing`).  Synchronises the context. */
int pq_load_tensor_data(pq_ctx* ctx, int64_t id, void* dst, int64_t n_elems, int dtype);
/* Rank and dims of a stored tensor (dims must hold PQ_MAX_RANK entries). */
int pq_tensor_shape(pq_ctx* ctx, int64_t id, int* rank, int64_t* dims);
int pq_has_tensor(pq_ctx* ctx, int64_t id);
/* src/backends/interactive.jl:159-161 `delete_tensor!`. */
int pq_delete_tensor(pq_ctx* ctx, int64_t id);
/* Squared 2-norm of tensor `id`, sum |x|^2 over its elements, accumulated in
 * FP64 with compensated (Neumaier) sums on the device, in a fixed order
 * (deterministic), written to *norm2.  The fidelity check of a state vector:
 * a unitary circuit's output has norm2 = 1, so |norm2 - 1| measures the
 * accumulated error.  No counterpart in the reference, which would take
 * LinearAlgebra.norm of the downloaded array.  Synchronises. */
int pq_tensor_norm2(pq_ctx* ctx, int64_t id, double* norm2);
/* src/backends/interactive.jl:84-88 `save_output(backend, node, name)`:
 * the tensor `node` is also stored under `name` (a copy on the device). */
int pq_save_output(pq_ctx* ctx, int64_t node, int64_t name);

/* ---- backend tensor operations -------------------------------------------- */
/* src/backends/interactive.jl:60-75 -> src/layer1.jl:85-92.
 * C = tensorcontract(A, a_labels, B, b_labels, symdiff(a_labels, b_labels)):
 * labels present in both operands are summed; C's modes are A's remaining
 * labels in A order followed by B's remaining labels in B order.  A and B are
 * deleted afterwards (consumed), as in the reference. */
int pq_contract_tensors(pq_ctx* ctx, int64_t a, const int32_t* a_labels, int a_rank,
                        int64_t b, const int32_t* b_labels, int b_rank, int64_t c);
/* src/backends/interactive.jl:105-108 -> src/layer1.jl:111-114 (permutedims);
 * `perm1` is 1-based, as in Julia. */
int pq_permute_tensor(pq_ctx* ctx, int64_t id, const int32_t* perm1, int rank);
/* src/backends/interactive.jl:97-100: reshape by index groups.  Group g holds
 * `group_sizes[g]` consecutive 1-based axis numbers taken from `axes1`; the
 * new dims are the products over each group (column-major, no data motion). */
int pq_reshape_tensor(pq_ctx* ctx, int64_t id, int n_groups, const int32_t* group_sizes,
                      const int32_t* axes1);
/* src/backends/interactive.jl:169-172 -> src/layer1.jl:191-194 (`view_tensor!`):
 * stores under `view_id` a copy of `node` with axis `bond_idx1` (1-based)
 * narrowed to the 1-based inclusive range lo1:hi1. */
int pq_view_tensor(pq_ctx* ctx, int64_t view_id, int64_t node, int bond_idx1,
                   int64_t lo1, int64_t hi1);
/* src/backends/interactive.jl:124-151 -> src/layer1.jl:146-184
 * (`decompose_tensor!`): splits tensor `id` by SVD into
 *   left_id  with dims (left dims..., chi)  and
 *   right_id with dims (chi, right dims...),
 * each factor carrying sqrt(S), as in the reference.  `left1`/`right1` are
 * 1-based axis numbers that together name every axis once.  chi counts the
 * singular values with s / ||s||_2 > max(threshold, sqrt(eps)) (eps of
 * ComplexF32, or of ComplexF64 in a PQ_PREC_C128 context), capped by
 * max_rank when max_rank > 0; it is written to *chi_out.  The input is
 * deleted.  The SVD is one-sided Jacobi on the device (one CTA), in complex
 * FP64 in a PQ_PREC_C128 context and in complex FP32 otherwise (LAPACK's
 * precision for the reference's ComplexF64 / ComplexF32 backends); the
 * smaller of the two matrix sides is limited to 256 and the product of the
 * sides to 2^24 (PQ_ERR_UNSUPPORTED beyond).  *sweeps_out (may be NULL)
 * receives the number of Jacobi sweeps taken (at most 60). */
int pq_decompose_tensor(pq_ctx* ctx, int64_t id, int n_left, const int32_t* left1,
                        int n_right, const int32_t* right1, double threshold,
                        int max_rank, int64_t left_id, int64_t right_id, int* chi_out,
                        int* sweeps_out);
/* Gather amplitudes: out[i] = T[idx[i]] for linear (column-major) indices,
 * written as `dtype` into host memory.  Synchronises. */
int pq_gather_elements(pq_ctx* ctx, int64_t id, const int64_t* idx, int64_t n,
                       void* out, int dtype);
/* pq_gather_elements for callers that cannot let the library allocate device
 * memory (a host that owns and accounts every device allocation itself, such
 * as a Julia process whose CUDA.jl pool must see all device memory, or an
 * application running under a fixed device-memory budget).  No counterpart
 * in the reference.  Same arguments, results and errors as
 * pq_gather_elements, but the index list and the gathered values are staged
 * in a fixed static device array instead of buffers allocated per call; the
 * call allocates no device memory.
 *   - At most 65536 indices per call; larger n fails with PQ_ERR_INVALID.
 *   - The array (1.5 MiB) is reserved on every device that loads the
 *     library until the process exits.
 *   - The first call on a device looks the array's device address up; make
 *     that first call before any stream capture on that device.
 *   - All calls on a device share the array and each overwrites what the
 *     previous one left (nothing in it needs to start zeroed); calls that
 *     overlap on the GPU (other contexts' streams of the same device)
 *     race on it. */
int pq_gather_elements_noalloc(pq_ctx* ctx, int64_t id, const int64_t* idx, int64_t n,
                               void* out, int dtype);

/* ---- contraction plans ----------------------------------------------------
 * A plan is a whole pairwise contraction of a network, compiled once
 * (mode analysis, kernel choice per pair, intermediate buffer offsets in a
 * single arena, optional CUDA-graph capture) and executed many times.  It is
 * the executor under `contract_network!` with a pair plan
 * (src/layer2.jl:294-321) and under the full-wavefunction order
 * (src/layer2.jl:132-195).
 *
 * Network description (host arrays):
 *   n_leaves, leaf_ranks[n_leaves], leaf_labels[sum(ranks)] (int32 labels in
 *   0..n_labels-1, each leaf's labels in its storage order), label_dims[n_labels].
 *   n_steps pairs in `steps[2*i], steps[2*i+1]`: SSA operand numbers, where
 *   0..n_leaves-1 are the leaves and n_leaves+i is the result of step i.
 *   out_labels[n_out]: mode order of the final tensor (the last step's result).
 * A label is summed at the first step after which no other live operand and
 * no output still carries it (so labels shared by more than two tensors act
 * as batch/hyper indices until their last use). */
int pq_plan_create(pq_ctx* ctx, int n_leaves, const int32_t* leaf_ranks,
                   const int32_t* leaf_labels, int n_labels, const int64_t* label_dims,
                   int n_steps, const int32_t* steps, int n_out, const int32_t* out_labels,
                   pq_plan** out);
int pq_plan_destroy(pq_plan* plan);
/* Cost summary of a compiled plan: complex multiply-adds (the reference's
 * `flops` metric, src/backends.jl:37), largest intermediate (elements),
 * arena bytes, and the number of kernel launches one execution makes. */
int pq_plan_info(pq_plan* plan, double* cmacs, int64_t* max_elems, int64_t* arena_bytes,
                 int64_t* launches);
/* Execute: leaves are tensor ids already stored in the context (they are not
 * consumed); the result is stored under `out_id`.  Asynchronous. */
int pq_plan_execute(pq_plan* plan, const int64_t* leaf_ids, int64_t out_id);
/* Capture one execution for `leaf_ids` into a CUDA graph; later
 * pq_plan_execute calls with the same leaf ids replay it. */
int pq_plan_capture(pq_plan* plan, const int64_t* leaf_ids, int64_t out_id);
/* Per-step timing: executes once with CUDA events around every step and
 * writes n_steps milliseconds into `ms` (used to build cost-model data). */
int pq_plan_profile(pq_plan* plan, const int64_t* leaf_ids, int64_t out_id, float* ms);
/* Per-step shape features: for each step, 8 doubles:
 *   log2|A|, log2|B|, log2|C|, log2 K, log2(stride-1 run of A),
 *   log2(stride-1 run of B), kernel class, bytes moved. */
int pq_plan_step_features(pq_plan* plan, double* feats);

/* Sliced execution.  `sliced_labels[n_sliced]` are labels of the network that
 * are fixed to one value per slice (src/layer2/slicing.jl:37-110); all
 * slices have identical shapes.  Slices [slice_begin, slice_end) (slice s
 * fixes label j to digit j of s in mixed radix over the sliced dims, first
 * label fastest) are contracted in batches of `batch` slices per launch and
 * summed on the device with an FP64 compensated (Neumaier) sum.  The plan's
 * output must be a scalar or small tensor; the running sum (n_out_elems
 * complex doubles, interleaved re/im, plus the same number of compensation
 * terms) lives on the device until `pq_sliced_result`.  Parts of the
 * contraction tree that touch no sliced leaf are computed once per call.
 * The run is recorded as a CUDA graph on the second consecutive call with the
 * same leaf storage, sliced labels, range, batch and reset flag, and
 * replayed from then on (new leaf data in the same storage, e.g. from
 * pq_save_tensors, is read by the replay). */
int pq_plan_run_sliced(pq_plan* plan, const int64_t* leaf_ids, int n_sliced,
                       const int32_t* sliced_labels, int64_t slice_begin, int64_t slice_end,
                       int batch, int reset_sum);
/* Copy the FP64 slice sum (interleaved re/im, n elements) to host memory. */
int pq_sliced_result(pq_plan* plan, double* out, int64_t n);
/* Profile sliced execution: runs the once-per-run steps and one batch of
 * `batch` slices with CUDA events around every step.  For each step i
 * (original plan order) writes ms[i], batched[i] (1 if the step runs once per
 * batch of slices, 0 if once per run) and 8 shape features feats[8*i..]
 * (as pq_plan_step_features, for the batched network). */
int pq_plan_profile_sliced(pq_plan* plan, const int64_t* leaf_ids, int n_sliced,
                           const int32_t* sliced_labels, int batch, float* ms,
                           int32_t* batched, double* feats);

/* ---- grouped state vectors of many circuits --------------------------------
 * An executor beside the pair-plan one for workloads of many circuits, each
 * asked for a few amplitudes; the reference contracts each circuit alone
 * (src/layer2.jl:294-321).  Circuit i has n_qubits[i] (<= 31) qubits and
 * n_blocks[i] blocks, applied in order to |0..0> in a complex64 state (qubit
 * q at bit q-1 of the amplitude index, the reference's output order
 * src/layer2.jl:180-189).  Block j (all circuits' blocks concatenated) acts
 * on block_k[j] (1..4) qubits listed in block_qubits (0-based bit positions,
 * concatenated; the first is the low bit of the block's matrix index) with
 * the 2^k x 2^k matrix in block_mats (complex128 interleaved, element
 * (out, in) at out + in 2^k, concatenated).  Circuit i asks for n_amps[i]
 * amplitudes at the state indices in amp_idx (concatenated).  Circuits are
 * packed by size into chunks whose states fit state_budget_bytes (at least
 * the largest state); launch s of a chunk applies the s-th block of every
 * circuit in it.  The first execution records every chunk's initialisation,
 * block launches and amplitude gather as one CUDA graph; executions replay
 * it and write the amplitudes (complex128 interleaved, in input order). */
typedef struct pq_svbatch pq_svbatch;
int pq_svbatch_create(pq_ctx* ctx, int n_circ, const int32_t* n_qubits, const int32_t* n_blocks,
                      const int32_t* block_k, const int32_t* block_qubits, const double* block_mats,
                      const int32_t* n_amps, const int64_t* amp_idx, int64_t state_budget_bytes,
                      pq_svbatch** out);
int pq_svbatch_execute(pq_svbatch* batch, double* amps_out);
/* Kernels one execution launches, chunks, and the state arena's bytes. */
int pq_svbatch_info(pq_svbatch* batch, int64_t* kernel_launches, int64_t* chunks, int64_t* arena_bytes);
int pq_svbatch_destroy(pq_svbatch* batch);

/* ---- planning ---------------------------------------------------------------
 * Boltzmann-greedy flop-count planner, after src/layer2/bgreedy_contraction.jl:17-66:
 * pairs that share a label (then disjoint pieces by outer product) are scored
 * by the Gray-Kourtis energy cost = |C| - alpha (|A| + |B|) (tensor sizes in
 * elements, bgreedy_contraction.jl:76-94) and sampled with weight
 * exp(-(cost - best) / (tau max(1, |best|))) (a temperature relative to the
 * best pair's cost; tau = 0 takes the best pair); `n_trials` plans are drawn
 * and the one with the fewest complex multiply-adds is kept.  Writes
 * 2*(n_leaves-1) SSA operands into `steps` and returns its cost in `cmacs`
 * and its largest intermediate in `max_elems`.  Labels in `out_labels` are
 * kept open. */
int pq_plan_greedy(int n_leaves, const int32_t* leaf_ranks, const int32_t* leaf_labels,
                   int n_labels, const int64_t* label_dims, int n_out, const int32_t* out_labels,
                   double alpha, double tau, int n_trials, uint64_t seed,
                   int32_t* steps, double* cmacs, int64_t* max_elems);
/* `n_draws` independent planner draws (the candidates a learned cost model
 * ranks): draw d samples with its own generator seeded by seed + d, draw 0
 * with tau = 0 (plain greedy), the others with `tau`; they run on
 * `n_threads` host threads (0: all hardware threads) and the results do not
 * depend on the thread count.  Draw d's 2*(n_leaves-1) SSA operands go to
 * steps[d*2*(n_leaves-1) ...], its cost to cmacs[d], its largest
 * intermediate to max_elems[d].  Same planner as pq_plan_greedy
 * (src/layer2/bgreedy_contraction.jl:17-66). */
int pq_plan_greedy_many(int n_leaves, const int32_t* leaf_ranks, const int32_t* leaf_labels,
                        int n_labels, const int64_t* label_dims, int n_out, const int32_t* out_labels,
                        double alpha, double tau, int n_draws, uint64_t seed, int n_threads,
                        int32_t* steps, double* cmacs, int64_t* max_elems);
/* Cost of SSA steps (no reference counterpart: the flop-count planner's
 * measure of a given order, src/backends.jl:30-41): complex multiply-adds
 * summed over the steps and the largest intermediate (elements), with the
 * executor's label rule (a label is summed once no other live tensor and no
 * output carries it).  Host only. */
int pq_plan_cost(int n_leaves, const int32_t* leaf_ranks, const int32_t* leaf_labels, int n_labels,
                 const int64_t* label_dims, int n_steps, const int32_t* steps, int n_out,
                 const int32_t* out_labels, double* cmacs, double* max_elems);
/* pq_plan_cost for n_cand candidate plans of the same leaves at once, on the
 * context's device (the candidate scoring of the planners: seeded greedy
 * draws after src/layer2/bgreedy_contraction.jl:17-131, randomized sweeps):
 * steps holds n_cand x 2 n_steps SSA operands, candidate after candidate;
 * cmacs[c] and max_elems[c] are plan c's values.  One warp per candidate
 * with its label counts in shared memory (at most 40000 labels, leaf ranks
 * at most 64).  A candidate with an intermediate of more than 64 labels gets
 * infinite values; one that is not an SSA plan of the leaves makes the call
 * fail with PQ_ERR_INVALID. */
int pq_plan_cost_batch(pq_ctx* ctx, int n_leaves, const int32_t* leaf_ranks, const int32_t* leaf_labels,
                       int n_labels, const int64_t* label_dims, int n_steps, int n_cand, const int32_t* steps,
                       int n_out, const int32_t* out_labels, double* cmacs, double* max_elems);
/* Choose labels to slice: repeatedly fix the label that most reduces the
 * largest intermediate (ties: least flop increase) until the largest
 * intermediate is <= 2^log2_target elements or `max_sliced` labels are
 * chosen.  Writes the chosen labels to `sliced` and their count to n_sliced. */
int pq_plan_choose_slices(int n_leaves, const int32_t* leaf_ranks, const int32_t* leaf_labels,
                          int n_labels, const int64_t* label_dims, int n_steps,
                          const int32_t* steps, int n_out, const int32_t* out_labels,
                          int max_sliced, double log2_target, int32_t* sliced, int* n_sliced);

/* ---- learned cost model ------------------------------------------------------
 * No counterpart in the reference (its planners are flop-count heuristics,
 * src/layer2/bgreedy_contraction.jl).  The per-pair timings that train the
 * model are measured by the backend itself. */

/* Time `n_pairs` pairwise contractions with this context's kernels and
 * storage policy (C = symdiff(A, B) as pq_contract_tensors).  Pair p has
 * a_ranks[p] then b_ranks[p] consecutive entries in `labels` / `dims` (the
 * extent of each label occurrence).  Each pair runs once to warm up, then
 * `reps` times between CUDA events; ms[p] is the mean and feats[8p..8p+7] its
 * shape features (as pq_plan_step_features). */
int pq_measure_pairs(pq_ctx* ctx, int n_pairs, const int32_t* a_ranks, const int32_t* b_ranks,
                     const int32_t* labels, const int64_t* dims, int reps, float* ms, double* feats);

typedef struct pq_mlp pq_mlp;
/* MLP n_in -> hidden (x hidden_layers, ReLU) -> 1, FP32 parameters in one
 * flat buffer ordered W1 b1 W2 b2 ... (W_l row-major [in x out]), trained on
 * the context's device by hand-written forward/backward/Adam kernels. */
int pq_mlp_create(pq_ctx* ctx, int n_in, int hidden, int hidden_layers, uint64_t seed, pq_mlp** out);
int pq_mlp_destroy(pq_mlp* m);
int pq_mlp_num_params(pq_mlp* m, int64_t* n);
int pq_mlp_get_params(pq_mlp* m, float* params, int64_t n);
int pq_mlp_set_params(pq_mlp* m, const float* params, int64_t n);
/* Mean-squared-error loss and its gradient w.r.t. all parameters for rows
 * X[n x n_in] (row-major) with targets y[n]. */
int pq_mlp_gradients(pq_mlp* m, const float* X, const float* y, int64_t n, float* grad, float* loss);
/* Adam over `epochs` passes of shuffled mini-batches; the loss of the last
 * batch is returned. */
int pq_mlp_train(pq_mlp* m, const float* X, const float* y, int64_t n, int epochs, int batch, float lr,
                 uint64_t seed, float* final_loss);
/* Predictions for n rows; bf16 != 0 runs inference with bf16 weights and
 * activations (FP32 accumulation). */
int pq_mlp_predict(pq_mlp* m, const float* X, int64_t n, float* out, int bf16);

/* ---- autotuning -------------------------------------------------------------
 * No counterpart in the reference, which leaves kernel choice to its array
 * library (TensorOperations -> BLAS / cuTENSOR, src/layer1.jl:85-92).
 * A pair's tuning class is a 64-bit key: the context's precision mode, the
 * ceil-log2 of its M (A-side free), N (B-side free), K (contracted) and batch
 * extents, and whether A's / B's unit-stride mode is contracted.  A choice is
 * three ints: kernel class (0 generic, 1 SIMT GEMM, 2 tensor core, 4 skinny),
 * tile width (16/32/64/128, 0 = default rule) and orientation (1 as given,
 * 2 as C = B x A, 0 = default rule) of the exact-accumulation tensor-core
 * class.
 *
 * pq_pair_tuning analyses C = symdiff(A, B) (A's a_rank labels and extents
 * first, then B's) in the context's precision, ignoring its table: writes
 * the key and every eligible choice (the default first; up to max_choices,
 * 3 ints each) and their count.
 * pq_ctx_set_tuning replaces the context's table with n (key, choice)
 * entries; from then on contractions, compiled plans and measurements run
 * a pair of a listed class with its choice (when eligible for that pair,
 * else the default).  n = 0 clears it. */
int pq_pair_tuning(pq_ctx* ctx, int a_rank, int b_rank, const int32_t* labels, const int64_t* dims,
                   uint64_t* key, int max_choices, int32_t* choices, int* n_choices);
int pq_ctx_set_tuning(pq_ctx* ctx, int n, const uint64_t* keys, const int32_t* choices);
int pq_ctx_tuning_size(pq_ctx* ctx, int* n);
/* The CUDA device's name (NUL-terminated, at most cap bytes), which keys the
 * autotuner's persisted cache. */
int pq_device_name(int device, char* out, int cap);

/* ---- diagnostics ----------------------------------------------------------
 * Exercises the error path of the tensor-core kernels' bounded waits: one
 * thread waits on a shared-memory mbarrier that nobody arrives at, for at
 * most `polls` polls (1..2^20), records the expiry in the context's status
 * word exactly as an expired wait in pq_tc.cu / pq_oz.cu does, and returns
 * (no copies, MMAs or TMEM in flight).  *expired = 1 when the wait ran out.
 * The call itself returns PQ_OK; the context's next synchronising call
 * (pq_ctx_sync, a load, a plan run) returns PQ_ERR_DEVICE once and clears
 * the status word, after which the context works normally.  Replaces the
 * reference's failure behaviour for a missing or bad device result
 * (src/backends/interactive.jl:44-49: an error, no process exit). */
int pq_selftest_wait_expiry(pq_ctx* ctx, uint32_t polls, int* expired);

#ifdef __cplusplus
}
#endif
#endif /* PQGB300_H */
