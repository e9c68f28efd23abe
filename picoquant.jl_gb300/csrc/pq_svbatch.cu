// Batched state-vector execution of many circuits of different sizes (the
// uneven-circuit workload: hundreds of circuits of 12-30 qubits, a few dozen
// amplitudes of each).
//
// Each circuit is given as blocks of at most four qubits (a 2^k x 2^k matrix
// per block, applied in order to a complex64 state of 2^n amplitudes, qubit q
// at bit q of the amplitude index).  Contracting such a circuit in the
// reference (src/layer2.jl:294-321, a pair plan over the gate nodes) is one
// pass over the state per gate; here the passes of different circuits share
// launches: launch s applies the s-th block of every circuit of a chunk, one
// persistent-style kernel over a per-launch table of (state, block) entries,
// the blocks of a launch divided among the entries in proportion to their
// state sizes.  Chunks of circuits whose states fit a byte budget run one
// after the other in one arena; the whole batch -- state initialisation, every
// block launch of every chunk and the amplitude gather -- is recorded as a
// CUDA graph on the first execution and replayed afterwards.
//
// A block pass is in place: thread r takes fiber r (the 2^k amplitudes whose
// index bits outside the block's qubits spell r), loads them, multiplies by the
// block's matrix from shared memory (FP32, as the skinny-pair kernel for
// complex64 results) and writes them back.  Memory-bound: 16 bytes moved per
// amplitude (read and write) against at most 16 complex multiply-adds.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "pq_types.cuh"

namespace pq {
int check_status(Ctx* ctx);
}
using namespace pq;

namespace {

constexpr int kSvThreads = 256;
constexpr int kSvMaxQ = 4;
constexpr int kSvMaxDim = 1 << kSvMaxQ;
constexpr int64_t kSvFibersPerThread = 2;  // fibers per thread per block (on average)

struct SvOp {
  float2* state;      // the circuit's state, 2^n complex64
  const float2* mat;  // 2^k x 2^k complex64, element (out, in) at out + in 2^k
  int64_t rows;       // 2^(n - k) fibers
  int k;
  int q[kSvMaxQ];     // bit positions of the block's qubits, bit i of a fiber index <-> q[i]
  int qs[kSvMaxQ];    // the same positions in ascending order
};

// The fibers [first, rows) step `stride` of one block pass with D = 2^k
// amplitudes per fiber (specialised per k: every thread of a CUDA block works
// on the same table entry, so the branch on k is uniform).
struct SvQubits {
  int q[kSvMaxQ], qs[kSvMaxQ];
};

template <int D>
__device__ __forceinline__ void sv_pass(float2* __restrict__ S, const float2* __restrict__ U, const SvQubits Q,
                                        int64_t first, int64_t rows, int64_t stride) {
  constexpr int k = D == 2 ? 1 : (D == 4 ? 2 : (D == 8 ? 3 : 4));
  constexpr int G = D < 4 ? D : 4;  // outputs per group (the matrix is read a group of rows at a time)
  // offset of amplitude c of a fiber relative to its base (states have at
  // most 2^31 amplitudes, so offsets fit 32 bits)
  auto off = [&](int c) {
    int o = 0;
#pragma unroll
    for (int i = 0; i < k; ++i) o += ((c >> i) & 1) << Q.q[i];
    return o;
  };
  for (int64_t r = first; r < rows; r += stride) {
    // base index: r with a zero bit inserted at each block position (ascending)
    int64_t base = r;
#pragma unroll
    for (int i = 0; i < k; ++i) {
      const int p = Q.qs[i];
      base = ((base >> p) << (p + 1)) | (base & ((int64_t(1) << p) - 1));
    }
    float2 a[D];
#pragma unroll
    for (int c = 0; c < D; ++c) a[c] = S[base + off(c)];
    // not unrolled: the matrix entries are read from shared memory per group
    // instead of being hoisted into registers
#pragma unroll 1
    for (int c0 = 0; c0 < D; c0 += G) {
      float2 acc[G];
#pragma unroll
      for (int j = 0; j < G; ++j) acc[j] = make_float2(0.f, 0.f);
#pragma unroll
      for (int ci = 0; ci < D; ++ci) {
#pragma unroll
        for (int j = 0; j < G; ++j) cfma(acc[j], a[ci], U[c0 + j + ci * D]);
      }
#pragma unroll
      for (int j = 0; j < G; ++j) S[base + off(c0 + j)] = acc[j];
    }
  }
}

__global__ void __launch_bounds__(kSvThreads)
    k_sv_group(const SvOp* __restrict__ ops, const int64_t* __restrict__ blk, int nops) {
  __shared__ float2 U[kSvMaxDim * kSvMaxDim];
  __shared__ int s_op;
  if (threadIdx.x == 0) {
    // the entry owning this block: the last one with blk[entry] <= blockIdx.x
    int lo = 0, hi = nops - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) / 2;
      if (blk[mid] <= (int64_t)blockIdx.x)
        lo = mid;
      else
        hi = mid - 1;
    }
    s_op = lo;
  }
  __syncthreads();
  const int o_id = s_op;
  const int k = ops[o_id].k;
  const int D = 1 << k;
  const float2* mat = ops[o_id].mat;
  for (int t = threadIdx.x; t < D * D; t += blockDim.x) U[t] = mat[t];
  __syncthreads();
  float2* S = ops[o_id].state;
  const int64_t rows = ops[o_id].rows;
  SvQubits Q;
#pragma unroll
  for (int i = 0; i < kSvMaxQ; ++i) {
    Q.q[i] = ops[o_id].q[i];
    Q.qs[i] = ops[o_id].qs[i];
  }
  const int64_t stride = (blk[o_id + 1] - blk[o_id]) * kSvThreads;
  const int64_t first = ((int64_t)blockIdx.x - blk[o_id]) * kSvThreads + threadIdx.x;
  switch (k) {
    case 1: sv_pass<2>(S, U, Q, first, rows, stride); break;
    case 2: sv_pass<4>(S, U, Q, first, rows, stride); break;
    case 3: sv_pass<8>(S, U, Q, first, rows, stride); break;
    default: sv_pass<16>(S, U, Q, first, rows, stride); break;
  }
}

// |0...0> in every state of a chunk: the used arena zeroed beforehand, then
// amplitude 0 of each state set to 1.
__global__ void k_sv_init(float2* arena, const int64_t* __restrict__ state_off, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) arena[state_off[i]] = make_float2(1.f, 0.f);
}

// out[i] = arena[idx[i]] as complex128.
__global__ void k_sv_gather(const float2* __restrict__ arena, const int64_t* __restrict__ idx, int64_t n,
                            double2* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const float2 v = arena[idx[i]];
    out[i] = make_double2((double)v.x, (double)v.y);
  }
}

struct Launch {
  int op0, nops;
  int64_t blk0, blocks;  // prefix table at d_blk[blk0 .. blk0 + nops], total blocks
};

struct Chunk {
  int64_t used_bytes;
  int soff0, nstates;  // state offsets at d_soff[soff0 ..]
  int launch0, nlaunch;
  int64_t amp0, namp;
};

}  // namespace

struct pq_svbatch {
  Ctx* ctx = nullptr;
  float2* arena = nullptr;
  size_t arena_bytes = 0;
  float2* mats = nullptr;
  size_t mats_bytes = 0;
  SvOp* d_ops = nullptr;
  size_t ops_bytes = 0;
  int64_t* d_blk = nullptr;
  size_t blk_bytes = 0;
  int64_t* d_soff = nullptr;
  size_t soff_bytes = 0;
  int64_t* d_idx = nullptr;
  size_t idx_bytes = 0;
  double2* d_amps = nullptr;
  size_t amps_bytes = 0;
  int64_t total_amps = 0;
  std::vector<Launch> launches;
  std::vector<Chunk> chunks;
  std::vector<int64_t> perm;  // input-order amplitude a is gathered at perm[a]
  cudaGraphExec_t gexec = nullptr;
  int64_t kernel_launches = 0;
};

namespace {

void release(pq_svbatch* b) {
  Ctx* ctx = b->ctx;
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  dev_free(ctx, b->arena, b->arena_bytes);
  dev_free(ctx, b->mats, b->mats_bytes);
  dev_free(ctx, b->d_ops, b->ops_bytes);
  dev_free(ctx, b->d_blk, b->blk_bytes);
  dev_free(ctx, b->d_soff, b->soff_bytes);
  dev_free(ctx, b->d_idx, b->idx_bytes);
  dev_free(ctx, b->d_amps, b->amps_bytes);
}

cudaError_t issue(pq_svbatch* b) {
  cudaStream_t s = b->ctx->stream;
  for (const Chunk& c : b->chunks) {
    cudaError_t e = cudaMemsetAsync(b->arena, 0, (size_t)c.used_bytes, s);
    if (e != cudaSuccess) return e;
    k_sv_init<<<(c.nstates + 255) / 256, 256, 0, s>>>(b->arena, b->d_soff + c.soff0, c.nstates);
    for (int l = c.launch0; l < c.launch0 + c.nlaunch; ++l) {
      const Launch& L = b->launches[l];
      k_sv_group<<<(unsigned)L.blocks, kSvThreads, 0, s>>>(b->d_ops + L.op0, b->d_blk + L.blk0, L.nops);
    }
    if (c.namp)
      k_sv_gather<<<(unsigned)((c.namp + 255) / 256), 256, 0, s>>>(b->arena, b->d_idx + c.amp0, c.namp,
                                                                    b->d_amps + c.amp0);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <typename T>
int upload(Ctx* ctx, const std::vector<T>& h, T** d, size_t* bytes) {
  *bytes = std::max<size_t>(16, h.size() * sizeof(T));
  int st = dev_alloc(ctx, *bytes, (void**)d);
  if (st) return st;
  if (!h.empty()) {
    cudaError_t e = cudaMemcpyAsync(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "svbatch upload");
  }
  return PQ_OK;
}

}  // namespace

extern "C" {

int pq_svbatch_create(pq_ctx* c, int n_circ, const int32_t* n_qubits, const int32_t* n_blocks,
                      const int32_t* block_k, const int32_t* block_qubits, const double* block_mats,
                      const int32_t* n_amps, const int64_t* amp_idx, int64_t state_budget_bytes,
                      pq_svbatch** out) {
  if (!c || !out) return PQ_ERR_INVALID;
  *out = nullptr;
  Ctx* ctx = &c->impl;
  if (n_circ < 0 || (n_circ && (!n_qubits || !n_blocks || !n_amps)))
    return fail(ctx, PQ_ERR_INVALID, "svbatch_create: bad arguments");
  // ---- validate and index the flattened inputs
  std::vector<int64_t> blk_first(n_circ + 1, 0), q_first, mat_first, amp_first(n_circ + 1, 0);
  int64_t nblk_total = 0;
  for (int i = 0; i < n_circ; ++i) {
    if (n_qubits[i] < 1 || n_qubits[i] > 31 || n_blocks[i] < 0 || n_amps[i] < 0)
      return fail(ctx, PQ_ERR_INVALID, "svbatch_create: circuit " + std::to_string(i) + " has bad sizes");
    blk_first[i + 1] = blk_first[i] + n_blocks[i];
    amp_first[i + 1] = amp_first[i] + n_amps[i];
  }
  nblk_total = blk_first[n_circ];
  if ((nblk_total && (!block_k || !block_qubits || !block_mats)) || (amp_first[n_circ] && !amp_idx))
    return fail(ctx, PQ_ERR_INVALID, "svbatch_create: missing block or amplitude arrays");
  q_first.assign(nblk_total + 1, 0);
  mat_first.assign(nblk_total + 1, 0);
  for (int i = 0; i < n_circ; ++i)
    for (int64_t j = blk_first[i]; j < blk_first[i + 1]; ++j) {
      const int k = block_k[j];
      if (k < 1 || k > kSvMaxQ || k > n_qubits[i])
        return fail(ctx, PQ_ERR_INVALID, "svbatch_create: block of " + std::to_string(k) + " qubits");
      q_first[j + 1] = q_first[j] + k;
      mat_first[j + 1] = mat_first[j] + (int64_t(1) << (2 * k));
      for (int t = 0; t < k; ++t) {
        const int qb = block_qubits[q_first[j] + t];
        if (qb < 0 || qb >= n_qubits[i])
          return fail(ctx, PQ_ERR_INVALID, "svbatch_create: qubit index out of range");
        for (int u = 0; u < t; ++u)
          if (block_qubits[q_first[j] + u] == qb) return fail(ctx, PQ_ERR_INVALID, "svbatch_create: repeated qubit");
      }
    }
  for (int i = 0; i < n_circ; ++i)
    for (int64_t a = amp_first[i]; a < amp_first[i + 1]; ++a)
      if (amp_idx[a] < 0 || amp_idx[a] >= (int64_t(1) << n_qubits[i]))
        return fail(ctx, PQ_ERR_INVALID, "svbatch_create: amplitude index out of range");
  const int64_t max_state = [&] {
    int64_t m = 0;
    for (int i = 0; i < n_circ; ++i) m = std::max<int64_t>(m, (int64_t(8) << n_qubits[i]));
    return m;
  }();
  const int64_t budget = std::max<int64_t>(state_budget_bytes, max_state);

  pq_svbatch* b = new pq_svbatch();
  b->ctx = ctx;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) {
    delete b;
    return cuda_fail(ctx, e, "svbatch_create: set device");
  }
  // ---- chunks: circuits by decreasing size, packed until the budget is full
  std::vector<int> order(n_circ);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return n_qubits[x] > n_qubits[y]; });
  std::vector<SvOp> ops;
  std::vector<int64_t> blk, soff, idx;
  std::vector<float2> mats((size_t)mat_first[nblk_total]);
  for (int64_t t = 0; t < mat_first[nblk_total]; ++t)
    mats[t] = make_float2((float)block_mats[2 * t], (float)block_mats[2 * t + 1]);
  std::vector<int64_t> amp_pos(n_circ, 0);  // where circuit i's amplitudes land in the gathered output
  int64_t arena_elems = 0;
  size_t p = 0;
  int64_t amp_cursor = 0;
  while (p < order.size()) {
    Chunk ch;
    ch.soff0 = (int)soff.size();
    ch.launch0 = (int)b->launches.size();
    ch.amp0 = amp_cursor;
    std::vector<int> members;
    std::vector<int64_t> base;
    int64_t used = 0;
    while (p < order.size()) {
      const int i = order[p];
      const int64_t sz = int64_t(1) << n_qubits[i];
      if (!members.empty() && (used + sz) * 8 > budget) break;
      members.push_back(i);
      base.push_back(used);
      used += sz;
      ++p;
    }
    ch.used_bytes = used * 8;
    ch.nstates = (int)members.size();
    arena_elems = std::max(arena_elems, used);
    for (size_t m = 0; m < members.size(); ++m) {
      soff.push_back(base[m]);
      const int i = members[m];
      amp_pos[i] = amp_cursor;
      for (int64_t a = amp_first[i]; a < amp_first[i + 1]; ++a) idx.push_back(base[m] + amp_idx[a]);
      amp_cursor += n_amps[i];
    }
    ch.namp = amp_cursor - ch.amp0;
    int max_steps = 0;
    for (int i : members) max_steps = std::max(max_steps, n_blocks[i]);
    for (int s = 0; s < max_steps; ++s) {
      Launch L;
      L.op0 = (int)ops.size();
      L.blk0 = (int64_t)blk.size();
      int64_t nb = 0;
      for (size_t m = 0; m < members.size(); ++m) {
        const int i = members[m];
        if (s >= n_blocks[i]) continue;
        const int64_t j = blk_first[i] + s;
        SvOp op;
        std::memset(&op, 0, sizeof(op));
        op.k = block_k[j];
        op.rows = int64_t(1) << (n_qubits[i] - op.k);
        op.state = nullptr;  // arena + base, fixed below once the arena exists
        op.mat = reinterpret_cast<const float2*>(mat_first[j]);  // element offset, fixed below
        for (int t = 0; t < op.k; ++t) op.q[t] = op.qs[t] = block_qubits[q_first[j] + t];
        std::sort(op.qs, op.qs + op.k);
        op.state = reinterpret_cast<float2*>(base[m]);
        ops.push_back(op);
        blk.push_back(nb);
        nb += std::max<int64_t>(1, (op.rows + kSvThreads * kSvFibersPerThread - 1) /
                                       (kSvThreads * kSvFibersPerThread));
      }
      blk.push_back(nb);
      L.nops = (int)ops.size() - L.op0;
      L.blocks = nb;
      if (nb > 0x7fffffffLL) {
        delete b;
        return fail(ctx, PQ_ERR_UNSUPPORTED, "svbatch_create: launch too large");
      }
      b->launches.push_back(L);
    }
    ch.nlaunch = (int)b->launches.size() - ch.launch0;
    b->chunks.push_back(ch);
  }
  b->total_amps = amp_cursor;
  // ---- device buffers
  b->arena_bytes = (size_t)std::max<int64_t>(arena_elems, 1) * 8;
  int st = dev_alloc(ctx, b->arena_bytes, (void**)&b->arena);
  if (!st) st = upload(ctx, mats, &b->mats, &b->mats_bytes);
  if (!st) {
    for (SvOp& op : ops) {
      op.state = b->arena + reinterpret_cast<int64_t>(op.state);
      op.mat = b->mats + reinterpret_cast<int64_t>(op.mat);
    }
    st = upload(ctx, ops, &b->d_ops, &b->ops_bytes);
  }
  if (!st) st = upload(ctx, blk, &b->d_blk, &b->blk_bytes);
  if (!st) st = upload(ctx, soff, &b->d_soff, &b->soff_bytes);
  if (!st) st = upload(ctx, idx, &b->d_idx, &b->idx_bytes);
  if (!st) {
    b->amps_bytes = std::max<size_t>(16, (size_t)b->total_amps * sizeof(double2));
    st = dev_alloc(ctx, b->amps_bytes, (void**)&b->d_amps);
  }
  if (!st) st = check_status(ctx);  // the uploads above read host vectors that end here
  if (st) {
    release(b);
    delete b;
    return st;
  }
  // gathered amplitudes are in chunk order: the map back to input order
  b->perm.resize((size_t)b->total_amps);
  for (int i = 0; i < n_circ; ++i)
    for (int64_t a = 0; a < n_amps[i]; ++a) b->perm[(size_t)(amp_first[i] + a)] = amp_pos[i] + a;
  b->kernel_launches = 0;
  for (const Chunk& ch : b->chunks) b->kernel_launches += 1 + ch.nlaunch + (ch.namp ? 1 : 0);
  *out = b;
  return PQ_OK;
}

int pq_svbatch_execute(pq_svbatch* b, double* amps_out) {
  if (!b) return PQ_ERR_INVALID;
  Ctx* ctx = b->ctx;
  if (b->total_amps && !amps_out) return fail(ctx, PQ_ERR_INVALID, "svbatch_execute: no output buffer");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "svbatch_execute: set device");
  if (!b->gexec) {
    // record the whole batch once; the first execution runs the graph too
    e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "svbatch_execute: begin capture");
    cudaError_t ei = issue(b);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(ctx->stream, &g);
    if (ei != cudaSuccess || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return cuda_fail(ctx, ei != cudaSuccess ? ei : e, "svbatch_execute: capture");
    }
    e = cudaGraphInstantiate(&b->gexec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "svbatch_execute: instantiate");
  }
  e = cudaGraphLaunch(b->gexec, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "svbatch_execute: graph launch");
  ctx->launches += b->kernel_launches;
  std::vector<double2> h((size_t)b->total_amps);
  if (b->total_amps) {
    e = cudaMemcpyAsync(h.data(), b->d_amps, h.size() * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "svbatch_execute: read amplitudes");
  }
  int st = check_status(ctx);
  if (st) return st;
  for (size_t a = 0; a < h.size(); ++a) {
    amps_out[2 * a] = h[(size_t)b->perm[a]].x;
    amps_out[2 * a + 1] = h[(size_t)b->perm[a]].y;
  }
  return PQ_OK;
}

int pq_svbatch_info(pq_svbatch* b, int64_t* launches, int64_t* chunks, int64_t* arena_bytes) {
  if (!b) return PQ_ERR_INVALID;
  if (launches) *launches = b->kernel_launches;
  if (chunks) *chunks = (int64_t)b->chunks.size();
  if (arena_bytes) *arena_bytes = (int64_t)b->arena_bytes;
  return PQ_OK;
}

int pq_svbatch_destroy(pq_svbatch* b) {
  if (!b) return PQ_ERR_INVALID;
  cudaSetDevice(b->ctx->device);
  release(b);
  cudaStreamSynchronize(b->ctx->stream);
  delete b;
  return PQ_OK;
}

}  // extern "C"
