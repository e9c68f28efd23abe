// Candidate-plan scoring on the device: the complex multiply-adds and the
// largest intermediate of many SSA pair plans of one network at once.
//
// The planners produce many candidate orders (seeded Boltzmann-greedy draws
// after src/layer2/bgreedy_contraction.jl:17-131, randomized qubit sweeps)
// and keep the cheapest by the reference's flop count (src/backends.jl:30-41:
// |C| times the contracted extent per pair).  Scoring a candidate is one
// sequential pass over its steps, so candidates are independent: one warp per
// candidate, its label counts in shared memory, the label lists of its
// intermediates in a global scratch area, the lanes of the warp sharing each
// step's label work.  The label rule is the executor's: a label is summed at
// the first step after which no live tensor and no output carries it.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "pq_types.cuh"

namespace pq {
int check_status(Ctx* ctx);
}
using namespace pq;

namespace {

constexpr int kPcCap = 64;                 // label capacity of one intermediate's list
constexpr int kPcMaxLabels = 40000;        // label counts of one candidate in shared memory

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One warp per candidate (blockDim.x == 32).  cmacs[c] = -1 marks a candidate
// whose steps are not a valid SSA plan, -2 one with an intermediate of more
// than kPcCap labels (at least 2^64 elements: its cost is reported as
// infinite).
__global__ void __launch_bounds__(32)
    k_plan_cost(const int32_t* __restrict__ leaf_off, const int32_t* __restrict__ leaf_rank,
                const int32_t* __restrict__ leaf_labels, int n_leaves, const double* __restrict__ l2dim,
                const int32_t* __restrict__ cnt0, int n_labels, const int32_t* __restrict__ steps, int n_steps,
                int32_t* __restrict__ vals, int32_t* __restrict__ vrank, double* __restrict__ cmacs,
                double* __restrict__ max_l2) {
  extern __shared__ int32_t cnt[];
  const int cand = blockIdx.x, lane = threadIdx.x;
  for (int i = lane; i < n_labels; i += 32) cnt[i] = cnt0[i];
  __syncwarp();
  const int32_t* st = steps + (size_t)cand * 2 * n_steps;
  int32_t* my_vals = vals + (size_t)cand * n_steps * kPcCap;
  int32_t* my_rank = vrank + (size_t)cand * n_steps;
  double cost = 0.0, mx = 0.0;
  bool bad = false, wide = false;
  for (int s = 0; s < n_steps && !bad; ++s) {
    const int x = st[2 * s], y = st[2 * s + 1];
    if (x < 0 || y < 0 || x >= n_leaves + s || y >= n_leaves + s) {
      bad = true;
      break;
    }
    const int32_t* pa = x < n_leaves ? leaf_labels + leaf_off[x] : my_vals + (size_t)(x - n_leaves) * kPcCap;
    const int32_t* pb = y < n_leaves ? leaf_labels + leaf_off[y] : my_vals + (size_t)(y - n_leaves) * kPcCap;
    const int ra = x < n_leaves ? leaf_rank[x] : my_rank[x - n_leaves];
    const int rb = y < n_leaves ? leaf_rank[y] : my_rank[y - n_leaves];
    for (int i = lane; i < ra; i += 32) atomicSub(&cnt[pa[i]], 1);
    for (int i = lane; i < rb; i += 32) atomicSub(&cnt[pb[i]], 1);
    __syncwarp();
    // the union of both lists, first occurrences in order (a tensor's own
    // labels are distinct): entry j < ra is pa[j]; entry ra + j is pb[j]
    // unless pa holds it
    double l2u = 0.0, l2k = 0.0;
    int nkeep = 0;
    int32_t* out = my_vals + (size_t)s * kPcCap;
    for (int base = 0; base < ra + rb; base += 32) {
      const int idx = base + lane;
      int l = -1;
      bool first = false;
      if (idx < ra) {
        l = pa[idx];
        first = true;
      } else if (idx < ra + rb) {
        l = pb[idx - ra];
        first = true;
        for (int j = 0; j < ra; ++j)
          if (pa[j] == l) first = false;
      }
      const bool keep = first && cnt[l] > 0;
      if (first) l2u += l2dim[l];
      if (keep) l2k += l2dim[l];
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      const int at = nkeep + __popc(m & ((1u << lane) - 1));
      if (keep && at < kPcCap) out[at] = l;
      nkeep += __popc(m);
    }
    __syncwarp();
    if (nkeep > kPcCap) {
      wide = true;
      break;
    }
    for (int i = lane; i < nkeep; i += 32) atomicAdd(&cnt[out[i]], 1);
    if (lane == 0) my_rank[s] = nkeep;
    __syncwarp();
    l2u = warp_sum(l2u);
    l2k = warp_sum(l2k);
    cost += exp2(l2u);
    mx = fmax(mx, l2k);
  }
  if (lane == 0) {
    cmacs[cand] = bad ? -1.0 : (wide ? -2.0 : cost);
    max_l2[cand] = mx;
  }
}

}  // namespace

extern "C" {

int pq_plan_cost_batch(pq_ctx* c, int n_leaves, const int32_t* leaf_ranks, const int32_t* leaf_labels,
                       int n_labels, const int64_t* label_dims, int n_steps, int n_cand, const int32_t* steps,
                       int n_out, const int32_t* out_labels, double* cmacs, double* max_elems) {
  if (!c) return PQ_ERR_INVALID;
  Ctx* ctx = &c->impl;
  if (n_leaves < 1 || !leaf_ranks || n_steps < 0 || n_cand < 0 || (n_cand && n_steps && !steps) ||
      (n_out && !out_labels) || (n_cand && (!cmacs || !max_elems)) || n_labels < 0 ||
      (n_labels && !label_dims))
    return fail(ctx, PQ_ERR_INVALID, "plan_cost_batch: bad arguments");
  if (n_labels > kPcMaxLabels)
    return fail(ctx, PQ_ERR_UNSUPPORTED, "plan_cost_batch: more than " + std::to_string(kPcMaxLabels) + " labels");
  if (n_cand == 0) return PQ_OK;
  std::vector<double> l2dim(std::max(1, n_labels));
  for (int i = 0; i < n_labels; ++i) {
    if (label_dims[i] < 1) return fail(ctx, PQ_ERR_INVALID, "plan_cost_batch: label extent below 1");
    l2dim[i] = std::log2((double)label_dims[i]);
  }
  std::vector<int32_t> off(n_leaves), cnt(std::max(1, n_labels), 0);
  int pos = 0;
  for (int i = 0; i < n_leaves; ++i) {
    if (leaf_ranks[i] < 0 || leaf_ranks[i] > kPcCap)
      return fail(ctx, PQ_ERR_INVALID, "plan_cost_batch: leaf rank out of range");
    off[i] = pos;
    for (int j = 0; j < leaf_ranks[i]; ++j) {
      const int x = leaf_labels[pos++];
      if (x < 0 || x >= n_labels) return fail(ctx, PQ_ERR_INVALID, "plan_cost_batch: label out of range");
      cnt[x]++;
    }
  }
  for (int i = 0; i < n_out; ++i) {
    if (out_labels[i] < 0 || out_labels[i] >= n_labels)
      return fail(ctx, PQ_ERR_INVALID, "plan_cost_batch: output label out of range");
    cnt[out_labels[i]]++;
  }
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "plan_cost_batch: set device");
  // one device block: [off | ranks | labels | cnt | steps | l2dim (8-aligned) | results | vals | vrank]
  const size_t n_lab_total = (size_t)pos;
  auto up8 = [](size_t b) { return (b + 7) & ~(size_t)7; };
  const size_t b_off = up8((size_t)n_leaves * 4), b_rank = b_off, b_lab = up8(std::max<size_t>(1, n_lab_total) * 4),
               b_cnt = up8(cnt.size() * 4), b_steps = up8(std::max<size_t>(1, (size_t)n_cand * 2 * n_steps) * 4),
               b_l2 = l2dim.size() * 8, b_res = (size_t)n_cand * 8,
               b_vals = (size_t)n_cand * std::max(1, n_steps) * kPcCap * 4,
               b_vrank = up8((size_t)n_cand * std::max(1, n_steps) * 4);
  const size_t total = b_off + b_rank + b_lab + b_cnt + b_steps + b_l2 + 2 * b_res + b_vals + b_vrank;
  char* d = nullptr;
  int st = dev_alloc(ctx, total, (void**)&d);
  if (st) return st;
  size_t o = 0;
  int32_t* d_off = (int32_t*)(d + o);
  o += b_off;
  int32_t* d_rank = (int32_t*)(d + o);
  o += b_rank;
  int32_t* d_lab = (int32_t*)(d + o);
  o += b_lab;
  int32_t* d_cnt = (int32_t*)(d + o);
  o += b_cnt;
  int32_t* d_steps = (int32_t*)(d + o);
  o += b_steps;
  double* d_l2 = (double*)(d + o);
  o += b_l2;
  double* d_cost = (double*)(d + o);
  o += b_res;
  double* d_mx = (double*)(d + o);
  o += b_res;
  int32_t* d_vals = (int32_t*)(d + o);
  o += b_vals;
  int32_t* d_vrank = (int32_t*)(d + o);
  const struct {
    void* dst;
    const void* src;
    size_t bytes;
  } ups[] = {{d_off, off.data(), (size_t)n_leaves * 4},
             {d_rank, leaf_ranks, (size_t)n_leaves * 4},
             {d_lab, leaf_labels, n_lab_total * 4},
             {d_cnt, cnt.data(), (size_t)n_labels * 4},
             {d_steps, steps, (size_t)n_cand * 2 * n_steps * 4},
             {d_l2, l2dim.data(), (size_t)n_labels * 8}};
  for (const auto& u : ups)
    if (u.bytes && e == cudaSuccess) e = cudaMemcpyAsync(u.dst, u.src, u.bytes, cudaMemcpyHostToDevice, ctx->stream);
  const size_t smem = (size_t)std::max(1, n_labels) * 4;
  if (e == cudaSuccess && smem > 48 * 1024)
    e = cudaFuncSetAttribute(k_plan_cost, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) {
    k_plan_cost<<<n_cand, 32, smem, ctx->stream>>>(
        d_off, d_rank, d_lab, n_leaves, d_l2, d_cnt, n_labels, d_steps, n_steps, d_vals, d_vrank, d_cost, d_mx);
    e = cudaGetLastError();
    ctx->launches += 1;
  }
  std::vector<double> mx(n_cand);
  if (e == cudaSuccess) e = cudaMemcpyAsync(cmacs, d_cost, (size_t)n_cand * 8, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(mx.data(), d_mx, (size_t)n_cand * 8, cudaMemcpyDeviceToHost, ctx->stream);
  dev_free(ctx, d, total);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "plan_cost_batch");
  st = check_status(ctx);  // also orders the host copies above
  if (st) return st;
  for (int i = 0; i < n_cand; ++i) {
    if (cmacs[i] == -1.0)
      return fail(ctx, PQ_ERR_INVALID, "plan_cost_batch: candidate " + std::to_string(i) +
                                           " is not an SSA plan of the leaves");
    if (cmacs[i] == -2.0) {
      cmacs[i] = max_elems[i] = HUGE_VAL;
      continue;
    }
    max_elems[i] = std::exp2(mx[i]);
  }
  return PQ_OK;
}

}  // extern "C"
