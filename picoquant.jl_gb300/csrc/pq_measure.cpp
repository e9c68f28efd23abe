// Timing harness for the learned cost model: runs arbitrary pairwise
// contractions with the context's kernels and storage policy and measures
// each with CUDA events (the training data of the MLP comes from here).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "pq_internal.h"

namespace pq {
int check_status(Ctx* ctx);
}
using namespace pq;

extern "C" {

int pq_measure_pairs(pq_ctx* c, int n_pairs, const int32_t* a_ranks, const int32_t* b_ranks, const int32_t* labels,
                     const int64_t* dims, int reps, float* ms, double* feats) {
  if (!c || n_pairs < 0 || (n_pairs && (!a_ranks || !b_ranks || !labels || !dims || !ms || !feats)) || reps < 1)
    return PQ_ERR_INVALID;
  Ctx* ctx = &c->impl;
  std::vector<PairPlan> plans(n_pairs);
  std::vector<int> ta(n_pairs), tb(n_pairs), tc(n_pairs);
  size_t amax = 16, bmax = 16, cmax = 16, smax = 0;
  int64_t pos = 0;
  for (int p = 0; p < n_pairs; ++p) {
    if (a_ranks[p] < 0 || b_ranks[p] < 0 || a_ranks[p] > PQ_MAX_RANK || b_ranks[p] > PQ_MAX_RANK)
      return fail(ctx, PQ_ERR_INVALID, "measure_pairs: bad rank");
    std::vector<int> la(labels + pos, labels + pos + a_ranks[p]);
    std::vector<int64_t> da(dims + pos, dims + pos + a_ranks[p]);
    pos += a_ranks[p];
    std::vector<int> lb(labels + pos, labels + pos + b_ranks[p]);
    std::vector<int64_t> db(dims + pos, dims + pos + b_ranks[p]);
    pos += b_ranks[p];
    std::string err;
    if (!analyse_pair(la, da, lb, db, symdiff_labels(la, lb), ctx->precision, plans[p], err, &ctx->tuning))
      return fail(ctx, PQ_ERR_INVALID, "measure_pairs: pair " + std::to_string(p) + ": " + err);
    const PairPlan& q = plans[p];
    ta[p] = storage_dtype(ctx, q.asize);
    tb[p] = storage_dtype(ctx, q.bsize);
    tc[p] = storage_dtype(ctx, q.csize);
    amax = std::max(amax, (size_t)q.asize * elem_bytes(ta[p]));
    bmax = std::max(bmax, (size_t)q.bsize * elem_bytes(tb[p]));
    cmax = std::max(cmax, (size_t)q.csize * elem_bytes(tc[p]));
    if (q.kclass == KC_TC) smax = std::max(smax, tc_scratch_bytes(ctx->precision, q.m));
  }
  void *A = nullptr, *B = nullptr, *C = nullptr, *S = nullptr;
  int st = dev_alloc(ctx, amax, &A);
  if (!st) st = dev_alloc(ctx, bmax, &B);
  if (!st) st = dev_alloc(ctx, cmax, &C);
  if (!st && smax) st = dev_alloc(ctx, smax, &S);
  cudaError_t e = cudaSuccess;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (!st) {
    // a fixed non-denormal bit pattern (timing does not depend on values)
    e = cudaMemsetAsync(A, 0x3c, amax, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(B, 0x3c, bmax, ctx->stream);
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto run = [&](int p) -> cudaError_t {
      const PairPlan& q = plans[p];
      ctx->launches += q.kclass == KC_TC ? 3 : 1;
      if (q.kclass == KC_TC)
        return launch_tc(ctx->precision, ta[p], tb[p], tc[p], A, B, C, q.m, S, smax, ctx->d_status, ctx->stream);
      if (q.kclass == KC_GEMM) return launch_gemm(ta[p], tb[p], tc[p], A, B, C, q.m, ctx->stream);
      if (q.kclass == KC_SKINNY) return launch_skinny(ta[p], tb[p], tc[p], A, B, C, q.m, ctx->stream);
      return launch_generic(ta[p], tb[p], tc[p], A, B, C, q.g, ctx->stream);
    };
    for (int p = 0; p < n_pairs && e == cudaSuccess; ++p) {
      e = run(p);  // warm-up
      if (e == cudaSuccess) e = cudaEventRecord(e0, ctx->stream);
      for (int r = 0; r < reps && e == cudaSuccess; ++r) e = run(p);
      if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->stream);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float t = 0;
      if (e == cudaSuccess) cudaEventElapsedTime(&t, e0, e1);
      ms[p] = t / reps;
      const PairPlan& q = plans[p];
      double* f = feats + 8 * p;
      f[0] = std::log2((double)q.asize);
      f[1] = std::log2((double)q.bsize);
      f[2] = std::log2((double)q.csize);
      f[3] = std::log2((double)q.ksize);
      f[4] = std::log2((double)q.run_a);
      f[5] = std::log2((double)q.run_b);
      f[6] = (double)q.kclass;
      f[7] = (double)elem_bytes(ta[p]) * q.asize + (double)elem_bytes(tb[p]) * q.bsize +
             (double)elem_bytes(tc[p]) * q.csize;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
  }
  dev_free(ctx, A, amax);
  dev_free(ctx, B, bmax);
  dev_free(ctx, C, cmax);
  if (S) dev_free(ctx, S, smax);
  if (st) return st;
  if (e != cudaSuccess) return cuda_fail(ctx, e, "measure_pairs");
  return check_status(ctx);
}

}  // extern "C"
