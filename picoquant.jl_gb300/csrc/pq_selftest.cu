// Self-test of the bounded-wait error path of the tcgen05 kernels.
//
// The tensor-core kernels (pq_tc.cu, pq_oz.cu) wait on shared-memory
// mbarriers with a poll limit; when a wait expires they record it in the
// context's status word (report_timeout), release what they hold and return,
// and the next synchronising call on the context reports PQ_ERR_DEVICE.  In
// a correct run no wait expires, so this file provides a kernel whose wait
// expires by construction: one thread initialises an mbarrier that expects
// one arrival, never arrives, and polls it a caller-given, bounded number of
// times.  It issues no bulk copy, no MMA and holds no TMEM, so nothing is in
// flight when it returns; the context stays usable.
#include <cuda_runtime.h>

#include "pq_tcgen05.cuh"
#include "pq_types.cuh"

namespace pq {
int check_status(Ctx* ctx);
}
using namespace pq;
using namespace pq::tcg;

namespace {

constexpr uint32_t kMaxSelftestPolls = 1u << 20;

__global__ void __launch_bounds__(32) k_wait_expiry(uint32_t polls, int* status, int* expired) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_init_fence();
  }
  __syncwarp();
  if (threadIdx.x == 0) {
    // phase 0 never completes: nobody arrives on `bar`
    const bool ok = mbar_wait_polls(&bar, 0, polls);
    if (!ok) report_timeout(status);
    *expired = ok ? 0 : 1;
  }
}

}  // namespace

extern "C" {

int pq_selftest_wait_expiry(pq_ctx* c, uint32_t polls, int* expired) {
  if (!c || !expired) return PQ_ERR_INVALID;
  Ctx* ctx = &c->impl;
  if (polls == 0 || polls > kMaxSelftestPolls)
    return fail(ctx, PQ_ERR_INVALID,
                "selftest_wait_expiry: polls must be in 1.." + std::to_string(kMaxSelftestPolls));
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "selftest_wait_expiry: set device");
  int* d_flag = nullptr;
  int st = dev_alloc(ctx, sizeof(int), (void**)&d_flag);
  if (st != PQ_OK) return st;
  k_wait_expiry<<<1, 32, 0, ctx->stream>>>(polls, ctx->d_status, d_flag);
  e = cudaGetLastError();
  ctx->launches += 1;
  int h = -1;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
  dev_free(ctx, d_flag, sizeof(int));
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "selftest_wait_expiry");
  *expired = h;
  // the status word is left set: the caller's next synchronising call reports it
  return PQ_OK;
}

}  // extern "C"
