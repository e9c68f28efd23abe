// Amplitude gather that allocates no memory.
//
// pq_gather_elements stages the caller's index list and the gathered values
// in device buffers it allocates for the call.  Some callers cannot allow
// that: hosts that own every device allocation themselves (a Julia process
// whose CUDA.jl pool must account for all device memory, an embedding
// application running under a fixed device-memory budget), or code that runs
// where allocation is not permitted.  pq_gather_elements_noalloc does the same
// work with its staging area in a fixed, file-scope device array instead.
//
// The array (kNoAllocMaxElems indices plus as many complex128 values, 1.5 MiB)
// is reserved on every device that loads this library, for as long as the
// process runs.  It is shared by all calls on a device: a call overwrites what
// the previous call left there, and calls that overlap on the GPU (two
// contexts on different streams of one device at the same time) race on it.
#include <cuda_runtime.h>

#include <mutex>

#include "pq_types.cuh"

namespace pq {
int check_status(Ctx* ctx);
}
using namespace pq;

namespace {

constexpr int64_t kNoAllocMaxElems = 65536;
constexpr size_t kIdxBytes = (size_t)kNoAllocMaxElems * sizeof(int64_t);
constexpr size_t kValBytes = (size_t)kNoAllocMaxElems * 16;

// Staging area: [indices (int64) | gathered values (complex64 or complex128)].
static __device__ __align__(256) unsigned char g_noalloc_scratch[kIdxBytes + kValBytes];

constexpr int kMaxDevices = 64;
std::mutex g_lock;
void* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of g_noalloc_scratch on `device` (which must be current),
// looked up once per device.  In host code the symbol itself is only a
// host-side stand-in, so kernels are always given this address.
cudaError_t scratch_for(int device, unsigned char** out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> g(g_lock);
  if (!g_scratch_ptr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[device] = p;
  }
  *out = (unsigned char*)g_scratch_ptr[device];
  return cudaSuccess;
}

template <typename TI, typename TO>
__global__ void k_gather_cvt(const TI* __restrict__ in, const int64_t* __restrict__ idx, int64_t n,
                             TO* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = store_as<TO>(in[idx[i]]);
}

}  // namespace

extern "C" {

int pq_gather_elements_noalloc(pq_ctx* c, int64_t id, const int64_t* idx, int64_t n, void* out, int dtype) {
  if (!c) return PQ_ERR_INVALID;
  Ctx* ctx = &c->impl;
  auto it = ctx->tensors.find(id);
  if (it == ctx->tensors.end())
    return fail(ctx, PQ_ERR_NOT_FOUND, "gather_elements_noalloc: no tensor " + std::to_string(id));
  if (n < 0 || (n && (!idx || !out))) return fail(ctx, PQ_ERR_INVALID, "gather_elements_noalloc: bad arguments");
  if (n > kNoAllocMaxElems)
    return fail(ctx, PQ_ERR_INVALID,
                "gather_elements_noalloc: " + std::to_string(n) + " indices exceed the static staging limit of " +
                    std::to_string(kNoAllocMaxElems) + "; use pq_gather_elements or split the request");
  if (dtype != PQ_C64 && dtype != PQ_C128) return fail(ctx, PQ_ERR_INVALID, "gather_elements_noalloc: bad dtype");
  const Tensor& T = it->second;
  for (int64_t i = 0; i < n; ++i)
    if (idx[i] < 0 || idx[i] >= T.size)
      return fail(ctx, PQ_ERR_INVALID, "gather_elements_noalloc: index out of range");
  if (n == 0) return PQ_OK;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gather_elements_noalloc: set device");
  unsigned char* scratch = nullptr;
  e = scratch_for(ctx->device, &scratch);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gather_elements_noalloc: cudaGetSymbolAddress");
  int64_t* d_idx = (int64_t*)scratch;
  void* d_val = scratch + kIdxBytes;
  e = cudaMemcpyAsync(d_idx, idx, (size_t)n * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) {
    const int grid = (int)((n + 255) / 256);
    if (T.dtype == PQ_C128 && dtype == PQ_C128)
      k_gather_cvt<double2, double2><<<grid, 256, 0, ctx->stream>>>((const double2*)T.ptr, d_idx, n, (double2*)d_val);
    else if (T.dtype == PQ_C128)
      k_gather_cvt<double2, float2><<<grid, 256, 0, ctx->stream>>>((const double2*)T.ptr, d_idx, n, (float2*)d_val);
    else if (dtype == PQ_C128)
      k_gather_cvt<float2, double2><<<grid, 256, 0, ctx->stream>>>((const float2*)T.ptr, d_idx, n, (double2*)d_val);
    else
      k_gather_cvt<float2, float2><<<grid, 256, 0, ctx->stream>>>((const float2*)T.ptr, d_idx, n, (float2*)d_val);
    e = cudaGetLastError();
    ctx->launches += 1;
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, d_val, (size_t)n * elem_bytes(dtype), cudaMemcpyDeviceToHost, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gather_elements_noalloc");
  return check_status(ctx);
}

}  // extern "C"
