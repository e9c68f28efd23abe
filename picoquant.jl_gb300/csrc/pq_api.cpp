// C ABI: context, tensor table and the backend tensor operations.
//
// Mirrors the method table of the reference's InteractiveBackend
// (src/backends/interactive.jl:10-172) with device-resident tensors.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "pq_internal.h"

namespace pq {

int fail(Ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
  return code;
}

int cuda_fail(Ctx* ctx, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  if (e == cudaErrorMemoryAllocation) return fail(ctx, PQ_ERR_OOM, m);
  return fail(ctx, PQ_ERR_CUDA, m);
}

int dev_alloc(Ctx* ctx, size_t bytes, void** p) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  if (ctx->mem_cap > 0 && ctx->mem_in_use + (int64_t)bytes > ctx->mem_cap)
    return fail(ctx, PQ_ERR_OOM,
                "device memory cap exceeded: requested " + std::to_string(bytes) + " bytes with " +
                    std::to_string(ctx->mem_in_use) + " of " + std::to_string(ctx->mem_cap) + " in use");
  cudaError_t e = cudaMallocFromPoolAsync(p, bytes, ctx->pool, ctx->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return cuda_fail(ctx, e, "cudaMallocFromPoolAsync");
  }
  ctx->mem_in_use += (int64_t)bytes;
  return PQ_OK;
}

void dev_free(Ctx* ctx, void* p, size_t bytes) {
  if (!p) return;
  if (bytes == 0) bytes = 16;
  cudaFreeAsync(p, ctx->stream);
  ctx->mem_in_use -= (int64_t)bytes;
}

static int64_t prod(const std::vector<int64_t>& d) {
  int64_t p = 1;
  for (auto x : d) p *= x;
  return p;
}

static void free_tensor(Ctx* ctx, Tensor& t) {
  dev_free(ctx, t.ptr, t.bytes);
  t.ptr = nullptr;
}

// Replace (or insert) a tensor entry, freeing the previous storage.
static void put_entry(Ctx* ctx, int64_t id, Tensor&& t) {
  auto it = ctx->tensors.find(id);
  if (it != ctx->tensors.end()) {
    if (it->second.ptr != t.ptr) free_tensor(ctx, it->second);
    it->second = std::move(t);
  } else {
    ctx->tensors.emplace(id, std::move(t));
  }
}

int alloc_tensor(Ctx* ctx, const std::vector<int64_t>& dims, int dtype, Tensor& t) {
  t.dims = dims;
  t.size = prod(dims);
  t.dtype = dtype;
  t.bytes = (size_t)t.size * elem_bytes(dtype);
  return dev_alloc(ctx, t.bytes, &t.ptr);
}

// Convert n complex elements between host representations.
static void convert_host(const void* src, int sdt, void* dst, int ddt, int64_t n) {
  if (sdt == ddt) {
    std::memcpy(dst, src, (size_t)n * elem_bytes(sdt));
  } else if (sdt == PQ_C128) {
    const double* s = (const double*)src;
    float* o = (float*)dst;
    for (int64_t i = 0; i < 2 * n; ++i) o[i] = (float)s[i];
  } else {
    const float* s = (const float*)src;
    double* o = (double*)dst;
    for (int64_t i = 0; i < 2 * n; ++i) o[i] = (double)s[i];
  }
}

int check_status(Ctx* ctx) {
  int h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "stream synchronize");
  if (h != 0) {
    cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream);
    return fail(ctx, PQ_ERR_DEVICE, "a kernel reported device status " + std::to_string(h));
  }
  return PQ_OK;
}

}  // namespace pq

using namespace pq;

#define CTX_OR_FAIL(c)              \
  if (!(c)) return PQ_ERR_INVALID; \
  Ctx* ctx = &(c)->impl;

extern "C" {

int pq_ctx_create(int device, int precision, pq_ctx** out) {
  if (!out) return PQ_ERR_INVALID;
  *out = nullptr;
  if (precision < PQ_PREC_C128 || precision > PQ_PREC_OZAKI4) return PQ_ERR_INVALID;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return PQ_ERR_CUDA;
  pq_ctx* c = new pq_ctx();
  Ctx* ctx = &c->impl;
  ctx->device = device;
  ctx->precision = precision;
  e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return PQ_ERR_CUDA;
  }
  // A private stream-ordered pool that keeps freed blocks for reuse.
  cudaMemPoolProps props;
  std::memset(&props, 0, sizeof(props));
  props.allocType = cudaMemAllocationTypePinned;
  props.handleTypes = cudaMemHandleTypeNone;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  e = cudaMemPoolCreate(&ctx->pool, &props);
  if (e != cudaSuccess) {
    cudaStreamDestroy(ctx->stream);
    delete c;
    return PQ_ERR_CUDA;
  }
  uint64_t thr = UINT64_MAX;
  cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &thr);
  e = cudaMalloc((void**)&ctx->d_status, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(ctx->d_status, 0, sizeof(int));
  if (e != cudaSuccess) {
    cudaMemPoolDestroy(ctx->pool);
    cudaStreamDestroy(ctx->stream);
    delete c;
    return PQ_ERR_CUDA;
  }
  *out = c;
  return PQ_OK;
}

int pq_ctx_destroy(pq_ctx* c) {
  if (!c) return PQ_ERR_INVALID;
  Ctx* ctx = &c->impl;
  cudaSetDevice(ctx->device);
  for (auto& kv : ctx->tensors) free_tensor(ctx, kv.second);
  ctx->tensors.clear();
  if (ctx->d_stage) dev_free(ctx, ctx->d_stage, ctx->d_stage_cap);
  cudaStreamSynchronize(ctx->stream);
  if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
  if (ctx->stage_done) cudaEventDestroy(ctx->stage_done);
  cudaFree(ctx->d_status);
  cudaMemPoolDestroy(ctx->pool);
  cudaStreamDestroy(ctx->stream);
  delete c;
  return PQ_OK;
}

const char* pq_last_error(pq_ctx* c) {
  if (!c) return "null context";
  return c->impl.last_error.c_str();
}

int pq_ctx_precision(pq_ctx* c) {
  CTX_OR_FAIL(c);
  return ctx->precision;
}

int pq_ctx_sync(pq_ctx* c) {
  CTX_OR_FAIL(c);
  return check_status(ctx);
}

int pq_ctx_set_mem_cap(pq_ctx* c, int64_t bytes) {
  CTX_OR_FAIL(c);
  ctx->mem_cap = bytes < 0 ? 0 : bytes;
  return PQ_OK;
}

int pq_ctx_mem_in_use(pq_ctx* c, int64_t* bytes) {
  CTX_OR_FAIL(c);
  if (bytes) *bytes = ctx->mem_in_use;
  return PQ_OK;
}

int pq_ctx_launch_count(pq_ctx* c, int64_t* count) {
  CTX_OR_FAIL(c);
  if (count) *count = ctx->launches;
  return PQ_OK;
}

int pq_ctx_stream(pq_ctx* c, void** stream) {
  CTX_OR_FAIL(c);
  if (stream) *stream = (void*)ctx->stream;
  return PQ_OK;
}

int pq_save_tensor_data(pq_ctx* c, int64_t id, int rank, const int64_t* dims, const void* data, int dtype) {
  CTX_OR_FAIL(c);
  if (rank < 0 || rank > PQ_MAX_RANK || (rank > 0 && !dims) || !data)
    return fail(ctx, PQ_ERR_INVALID, "save_tensor_data: bad rank/dims/data");
  if (dtype != PQ_C64 && dtype != PQ_C128) return fail(ctx, PQ_ERR_INVALID, "save_tensor_data: bad dtype");
  std::vector<int64_t> d(dims, dims + rank);
  for (auto x : d)
    if (x < 1) return fail(ctx, PQ_ERR_INVALID, "save_tensor_data: extents must be >= 1");
  Tensor t;
  int st = alloc_tensor(ctx, d, storage_dtype(ctx, prod(d)), t);
  if (st) return st;
  cudaError_t e;
  if (t.dtype == dtype) {
    e = cudaMemcpyAsync(t.ptr, data, t.bytes, cudaMemcpyHostToDevice, ctx->stream);
  } else {
    // convert on the host (large states should be uploaded in the storage type)
    std::vector<unsigned char> tmp(t.bytes);
    convert_host(data, dtype, tmp.data(), t.dtype, t.size);
    e = cudaMemcpyAsync(t.ptr, tmp.data(), t.bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  }
  if (e != cudaSuccess) {
    free_tensor(ctx, t);
    return cuda_fail(ctx, e, "save_tensor_data upload");
  }
  put_entry(ctx, id, std::move(t));
  return PQ_OK;
}

int pq_save_tensors(pq_ctx* c, int n, const int64_t* ids, const int32_t* ranks, const int64_t* dims_flat,
                    const void* const* data, const int32_t* dtypes) {
  CTX_OR_FAIL(c);
  if (n < 0 || (n > 0 && (!ids || !ranks || !data || !dtypes)))
    return fail(ctx, PQ_ERR_INVALID, "save_tensors: bad arguments");
  if (n == 0) return PQ_OK;
  // validate and lay out: data in the storage type, each at a 16-byte offset,
  // then the copy table
  std::vector<std::vector<int64_t>> dims(n);
  std::vector<int> sdt(n);
  std::vector<size_t> off(n), bytes(n);
  size_t pos = 0, dpos = 0;
  for (int i = 0; i < n; ++i) {
    if (ranks[i] < 0 || ranks[i] > PQ_MAX_RANK || !data[i] || (ranks[i] > 0 && !dims_flat))
      return fail(ctx, PQ_ERR_INVALID, "save_tensors: bad rank/data of tensor " + std::to_string(i));
    if (dtypes[i] != PQ_C64 && dtypes[i] != PQ_C128)
      return fail(ctx, PQ_ERR_INVALID, "save_tensors: bad dtype of tensor " + std::to_string(i));
    dims[i].assign(dims_flat + dpos, dims_flat + dpos + ranks[i]);
    dpos += ranks[i];
    for (auto x : dims[i])
      if (x < 1) return fail(ctx, PQ_ERR_INVALID, "save_tensors: extents must be >= 1");
    const int64_t size = prod(dims[i]);
    sdt[i] = storage_dtype(ctx, size);
    bytes[i] = (size_t)size * elem_bytes(sdt[i]);
    off[i] = pos;
    pos += (bytes[i] + 15) & ~(size_t)15;
  }
  {
    std::vector<int64_t> sorted_ids(ids, ids + n);
    std::sort(sorted_ids.begin(), sorted_ids.end());
    if (std::adjacent_find(sorted_ids.begin(), sorted_ids.end()) != sorted_ids.end())
      return fail(ctx, PQ_ERR_INVALID, "save_tensors: an id appears twice in one batch");
  }
  const size_t table_off = pos;
  const size_t total = table_off + (size_t)n * sizeof(CopyJob);
  cudaError_t e = cudaSuccess;
  if (ctx->stage_done) {
    e = cudaEventSynchronize(ctx->stage_done);  // the previous batch has left the host buffer
    if (e != cudaSuccess) return cuda_fail(ctx, e, "save_tensors wait");
  } else if ((e = cudaEventCreateWithFlags(&ctx->stage_done, cudaEventDisableTiming)) != cudaSuccess) {
    return cuda_fail(ctx, e, "save_tensors event");
  }
  if (total > ctx->h_stage_cap) {
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    ctx->h_stage = nullptr;
    ctx->h_stage_cap = 0;
    const size_t cap = total + total / 2;
    if ((e = cudaHostAlloc(&ctx->h_stage, cap, cudaHostAllocDefault)) != cudaSuccess)
      return cuda_fail(ctx, e, "save_tensors pinned staging");
    ctx->h_stage_cap = cap;
  }
  if (total > ctx->d_stage_cap) {
    if (ctx->d_stage) dev_free(ctx, ctx->d_stage, ctx->d_stage_cap);
    ctx->d_stage = nullptr;
    ctx->d_stage_cap = 0;
    const size_t cap = total + total / 2;
    int st = dev_alloc(ctx, cap, &ctx->d_stage);
    if (st) return st;
    ctx->d_stage_cap = cap;
  }
  unsigned char* h = (unsigned char*)ctx->h_stage;
  CopyJob* jobs = (CopyJob*)(h + table_off);
  for (int i = 0; i < n; ++i) {
    const int64_t size = prod(dims[i]);
    if (dtypes[i] == sdt[i])
      std::memcpy(h + off[i], data[i], bytes[i]);
    else
      convert_host(data[i], dtypes[i], h + off[i], sdt[i], size);
    // a tensor replaced by one of the same extents and type keeps its storage
    auto it = ctx->tensors.find(ids[i]);
    if (it != ctx->tensors.end() && it->second.dims == dims[i] && it->second.dtype == sdt[i] && it->second.ptr) {
      jobs[i] = CopyJob{(int64_t)off[i], it->second.ptr, (int64_t)bytes[i]};
      continue;
    }
    Tensor t;
    int st = alloc_tensor(ctx, dims[i], sdt[i], t);
    if (st) return st;
    jobs[i] = CopyJob{(int64_t)off[i], t.ptr, (int64_t)bytes[i]};
    put_entry(ctx, ids[i], std::move(t));
  }
  e = cudaMemcpyAsync(ctx->d_stage, h, total, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaEventRecord(ctx->stage_done, ctx->stream);
  if (e == cudaSuccess)
    e = launch_scatter(ctx->d_stage, (const CopyJob*)((unsigned char*)ctx->d_stage + table_off), n, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "save_tensors upload");
  ctx->launches += 1;
  return PQ_OK;
}

int pq_load_tensor_data(pq_ctx* c, int64_t id, void* dst, int64_t n_elems, int dtype) {
  CTX_OR_FAIL(c);
  auto it = ctx->tensors.find(id);
  if (it == ctx->tensors.end()) return fail(ctx, PQ_ERR_NOT_FOUND, "load_tensor_data: no tensor " + std::to_string(id));
  const Tensor& t = it->second;
  if (!dst || n_elems < t.size) return fail(ctx, PQ_ERR_INVALID, "load_tensor_data: destination too small");
  if (dtype != PQ_C64 && dtype != PQ_C128) return fail(ctx, PQ_ERR_INVALID, "load_tensor_data: bad dtype");
  cudaError_t e;
  if (t.dtype == dtype) {
    e = cudaMemcpyAsync(dst, t.ptr, t.bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "load_tensor_data download");
    return check_status(ctx);
  }
  std::vector<unsigned char> tmp(t.bytes);
  e = cudaMemcpyAsync(tmp.data(), t.ptr, t.bytes, cudaMemcpyDeviceToHost, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "load_tensor_data download");
  int st = check_status(ctx);
  if (st) return st;
  convert_host(tmp.data(), t.dtype, dst, dtype, t.size);
  return PQ_OK;
}

int pq_tensor_shape(pq_ctx* c, int64_t id, int* rank, int64_t* dims) {
  CTX_OR_FAIL(c);
  auto it = ctx->tensors.find(id);
  if (it == ctx->tensors.end()) return fail(ctx, PQ_ERR_NOT_FOUND, "tensor_shape: no tensor " + std::to_string(id));
  if (rank) *rank = (int)it->second.dims.size();
  if (dims)
    for (size_t i = 0; i < it->second.dims.size(); ++i) dims[i] = it->second.dims[i];
  return PQ_OK;
}

int pq_has_tensor(pq_ctx* c, int64_t id) {
  if (!c) return 0;
  return c->impl.tensors.count(id) ? 1 : 0;
}

int pq_delete_tensor(pq_ctx* c, int64_t id) {
  CTX_OR_FAIL(c);
  auto it = ctx->tensors.find(id);
  if (it == ctx->tensors.end()) return PQ_OK;  // deleting a missing tensor is a no-op
  free_tensor(ctx, it->second);
  ctx->tensors.erase(it);
  return PQ_OK;
}

int pq_tensor_norm2(pq_ctx* c, int64_t id, double* norm2) {
  CTX_OR_FAIL(c);
  if (!norm2) return fail(ctx, PQ_ERR_INVALID, "tensor_norm2: null output");
  auto it = ctx->tensors.find(id);
  if (it == ctx->tensors.end()) return fail(ctx, PQ_ERR_NOT_FOUND, "tensor_norm2: no tensor " + std::to_string(id));
  const Tensor& T = it->second;
  const int nb = norm2_blocks(T.size);
  const size_t bytes = (size_t)(2 * nb + 1) * sizeof(double);
  double* d = nullptr;
  int st = dev_alloc(ctx, bytes, (void**)&d);
  if (st) return st;
  cudaError_t e = launch_norm2(T.dtype, T.ptr, T.size, d, d + 2 * nb, ctx->stream);
  ctx->launches += 2;
  if (e == cudaSuccess) e = cudaMemcpyAsync(norm2, d + 2 * nb, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  dev_free(ctx, d, bytes);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "tensor_norm2");
  return check_status(ctx);  // also completes the copy
}

int pq_save_output(pq_ctx* c, int64_t node, int64_t name) {
  CTX_OR_FAIL(c);
  auto it = ctx->tensors.find(node);
  if (it == ctx->tensors.end()) return fail(ctx, PQ_ERR_NOT_FOUND, "save_output: no tensor " + std::to_string(node));
  if (node == name) return PQ_OK;
  Tensor t;
  int st = alloc_tensor(ctx, it->second.dims, it->second.dtype, t);
  if (st) return st;
  cudaError_t e = cudaMemcpyAsync(t.ptr, it->second.ptr, t.bytes, cudaMemcpyDeviceToDevice, ctx->stream);
  if (e != cudaSuccess) {
    free_tensor(ctx, t);
    return cuda_fail(ctx, e, "save_output copy");
  }
  put_entry(ctx, name, std::move(t));
  return PQ_OK;
}

int pq_contract_tensors(pq_ctx* c, int64_t a, const int32_t* a_labels, int a_rank, int64_t b,
                        const int32_t* b_labels, int b_rank, int64_t cid) {
  CTX_OR_FAIL(c);
  auto ia = ctx->tensors.find(a), ib = ctx->tensors.find(b);
  if (ia == ctx->tensors.end()) return fail(ctx, PQ_ERR_NOT_FOUND, "contract_tensors: no tensor " + std::to_string(a));
  if (ib == ctx->tensors.end()) return fail(ctx, PQ_ERR_NOT_FOUND, "contract_tensors: no tensor " + std::to_string(b));
  if (a == b) return fail(ctx, PQ_ERR_INVALID, "contract_tensors: A and B are the same tensor");
  Tensor& A = ia->second;
  Tensor& B = ib->second;
  if ((int)A.dims.size() != a_rank || (int)B.dims.size() != b_rank || (a_rank && !a_labels) ||
      (b_rank && !b_labels))
    return fail(ctx, PQ_ERR_INVALID, "contract_tensors: label count does not match tensor rank");
  std::vector<int> la(a_labels, a_labels + a_rank), lb(b_labels, b_labels + b_rank);
  std::vector<int> lc = symdiff_labels(la, lb);
  PairPlan pp;
  std::string err;
  if (!analyse_pair(la, A.dims, lb, B.dims, lc, ctx->precision, pp, err, &ctx->tuning))
    return fail(ctx, PQ_ERR_INVALID, "contract_tensors: " + err);
  Tensor C;
  int st = alloc_tensor(ctx, pp.c_dims, storage_dtype(ctx, pp.csize), C);
  if (st) return st;
  cudaError_t e;
  void* scratch = nullptr;
  size_t sbytes = 0;
  if (pp.kclass == KC_TC) {
    sbytes = tc_scratch_bytes(ctx->precision, pp.m);
    st = dev_alloc(ctx, sbytes, &scratch);
    if (st) {
      free_tensor(ctx, C);
      return st;
    }
    e = launch_tc(ctx->precision, A.dtype, B.dtype, C.dtype, A.ptr, B.ptr, C.ptr, pp.m, scratch, sbytes,
                  ctx->d_status, ctx->stream);
    ctx->launches += tc_launch_count(ctx->precision, pp.m);
  } else if (pp.kclass == KC_GEMM) {
    e = launch_gemm(A.dtype, B.dtype, C.dtype, A.ptr, B.ptr, C.ptr, pp.m, ctx->stream);
    ctx->launches += 1;
  } else if (pp.kclass == KC_SKINNY) {
    e = launch_skinny(A.dtype, B.dtype, C.dtype, A.ptr, B.ptr, C.ptr, pp.m, ctx->stream);
    ctx->launches += 1;
  } else {
    e = launch_generic(A.dtype, B.dtype, C.dtype, A.ptr, B.ptr, C.ptr, pp.g, ctx->stream);
    ctx->launches += 1;
  }
  if (scratch) dev_free(ctx, scratch, sbytes);
  if (e != cudaSuccess) {
    free_tensor(ctx, C);
    return cuda_fail(ctx, e, "contract_tensors launch");
  }
  // A and B are consumed (src/backends/interactive.jl:73-74)
  free_tensor(ctx, A);
  free_tensor(ctx, B);
  ctx->tensors.erase(a);
  ctx->tensors.erase(b);
  put_entry(ctx, cid, std::move(C));
  return PQ_OK;
}

int pq_permute_tensor(pq_ctx* c, int64_t id, const int32_t* perm1, int rank) {
  CTX_OR_FAIL(c);
  auto it = ctx->tensors.find(id);
  if (it == ctx->tensors.end()) return fail(ctx, PQ_ERR_NOT_FOUND, "permute_tensor: no tensor " + std::to_string(id));
  Tensor& T = it->second;
  if ((int)T.dims.size() != rank || (rank && !perm1))
    return fail(ctx, PQ_ERR_INVALID, "permute_tensor: permutation length does not match rank");
  std::vector<int> seen(rank, 0);
  for (int i = 0; i < rank; ++i) {
    int p = perm1[i] - 1;
    if (p < 0 || p >= rank || seen[p]) return fail(ctx, PQ_ERR_INVALID, "permute_tensor: not a permutation");
    seen[p] = 1;
  }
  // a permutation is a contraction with nothing: result label i = input label perm[i]
  std::vector<int> la(rank), lc(rank);
  for (int i = 0; i < rank; ++i) la[i] = i;
  for (int i = 0; i < rank; ++i) lc[i] = perm1[i] - 1;
  PairPlan pp;
  std::string err;
  if (!analyse_pair(la, T.dims, {}, {}, lc, ctx->precision, pp, err))
    return fail(ctx, PQ_ERR_INVALID, "permute_tensor: " + err);
  Tensor O;
  int st = alloc_tensor(ctx, pp.c_dims, T.dtype, O);
  if (st) return st;
  cudaError_t e = launch_permute(T.dtype, O.dtype, T.ptr, 0, O.ptr, pp.g, ctx->stream);
  ctx->launches += 1;
  if (e != cudaSuccess) {
    free_tensor(ctx, O);
    return cuda_fail(ctx, e, "permute launch");
  }
  put_entry(ctx, id, std::move(O));
  return PQ_OK;
}

int pq_reshape_tensor(pq_ctx* c, int64_t id, int n_groups, const int32_t* group_sizes, const int32_t* axes1) {
  CTX_OR_FAIL(c);
  auto it = ctx->tensors.find(id);
  if (it == ctx->tensors.end()) return fail(ctx, PQ_ERR_NOT_FOUND, "reshape_tensor: no tensor " + std::to_string(id));
  Tensor& T = it->second;
  if (n_groups < 0 || n_groups > PQ_MAX_RANK || (n_groups && (!group_sizes || !axes1)))
    return fail(ctx, PQ_ERR_INVALID, "reshape_tensor: bad groups");
  std::vector<int64_t> nd;
  int pos = 0;
  const int r = (int)T.dims.size();
  for (int g = 0; g < n_groups; ++g) {
    int64_t p = 1;
    for (int j = 0; j < group_sizes[g]; ++j) {
      int ax = axes1[pos++] - 1;
      if (ax < 0 || ax >= r) return fail(ctx, PQ_ERR_INVALID, "reshape_tensor: axis out of range");
      p *= T.dims[ax];
    }
    nd.push_back(p);
  }
  if (prod(nd) != T.size) return fail(ctx, PQ_ERR_INVALID, "reshape_tensor: size changes");
  T.dims = nd;
  return PQ_OK;
}

int pq_decompose_tensor(pq_ctx* c, int64_t id, int n_left, const int32_t* left1, int n_right, const int32_t* right1,
                        double threshold, int max_rank, int64_t left_id, int64_t right_id, int* chi_out,
                        int* sweeps_out) {
  CTX_OR_FAIL(c);
  auto it = ctx->tensors.find(id);
  if (it == ctx->tensors.end()) return fail(ctx, PQ_ERR_NOT_FOUND, "decompose_tensor: no tensor " + std::to_string(id));
  const Tensor& T = it->second;
  const int rank = (int)T.dims.size();
  if (n_left < 0 || n_right < 0 || n_left + n_right != rank || (n_left && !left1) || (n_right && !right1) ||
      !chi_out || left_id == right_id || left_id == id || right_id == id || max_rank < 0)
    return fail(ctx, PQ_ERR_INVALID, "decompose_tensor: bad arguments");
  std::vector<int> seen(rank, 0), perm(rank);
  std::vector<int64_t> ld, rd;
  int64_t m = 1, n = 1;
  for (int i = 0; i < rank; ++i) {
    const int p = (i < n_left ? left1[i] : right1[i - n_left]) - 1;
    if (p < 0 || p >= rank || seen[p]) return fail(ctx, PQ_ERR_INVALID, "decompose_tensor: positions not a permutation");
    seen[p] = 1;
    perm[i] = p;
    (i < n_left ? ld : rd).push_back(T.dims[p]);
    (i < n_left ? m : n) *= T.dims[p];
  }
  const int64_t R = m < n ? n : m;
  const int64_t Cn = m < n ? m : n;
  if (Cn > 256 || R * Cn > (int64_t(1) << 24))
    return fail(ctx, PQ_ERR_UNSUPPORTED, "decompose_tensor: the device SVD takes at most 256 columns and 2^24 "
                                         "elements (the smaller side of the split is " + std::to_string(Cn) + ")");
  // arithmetic of the context's element type, as LAPACK's for the reference
  // backend's T: complex FP64 in complex128 contexts, complex FP32 otherwise
  const int wt = ctx->precision == PQ_PREC_C128 ? PQ_C128 : PQ_C64;
  const size_t csz = wt == PQ_C128 ? 16 : 8, rsz = csz / 2;
  // the matrix A (m x n, column-major): the tensor permuted to (left..., right...)
  std::vector<int> la(rank), lc(rank);
  for (int i = 0; i < rank; ++i) la[i] = i;
  for (int i = 0; i < rank; ++i) lc[i] = perm[i];
  PairPlan pp;
  std::string err;
  if (!analyse_pair(la, T.dims, {}, {}, lc, ctx->precision, pp, err))
    return fail(ctx, PQ_ERR_INVALID, "decompose_tensor: " + err);
  // scratch: [A | W | V | sig | order | sweeps], each piece 16-byte aligned
  auto up16 = [](size_t b) { return (b + 15) & ~(size_t)15; };
  const size_t b_mat = up16((size_t)(m * n) * csz), b_v = up16((size_t)(Cn * Cn) * csz),
               b_sig = up16((size_t)Cn * rsz), b_ord = up16((size_t)Cn * sizeof(int) + sizeof(int));
  const size_t scratch = 2 * b_mat + b_v + b_sig + b_ord;
  char* d = nullptr;
  int st = dev_alloc(ctx, scratch, (void**)&d);
  if (st) return st;
  void* A = d;
  void* W = d + b_mat;
  void* V = d + 2 * b_mat;
  void* sig = d + 2 * b_mat + b_v;
  int* order = (int*)(d + 2 * b_mat + b_v + b_sig);
  int* sweeps = order + Cn;
  cudaError_t e = launch_permute(T.dtype, wt, T.ptr, 0, A, pp.g, ctx->stream);
  ctx->launches += 1;
  if (e == cudaSuccess) {
    e = launch_jacobi_svd(wt, A, m, n, W, V, sig, 60, wt == PQ_C128 ? 1e-14 : 1e-6, sweeps, ctx->stream);
    ctx->launches += 1;
  }
  std::vector<double> hs((size_t)Cn);
  std::vector<float> hsf(wt == PQ_C128 ? 0 : (size_t)Cn);
  if (e == cudaSuccess && Cn)
    e = cudaMemcpyAsync(wt == PQ_C128 ? (void*)hs.data() : (void*)hsf.data(), sig, (size_t)Cn * rsz,
                        cudaMemcpyDeviceToHost, ctx->stream);
  int h_sweeps = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&h_sweeps, sweeps, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
  if (e != cudaSuccess) {
    dev_free(ctx, d, scratch);
    return cuda_fail(ctx, e, "decompose_tensor: device SVD");
  }
  st = check_status(ctx);
  if (st) {
    dev_free(ctx, d, scratch);
    return st;
  }
  for (size_t i = 0; i < hsf.size(); ++i) hs[i] = hsf[i];
  // the reference's truncation (src/layer1.jl:166-176): singular values above
  // max(threshold, sqrt(eps)) of their 2-norm, at most max_rank of them
  std::vector<int> idx((size_t)Cn);
  for (int i = 0; i < (int)Cn; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return hs[a] > hs[b]; });
  // eps of the element type (complex128 contexts: FP64; the mixed ones:
  // FP32, as the reference's ComplexF32 default)
  const double eps = ctx->precision == PQ_PREC_C128 ? 2.220446049250313e-16 : 1.1920928955078125e-07;
  const double thr = std::max(threshold, std::sqrt(eps));
  double norm2 = 0.0;
  for (double v : hs) norm2 += v * v;
  const double norm = std::sqrt(norm2);
  int chi = 0;
  if (norm > 0)
    for (int i = 0; i < (int)Cn; ++i)
      if (hs[idx[i]] / norm > thr) ++chi;
  if (max_rank > 0) chi = std::min(chi, max_rank);
  std::vector<int64_t> bdims = ld, cdims = {chi};
  bdims.push_back(chi);
  cdims.insert(cdims.end(), rd.begin(), rd.end());
  Tensor Bt, Ct;
  st = alloc_tensor(ctx, bdims, storage_dtype(ctx, m * chi), Bt);
  if (!st) {
    st = alloc_tensor(ctx, cdims, storage_dtype(ctx, n * chi), Ct);
    if (st) free_tensor(ctx, Bt);
  }
  if (!st) {
    if (chi > 0)
      e = cudaMemcpyAsync(order, idx.data(), (size_t)chi * sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
      e = launch_svd_factors(wt, W, V, sig, order, chi, m, n, Bt.dtype, Bt.ptr, Ct.dtype, Ct.ptr, ctx->stream);
    ctx->launches += 1;
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);  // idx (host) is read by the copy above
    if (e != cudaSuccess) {
      free_tensor(ctx, Bt);
      free_tensor(ctx, Ct);
      st = cuda_fail(ctx, e, "decompose_tensor: factors");
    }
  }
  dev_free(ctx, d, scratch);
  if (st) return st;
  auto old = ctx->tensors.find(id);
  free_tensor(ctx, old->second);
  ctx->tensors.erase(old);
  put_entry(ctx, left_id, std::move(Bt));
  put_entry(ctx, right_id, std::move(Ct));
  *chi_out = chi;
  if (sweeps_out) *sweeps_out = h_sweeps;
  return PQ_OK;
}

int pq_view_tensor(pq_ctx* c, int64_t view_id, int64_t node, int bond_idx1, int64_t lo1, int64_t hi1) {
  CTX_OR_FAIL(c);
  auto it = ctx->tensors.find(node);
  if (it == ctx->tensors.end()) return fail(ctx, PQ_ERR_NOT_FOUND, "view_tensor: no tensor " + std::to_string(node));
  Tensor& T = it->second;
  const int r = (int)T.dims.size();
  const int ax = bond_idx1 - 1;
  if (ax < 0 || ax >= r || lo1 < 1 || hi1 < lo1 || hi1 > T.dims[ax])
    return fail(ctx, PQ_ERR_INVALID, "view_tensor: bad bond index or range");
  std::vector<int64_t> vd = T.dims;
  vd[ax] = hi1 - lo1 + 1;
  // copy descriptor: narrowed extents, strides of the full tensor
  GenericDesc g;
  std::memset(&g, 0, sizeof(g));
  int64_t stride = 1, size = 1;
  g.pow2 = 0;
  for (int i = 0; i < r; ++i) {
    g.cdim[g.nc] = vd[i];
    g.csa[g.nc] = stride;
    g.csb[g.nc] = 0;
    g.clog[g.nc] = -1;
    stride *= T.dims[i];
    size *= vd[i];
    if (vd[i] > 1) ++g.nc;
  }
  g.csize = size;
  g.ksize = 1;
  int64_t base = (lo1 - 1);
  for (int i = 0; i < ax; ++i) base *= T.dims[i];
  Tensor O;
  int st = alloc_tensor(ctx, vd, T.dtype, O);
  if (st) return st;
  cudaError_t e = launch_permute(T.dtype, O.dtype, T.ptr, base, O.ptr, g, ctx->stream);
  ctx->launches += 1;
  if (e != cudaSuccess) {
    free_tensor(ctx, O);
    return cuda_fail(ctx, e, "view launch");
  }
  put_entry(ctx, view_id, std::move(O));
  return PQ_OK;
}

int pq_gather_elements(pq_ctx* c, int64_t id, const int64_t* idx, int64_t n, void* out, int dtype) {
  CTX_OR_FAIL(c);
  auto it = ctx->tensors.find(id);
  if (it == ctx->tensors.end()) return fail(ctx, PQ_ERR_NOT_FOUND, "gather_elements: no tensor " + std::to_string(id));
  if (n < 0 || (n && (!idx || !out))) return fail(ctx, PQ_ERR_INVALID, "gather_elements: bad arguments");
  if (dtype != PQ_C64 && dtype != PQ_C128) return fail(ctx, PQ_ERR_INVALID, "gather_elements: bad dtype");
  const Tensor& T = it->second;
  for (int64_t i = 0; i < n; ++i)
    if (idx[i] < 0 || idx[i] >= T.size) return fail(ctx, PQ_ERR_INVALID, "gather_elements: index out of range");
  if (n == 0) return PQ_OK;
  const size_t eb = elem_bytes(T.dtype);
  void* d_idx = nullptr;
  void* d_out = nullptr;
  int st = dev_alloc(ctx, (size_t)n * 8, &d_idx);
  if (st) return st;
  st = dev_alloc(ctx, (size_t)n * eb, &d_out);
  if (st) {
    dev_free(ctx, d_idx, (size_t)n * 8);
    return st;
  }
  cudaError_t e = cudaMemcpyAsync(d_idx, idx, (size_t)n * 8, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = launch_gather(T.dtype, T.ptr, (const int64_t*)d_idx, n, d_out, ctx->stream);
  ctx->launches += 1;
  std::vector<unsigned char> tmp((size_t)n * eb);
  if (e == cudaSuccess) e = cudaMemcpyAsync(tmp.data(), d_out, tmp.size(), cudaMemcpyDeviceToHost, ctx->stream);
  dev_free(ctx, d_idx, (size_t)n * 8);
  dev_free(ctx, d_out, (size_t)n * eb);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gather_elements");
  st = check_status(ctx);
  if (st) return st;
  convert_host(tmp.data(), T.dtype, out, dtype, n);
  return PQ_OK;
}

int pq_ctx_set_small_elems(pq_ctx* c, int64_t n) {
  CTX_OR_FAIL(c);
  if (n < 0) return fail(ctx, PQ_ERR_INVALID, "set_small_elems: negative threshold");
  ctx->small_elems = n;
  return PQ_OK;
}

}  // extern "C"
