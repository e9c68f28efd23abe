// SIMT kernels for sm_103a: the fused permute+contract kernel for
// memory-bound pairs, and data movement (permute/view, gather, slice gather,
// FP64 compensated slice sum).
//
// Every operand and the result carry their own storage type (complex64 or
// complex128).  Results stored as complex128 are accumulated in FP64; results
// stored as complex64 are accumulated in FP32 over chunks of kChunk terms that
// are folded with Kahan compensation.
#include <algorithm>

#include "pq_types.cuh"

namespace pq {

// Decode linear index `c` over the result modes into offsets in A and B.
template <bool POW2>
__device__ __forceinline__ void decode2(int64_t c, const GenericDesc& d, int64_t& oa, int64_t& ob) {
  oa = 0;
  ob = 0;
#pragma unroll 1
  for (int i = 0; i < d.nc; ++i) {
    int64_t r;
    if (POW2) {
      r = c & (d.cdim[i] - 1);
      c >>= d.clog[i];
    } else {
      int64_t q = c / d.cdim[i];
      r = c - q * d.cdim[i];
      c = q;
    }
    oa += r * d.csa[i];
    ob += r * d.csb[i];
  }
}

template <bool POW2>
__device__ __forceinline__ void decodek(int64_t k, const GenericDesc& d, int64_t& oa, int64_t& ob) {
  oa = 0;
  ob = 0;
#pragma unroll 1
  for (int i = 0; i < d.nk; ++i) {
    int64_t r;
    if (POW2) {
      r = k & (d.kdim[i] - 1);
      k >>= d.klog[i];
    } else {
      int64_t q = k / d.kdim[i];
      r = k - q * d.kdim[i];
      k = q;
    }
    oa += r * d.ksa[i];
    ob += r * d.ksb[i];
  }
}

constexpr int kGenThreads = 256;

// Sum over k of A[a + ka[k]] * B[b + kb[k]] for k in [0, kn), accumulated
// into `acc` (FP64) or into the compensated accumulator (FP32).
template <typename TA, typename TB>
__device__ __forceinline__ void dot_chunk(double2& acc, KahanC&, const TA* a, const TB* b, const int64_t* ka,
                                          const int64_t* kb, int kn) {
#pragma unroll 4
  for (int k = 0; k < kn; ++k) cfma(acc, cvt<double>(__ldg(a + ka[k])), cvt<double>(__ldg(b + kb[k])));
}
template <typename TA, typename TB>
__device__ __forceinline__ void dot_chunk(float2&, KahanC& ks, const TA* a, const TB* b, const int64_t* ka,
                                          const int64_t* kb, int kn) {
  int k = 0;
  for (; k + kChunk <= kn; k += kChunk) {
    float2 p = make_float2(0.f, 0.f);
#pragma unroll
    for (int j = 0; j < kChunk; ++j) cfma(p, cvt<float>(__ldg(a + ka[k + j])), cvt<float>(__ldg(b + kb[k + j])));
    kahan_add(ks, p);
  }
  float2 p = make_float2(0.f, 0.f);
  for (; k < kn; ++k) cfma(p, cvt<float>(__ldg(a + ka[k])), cvt<float>(__ldg(b + kb[k])));
  kahan_add(ks, p);
}

__device__ __forceinline__ double2 acc_value(const double2& acc, const KahanC&) { return acc; }
__device__ __forceinline__ float2 acc_value(const float2&, const KahanC& ks) { return kahan_value(ks); }

template <typename TA, typename TB, typename TC, typename R, bool POW2>
__global__ void __launch_bounds__(kGenThreads)
    k_generic(const TA* __restrict__ A, const TB* __restrict__ B, TC* __restrict__ C,
              const __grid_constant__ GenericDesc d) {
  __shared__ int64_t ka[kGenericKTab];
  __shared__ int64_t kb[kGenericKTab];
  using AC = typename Acc<R>::C;
  const int64_t K = d.ksize;
  const int KT = (int)(K < kGenericKTab ? K : kGenericKTab);
  const bool one_chunk = K <= kGenericKTab;
  if (one_chunk) {
    for (int k = threadIdx.x; k < KT; k += blockDim.x) {
      int64_t x, y;
      decodek<POW2>(k, d, x, y);
      ka[k] = x;
      kb[k] = y;
    }
    __syncthreads();
  }
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < d.csize; base += step) {
    const int64_t c = base + threadIdx.x;
    const bool active = c < d.csize;
    int64_t oa = 0, ob = 0;
    if (active) decode2<POW2>(c, d, oa, ob);
    AC acc = czero(R());
    KahanC ks;
    kahan_init(ks);
    if (one_chunk) {
      if (active) dot_chunk(acc, ks, A + oa, B + ob, ka, kb, KT);
    } else {
      for (int64_t k0 = 0; k0 < K; k0 += KT) {
        const int kn = (int)((K - k0) < KT ? (K - k0) : KT);
        __syncthreads();
        for (int k = threadIdx.x; k < kn; k += blockDim.x) {
          int64_t x, y;
          decodek<POW2>(k0 + k, d, x, y);
          ka[k] = x;
          kb[k] = y;
        }
        __syncthreads();
        if (active) dot_chunk(acc, ks, A + oa, B + ob, ka, kb, kn);
      }
    }
    if (active) C[c] = store_as<TC>(acc_value(acc, ks));
  }
}

template <typename TA, typename TB, typename TC>
static void gen_launch(const void* A, const void* B, void* C, const GenericDesc& d, cudaStream_t s) {
  const int grid = grid_for(d.csize, kGenThreads);
  using R = typename std::conditional<std::is_same<TC, double2>::value, double, float>::type;
  if (d.pow2)
    k_generic<TA, TB, TC, R, true><<<grid, kGenThreads, 0, s>>>((const TA*)A, (const TB*)B, (TC*)C, d);
  else
    k_generic<TA, TB, TC, R, false><<<grid, kGenThreads, 0, s>>>((const TA*)A, (const TB*)B, (TC*)C, d);
}

template <typename TA, typename TB>
static void gen_launch_c(int tc, const void* A, const void* B, void* C, const GenericDesc& d, cudaStream_t s) {
  if (tc == PQ_C128)
    gen_launch<TA, TB, double2>(A, B, C, d, s);
  else
    gen_launch<TA, TB, float2>(A, B, C, d, s);
}

cudaError_t launch_generic(int ta, int tb, int tc, const void* A, const void* B, void* C, const GenericDesc& d,
                           cudaStream_t stream) {
  if (d.csize == 0) return cudaSuccess;
  if (ta == PQ_C128 && tb == PQ_C128)
    gen_launch_c<double2, double2>(tc, A, B, C, d, stream);
  else if (ta == PQ_C128)
    gen_launch_c<double2, float2>(tc, A, B, C, d, stream);
  else if (tb == PQ_C128)
    gen_launch_c<float2, double2>(tc, A, B, C, d, stream);
  else
    gen_launch_c<float2, float2>(tc, A, B, C, d, stream);
  return cudaGetLastError();
}

// Grouped small steps: one launch runs up to kGroupMax independent small
// contractions (complex128 operands and results, K <= kGroupK), each on its
// own range of blocks.  A block finds its member in the prefix table, copies
// the member's descriptor (prepared once per plan) into shared memory and
// runs the generic kernel's loop on it.
__global__ void __launch_bounds__(kGenThreads)
    k_generic_group(const __grid_constant__ GenericGroup g, const GenericDesc* __restrict__ descs) {
  __shared__ GenericDesc sd;
  __shared__ int64_t ka[kGroupK];
  __shared__ int64_t kb[kGroupK];
  int m = 0;
  while (m + 1 < g.n && g.blk[m + 1] <= (int)blockIdx.x) ++m;
  {
    const int* src = reinterpret_cast<const int*>(descs + g.desc[m]);
    int* dst = reinterpret_cast<int*>(&sd);
    for (int t = threadIdx.x; t < (int)(sizeof(GenericDesc) / sizeof(int)); t += blockDim.x) dst[t] = src[t];
  }
  __syncthreads();
  const int KT = (int)sd.ksize;
  for (int k = threadIdx.x; k < KT; k += blockDim.x) {
    int64_t x, y;
    if (sd.pow2)
      decodek<true>(k, sd, x, y);
    else
      decodek<false>(k, sd, x, y);
    ka[k] = x;
    kb[k] = y;
  }
  __syncthreads();
  const double2* A = static_cast<const double2*>(g.A[m]);
  const double2* B = static_cast<const double2*>(g.B[m]);
  double2* C = static_cast<double2*>(g.C[m]);
  const int64_t nb = g.blk[m + 1] - g.blk[m];
  const int64_t step = nb * blockDim.x;
  for (int64_t c = (int64_t)(blockIdx.x - g.blk[m]) * blockDim.x + threadIdx.x; c < sd.csize; c += step) {
    int64_t oa, ob;
    if (sd.pow2)
      decode2<true>(c, sd, oa, ob);
    else
      decode2<false>(c, sd, oa, ob);
    double2 acc = make_double2(0.0, 0.0);
    KahanC ks;
    dot_chunk(acc, ks, A + oa, B + ob, ka, kb, KT);
    C[c] = acc;
  }
}

cudaError_t launch_generic_group(const GenericGroup& g, const GenericDesc* d_descs, cudaStream_t stream) {
  if (g.n <= 0 || g.blk[g.n] <= 0) return cudaSuccess;
  k_generic_group<<<g.blk[g.n], kGenThreads, 0, stream>>>(g, d_descs);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Data movement
// ---------------------------------------------------------------------------
template <typename TI, typename TO, bool POW2>
__global__ void __launch_bounds__(kGenThreads)
    k_permute(const TI* __restrict__ in, int64_t base, TO* __restrict__ out, const __grid_constant__ GenericDesc d) {
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < d.csize; c += step) {
    int64_t oa, ob;
    decode2<POW2>(c, d, oa, ob);
    out[c] = store_as<TO>(in[base + oa]);
  }
}

template <typename TI, typename TO>
static void perm_launch(const void* in, int64_t base, void* out, const GenericDesc& d, cudaStream_t s) {
  const int grid = grid_for(d.csize, kGenThreads);
  if (d.pow2)
    k_permute<TI, TO, true><<<grid, kGenThreads, 0, s>>>((const TI*)in, base, (TO*)out, d);
  else
    k_permute<TI, TO, false><<<grid, kGenThreads, 0, s>>>((const TI*)in, base, (TO*)out, d);
}

cudaError_t launch_permute(int tin, int tout, const void* in, int64_t base, void* out, const GenericDesc& d,
                           cudaStream_t stream) {
  if (d.csize == 0) return cudaSuccess;
  if (tin == PQ_C128) {
    if (tout == PQ_C128)
      perm_launch<double2, double2>(in, base, out, d, stream);
    else
      perm_launch<double2, float2>(in, base, out, d, stream);
  } else {
    if (tout == PQ_C128)
      perm_launch<float2, double2>(in, base, out, d, stream);
    else
      perm_launch<float2, float2>(in, base, out, d, stream);
  }
  return cudaGetLastError();
}

template <typename T>
__global__ void k_gather(const T* __restrict__ in, const int64_t* __restrict__ idx, int64_t n, T* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[idx[i]];
}

cudaError_t launch_gather(int dt, const void* in, const int64_t* d_idx, int64_t n, void* out, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  int grid = (int)((n + 255) / 256);
  if (dt == PQ_C128)
    k_gather<double2><<<grid, 256, 0, stream>>>((const double2*)in, d_idx, n, (double2*)out);
  else
    k_gather<float2><<<grid, 256, 0, stream>>>((const float2*)in, d_idx, n, (float2*)out);
  return cudaGetLastError();
}

// One block per job (grid-stride over jobs): 16-byte vector copies, an
// 8-byte tail by thread 0.
__global__ void __launch_bounds__(256) k_scatter(const unsigned char* __restrict__ src,
                                                 const CopyJob* __restrict__ jobs, int n) {
  for (int j = blockIdx.x; j < n; j += gridDim.x) {
    const CopyJob cj = jobs[j];
    const uint4* s = reinterpret_cast<const uint4*>(src + cj.src_off);
    uint4* d = reinterpret_cast<uint4*>(cj.dst);
    const int64_t n16 = cj.bytes / 16;
    for (int64_t i = threadIdx.x; i < n16; i += blockDim.x) d[i] = s[i];
    if (threadIdx.x == 0 && (cj.bytes & 15))
      reinterpret_cast<uint2*>(cj.dst)[2 * n16] = reinterpret_cast<const uint2*>(src + cj.src_off)[2 * n16];
  }
}

cudaError_t launch_scatter(const void* src, const CopyJob* d_jobs, int n, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const int grid = n < 152 * 8 ? n : 152 * 8;
  k_scatter<<<grid, 256, 0, stream>>>((const unsigned char*)src, d_jobs, n);
  return cudaGetLastError();
}

struct SliceTab {
  int n;
  int64_t dim[kMaxModes];
  int64_t stride[kMaxModes];
};

template <typename T>
__global__ void __launch_bounds__(kGenThreads)
    k_slice_gather(const T* __restrict__ in, T* __restrict__ out, const __grid_constant__ GenericDesc d,
                   const __grid_constant__ SliceTab st, int64_t s0, int64_t nb, int64_t s_end) {
  const int64_t total = d.csize * nb;
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += step) {
    int64_t b = e / d.csize;
    int64_t x = e - b * d.csize;
    int64_t s = s0 + b, so = 0;
    if (s >= s_end) {
      out[e] = T{0, 0};
      continue;
    }
    for (int i = 0; i < st.n; ++i) {
      int64_t q = s / st.dim[i];
      so += (s - q * st.dim[i]) * st.stride[i];
      s = q;
    }
    int64_t oa, ob;
    decode2<false>(x, d, oa, ob);
    out[e] = in[so + oa];
  }
}

cudaError_t launch_slice_gather(int dt, const void* in, void* out, const GenericDesc& d, int nsl,
                                const int64_t* sl_dim, const int64_t* sl_stride, int64_t s0, int64_t nb,
                                int64_t s_end, cudaStream_t stream) {
  SliceTab st;
  st.n = nsl;
  for (int i = 0; i < nsl && i < kMaxModes; ++i) {
    st.dim[i] = sl_dim[i];
    st.stride[i] = sl_stride[i];
  }
  const int grid = grid_for(d.csize * nb, kGenThreads);
  if (dt == PQ_C128)
    k_slice_gather<double2><<<grid, kGenThreads, 0, stream>>>((const double2*)in, (double2*)out, d, st, s0, nb, s_end);
  else
    k_slice_gather<float2><<<grid, kGenThreads, 0, stream>>>((const float2*)in, (float2*)out, d, st, s0, nb, s_end);
  return cudaGetLastError();
}

// Neumaier compensated accumulation of one value into (s, c).
__device__ __forceinline__ void neumaier(double& s, double& c, double x) {
  double t = s + x;
  if (fabs(s) >= fabs(x))
    c += (s - t) + x;
  else
    c += (x - t) + s;
  s = t;
}

// One warp per element: lanes accumulate strided subsets of the batch, then
// lane 0 folds the 32 partial (sum, compensation) pairs in lane order, so the
// result is deterministic.
template <typename T>
__global__ void k_slice_sum(const T* __restrict__ X, int64_t n, int64_t nb, double* acc, double* comp) {
  const int lane = threadIdx.x & 31;
  const int64_t e = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  if (e >= n) return;
  double sr = 0, cr = 0, si = 0, ci = 0;
  for (int64_t b = lane; b < nb; b += 32) {
    T v = X[e + n * b];
    neumaier(sr, cr, (double)v.x);
    neumaier(si, ci, (double)v.y);
  }
  double r_s = acc[2 * e], r_c = comp[2 * e], i_s = acc[2 * e + 1], i_c = comp[2 * e + 1];
  for (int l = 0; l < 32; ++l) {
    double a = __shfl_sync(0xffffffffu, sr, l), b = __shfl_sync(0xffffffffu, cr, l);
    double c = __shfl_sync(0xffffffffu, si, l), dd = __shfl_sync(0xffffffffu, ci, l);
    if (lane == 0) {
      neumaier(r_s, r_c, a);
      r_c += b;
      neumaier(i_s, i_c, c);
      i_c += dd;
    }
  }
  if (lane == 0) {
    acc[2 * e] = r_s;
    comp[2 * e] = r_c;
    acc[2 * e + 1] = i_s;
    comp[2 * e + 1] = i_c;
  }
}

// Squared 2-norm of a complex tensor in FP64 (the fidelity check of a state
// vector): pass 1, every thread a Neumaier sum of |x|^2 over a grid-stride
// range, the block's sums folded by one thread in a fixed order into
// part[block] (value, compensation); pass 2, one thread folds the blocks' parts
// in block order.  Deterministic: no atomics.
constexpr int kNormThreads = 256;
template <typename T>
__global__ void __launch_bounds__(kNormThreads) k_norm2(const T* __restrict__ X, int64_t n, double* part) {
  __shared__ double ss[kNormThreads], sc[kNormThreads];
  double s = 0, c = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T v = X[i];
    neumaier(s, c, (double)v.x * (double)v.x);
    neumaier(s, c, (double)v.y * (double)v.y);
  }
  ss[threadIdx.x] = s;
  sc[threadIdx.x] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    double bs = 0, bc = 0;
    for (int t = 0; t < (int)blockDim.x; ++t) {
      neumaier(bs, bc, ss[t]);
      bc += sc[t];
    }
    part[2 * blockIdx.x] = bs;
    part[2 * blockIdx.x + 1] = bc;
  }
}
__global__ void k_norm2_fold(const double* __restrict__ part, int nblocks, double* out) {
  if (threadIdx.x != 0) return;
  double s = 0, c = 0;
  for (int b = 0; b < nblocks; ++b) {
    neumaier(s, c, part[2 * b]);
    c += part[2 * b + 1];
  }
  *out = s + c;
}

int norm2_blocks(int64_t n) { return (int)std::min<int64_t>(std::max<int64_t>((n + kNormThreads - 1) / kNormThreads, 1), 1024); }

cudaError_t launch_norm2(int dt, const void* X, int64_t n, double* part, double* out, cudaStream_t stream) {
  const int nb = norm2_blocks(n);
  if (dt == PQ_C128)
    k_norm2<double2><<<nb, kNormThreads, 0, stream>>>((const double2*)X, n, part);
  else
    k_norm2<float2><<<nb, kNormThreads, 0, stream>>>((const float2*)X, n, part);
  k_norm2_fold<<<1, 32, 0, stream>>>(part, nb, out);
  return cudaGetLastError();
}

cudaError_t launch_slice_sum(int dt, const void* X, int64_t n, int64_t nb, double* acc, double* comp,
                             cudaStream_t stream) {
  if (n == 0 || nb == 0) return cudaSuccess;
  const int warps = 4;
  int grid = (int)((n + warps - 1) / warps);
  if (dt == PQ_C128)
    k_slice_sum<double2><<<grid, 32 * warps, 0, stream>>>((const double2*)X, n, nb, acc, comp);
  else
    k_slice_sum<float2><<<grid, 32 * warps, 0, stream>>>((const float2*)X, n, nb, acc, comp);
  return cudaGetLastError();
}

}  // namespace pq
