// SIMT contraction kernels for sm_103a.
//
//  * k_generic  — fused permute+contract for memory-bound pairs (gate
//                 applications, small K): one thread per result element,
//                 index maps decoded from the merged mode table, the K offsets
//                 held in shared memory.
//  * k_gemm     — tiled complex GEMM with the index permutation folded into
//                 gathered tile loads (any mode order in A, B and C).  In
//                 complex128 this is the plain FP64 path for large pairs.
//  * k_permute / k_gather / k_slice_gather / k_slice_sum — data movement and
//                 the FP64 compensated slice sum.
#include <cuda_runtime.h>

#include "pq_internal.h"

namespace pq {

template <typename T>
struct Cplx;
template <>
struct Cplx<double2> {
  using R = double;
  static __device__ __forceinline__ double2 zero() { return make_double2(0.0, 0.0); }
};
template <>
struct Cplx<float2> {
  using R = float;
  static __device__ __forceinline__ float2 zero() { return make_float2(0.f, 0.f); }
};

__device__ __forceinline__ void cfma(double2& acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
__device__ __forceinline__ void cfma(float2& acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(a.y, b.x, acc.y);
}

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

template <typename T, bool POW2>
__global__ void __launch_bounds__(kGenThreads)
    k_generic(const T* __restrict__ A, const T* __restrict__ B, T* __restrict__ C,
              const __grid_constant__ GenericDesc d) {
  __shared__ int64_t ka[kGenericKTab];
  __shared__ int64_t kb[kGenericKTab];
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
    T acc = Cplx<T>::zero();
    if (one_chunk) {
      if (active) {
        const T* a = A + oa;
        const T* b = B + ob;
#pragma unroll 4
        for (int k = 0; k < KT; ++k) cfma(acc, __ldg(a + ka[k]), __ldg(b + kb[k]));
      }
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
        if (active) {
          const T* a = A + oa;
          const T* b = B + ob;
#pragma unroll 4
          for (int k = 0; k < kn; ++k) cfma(acc, __ldg(a + ka[k]), __ldg(b + kb[k]));
        }
      }
    }
    if (active) C[c] = acc;
  }
}

static int grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  const int64_t cap = 152 * 8;  // 8 resident 256-thread blocks per SM
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

cudaError_t launch_generic(int precision, const void* A, const void* B, void* C,
                           const GenericDesc& d, cudaStream_t stream) {
  if (d.csize == 0) return cudaSuccess;
  const int grid = grid_for(d.csize, kGenThreads);
  if (precision == PQ_PREC_C128) {
    if (d.pow2)
      k_generic<double2, true><<<grid, kGenThreads, 0, stream>>>((const double2*)A, (const double2*)B,
                                                                 (double2*)C, d);
    else
      k_generic<double2, false><<<grid, kGenThreads, 0, stream>>>((const double2*)A, (const double2*)B,
                                                                  (double2*)C, d);
  } else {
    if (d.pow2)
      k_generic<float2, true><<<grid, kGenThreads, 0, stream>>>((const float2*)A, (const float2*)B,
                                                                (float2*)C, d);
    else
      k_generic<float2, false><<<grid, kGenThreads, 0, stream>>>((const float2*)A, (const float2*)B,
                                                                 (float2*)C, d);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Tiled SIMT complex GEMM with gathered (permuted) operands.
// ---------------------------------------------------------------------------
constexpr int GBM = 64, GBN = 64, GBK = 16, GTHREADS = 256;

__device__ __forceinline__ int64_t decode_off(int64_t x, int n, const int64_t* dim, const int64_t* s1,
                                              const int64_t* s2, int64_t& o2) {
  int64_t o1 = 0;
  o2 = 0;
#pragma unroll 1
  for (int i = 0; i < n; ++i) {
    int64_t q = x / dim[i];
    int64_t r = x - q * dim[i];
    x = q;
    o1 += r * s1[i];
    if (s2) o2 += r * s2[i];
  }
  return o1;
}

template <typename T>
__global__ void __launch_bounds__(GTHREADS)
    k_gemm(const T* __restrict__ A, const T* __restrict__ B, T* __restrict__ C,
           const __grid_constant__ GemmDesc d) {
  __shared__ T As[GBK][GBM];
  __shared__ T Bs[GBK][GBN];
  __shared__ int64_t am[GBM], cm[GBM], bn[GBN], cn[GBN], ak[GBK], bk[GBK];
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  const int64_t m0 = (int64_t)blockIdx.x * GBM;
  const int64_t n0 = (int64_t)blockIdx.y * GBN;
  if (tid < GBM) {
    int64_t m = m0 + tid;
    if (m < d.M) {
      int64_t o2;
      am[tid] = decode_off(m, d.nm, d.mdim, d.msa, d.msc, o2);
      cm[tid] = o2;
    } else {
      am[tid] = -1;
      cm[tid] = -1;
    }
  } else if (tid < GBM + GBN) {
    int j = tid - GBM;
    int64_t n = n0 + j;
    if (n < d.N) {
      int64_t o2;
      bn[j] = decode_off(n, d.nn, d.ndim, d.nsb, d.nsc, o2);
      cn[j] = o2;
    } else {
      bn[j] = -1;
      cn[j] = -1;
    }
  }
  for (int64_t z = blockIdx.z; z < d.Z; z += gridDim.z) {
    // batch offsets
    int64_t za = 0, zb = 0, zc = 0;
    {
      int64_t x = z;
      for (int i = 0; i < d.nz; ++i) {
        int64_t q = x / d.zdim[i];
        int64_t r = x - q * d.zdim[i];
        x = q;
        za += r * d.zsa[i];
        zb += r * d.zsb[i];
        zc += r * d.zsc[i];
      }
    }
    T acc[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int s = 0; s < 4; ++s) acc[r][s] = Cplx<T>::zero();
    for (int64_t k0 = 0; k0 < d.K; k0 += GBK) {
      __syncthreads();
      if (tid < GBK) {
        int64_t k = k0 + tid;
        if (k < d.K) {
          int64_t o2;
          ak[tid] = decode_off(k, d.nk, d.kdim, d.ksa, d.ksb, o2);
          bk[tid] = o2;
        } else {
          ak[tid] = -1;
          bk[tid] = -1;
        }
      }
      __syncthreads();
#pragma unroll
      for (int r = 0; r < (GBK * GBM) / GTHREADS; ++r) {
        int e = tid + r * GTHREADS;
        int i = e % GBM, kk = e / GBM;
        T v = Cplx<T>::zero();
        if (am[i] >= 0 && ak[kk] >= 0) v = __ldg(A + za + am[i] + ak[kk]);
        As[kk][i] = v;
      }
#pragma unroll
      for (int r = 0; r < (GBK * GBN) / GTHREADS; ++r) {
        int e = tid + r * GTHREADS;
        int j = e % GBN, kk = e / GBN;
        T v = Cplx<T>::zero();
        if (bn[j] >= 0 && bk[kk] >= 0) v = __ldg(B + zb + bn[j] + bk[kk]);
        Bs[kk][j] = v;
      }
      __syncthreads();
#pragma unroll 4
      for (int kk = 0; kk < GBK; ++kk) {
        T a[4], b[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) a[r] = As[kk][ty + 16 * r];
#pragma unroll
        for (int s = 0; s < 4; ++s) b[s] = Bs[kk][tx + 16 * s];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int s = 0; s < 4; ++s) cfma(acc[r][s], a[r], b[s]);
      }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      int i = ty + 16 * r;
      if (cm[i] < 0) continue;
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        int j = tx + 16 * s;
        if (cn[j] < 0) continue;
        C[zc + cm[i] + cn[j]] = acc[r][s];
      }
    }
  }
}

cudaError_t launch_gemm(int precision, const void* A, const void* B, void* C, const GemmDesc& d,
                        cudaStream_t stream) {
  if (d.M * d.N * d.Z == 0) return cudaSuccess;
  dim3 grid((unsigned)((d.M + GBM - 1) / GBM), (unsigned)((d.N + GBN - 1) / GBN),
            (unsigned)(d.Z < 65535 ? d.Z : 65535));
  if (grid.x > 2147483647u || grid.y > 65535u) return cudaErrorInvalidConfiguration;
  if (precision == PQ_PREC_C128)
    k_gemm<double2><<<grid, GTHREADS, 0, stream>>>((const double2*)A, (const double2*)B, (double2*)C, d);
  else
    k_gemm<float2><<<grid, GTHREADS, 0, stream>>>((const float2*)A, (const float2*)B, (float2*)C, d);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Data movement
// ---------------------------------------------------------------------------
template <typename T, bool POW2>
__global__ void __launch_bounds__(kGenThreads)
    k_permute(const T* __restrict__ in, int64_t base, T* __restrict__ out,
              const __grid_constant__ GenericDesc d) {
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < d.csize; c += step) {
    int64_t oa, ob;
    decode2<POW2>(c, d, oa, ob);
    out[c] = in[base + oa];
  }
}

cudaError_t launch_permute(int precision, const void* in, int64_t base, void* out, const GenericDesc& d,
                           cudaStream_t stream) {
  if (d.csize == 0) return cudaSuccess;
  const int grid = grid_for(d.csize, kGenThreads);
  if (precision == PQ_PREC_C128) {
    if (d.pow2)
      k_permute<double2, true><<<grid, kGenThreads, 0, stream>>>((const double2*)in, base, (double2*)out, d);
    else
      k_permute<double2, false><<<grid, kGenThreads, 0, stream>>>((const double2*)in, base, (double2*)out, d);
  } else {
    if (d.pow2)
      k_permute<float2, true><<<grid, kGenThreads, 0, stream>>>((const float2*)in, base, (float2*)out, d);
    else
      k_permute<float2, false><<<grid, kGenThreads, 0, stream>>>((const float2*)in, base, (float2*)out, d);
  }
  return cudaGetLastError();
}

template <typename T>
__global__ void k_gather(const T* __restrict__ in, const int64_t* __restrict__ idx, int64_t n,
                         T* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[idx[i]];
}

cudaError_t launch_gather(int precision, const void* in, const int64_t* d_idx, int64_t n, void* out,
                          cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  int grid = (int)((n + 255) / 256);
  if (precision == PQ_PREC_C128)
    k_gather<double2><<<grid, 256, 0, stream>>>((const double2*)in, d_idx, n, (double2*)out);
  else
    k_gather<float2><<<grid, 256, 0, stream>>>((const float2*)in, d_idx, n, (float2*)out);
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
      out[e] = Cplx<T>::zero();
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

cudaError_t launch_slice_gather(int precision, const void* in, void* out, const GenericDesc& d, int nsl,
                                const int64_t* sl_dim, const int64_t* sl_stride, int64_t s0, int64_t nb,
                                int64_t s_end, cudaStream_t stream) {
  SliceTab st;
  st.n = nsl;
  for (int i = 0; i < nsl && i < kMaxModes; ++i) {
    st.dim[i] = sl_dim[i];
    st.stride[i] = sl_stride[i];
  }
  const int grid = grid_for(d.csize * nb, kGenThreads);
  if (precision == PQ_PREC_C128)
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

cudaError_t launch_slice_sum(int precision, const void* X, int64_t n, int64_t nb, double* acc, double* comp,
                             cudaStream_t stream) {
  if (n == 0 || nb == 0) return cudaSuccess;
  const int warps = 4;
  int grid = (int)((n + warps - 1) / warps);
  if (precision == PQ_PREC_C128)
    k_slice_sum<double2><<<grid, 32 * warps, 0, stream>>>((const double2*)X, n, nb, acc, comp);
  else
    k_slice_sum<float2><<<grid, 32 * warps, 0, stream>>>((const float2*)X, n, nb, acc, comp);
  return cudaGetLastError();
}

}  // namespace pq
