// Tiled SIMT complex GEMM with the index permutation folded into gathered tile
// loads (any mode order in A, B and C), for sm_103a.
//
// Complex128 results accumulate in FP64 (the plain FP64 path).  Complex64
// results accumulate each 16-deep K tile in FP32 and fold the tile sums into a
// Kahan-compensated accumulator, so the rounding error does not grow with K.
#include "pq_types.cuh"

namespace pq {

constexpr int GBM = 64, GBN = 64, GBK = 16, GTHREADS = 256;
static_assert(GBK == kChunk, "the K tile is the compensation chunk");

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

template <typename R>
struct TileAcc;
template <>
struct TileAcc<double> {
  double2 v[4][4];
  __device__ __forceinline__ void init() {
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int s = 0; s < 4; ++s) v[r][s] = make_double2(0.0, 0.0);
  }
  __device__ __forceinline__ double2& part(int r, int s) { return v[r][s]; }
  __device__ __forceinline__ void fold() {}
  __device__ __forceinline__ double2 value(int r, int s) const { return v[r][s]; }
};
template <>
struct TileAcc<float> {
  float2 p[4][4];
  KahanC k[4][4];
  __device__ __forceinline__ void init() {
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        p[r][s] = make_float2(0.f, 0.f);
        kahan_init(k[r][s]);
      }
  }
  __device__ __forceinline__ float2& part(int r, int s) { return p[r][s]; }
  __device__ __forceinline__ void fold() {
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        kahan_add(k[r][s], p[r][s]);
        p[r][s] = make_float2(0.f, 0.f);
      }
  }
  __device__ __forceinline__ float2 value(int r, int s) const { return kahan_value(k[r][s]); }
};

template <typename TA, typename TB, typename TC, typename R>
__global__ void __launch_bounds__(GTHREADS)
    k_gemm(const TA* __restrict__ A, const TB* __restrict__ B, TC* __restrict__ C, const __grid_constant__ GemmDesc d,
           int swap_xy) {
  using AC = typename Acc<R>::C;
  __shared__ AC As[GBK][GBM];
  __shared__ AC Bs[GBK][GBN];
  __shared__ int64_t am[GBM], cm[GBM], bn[GBN], cn[GBN], ak[GBK], bk[GBK];
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  const int64_t bx = swap_xy ? blockIdx.y : blockIdx.x;
  const int64_t by = swap_xy ? blockIdx.x : blockIdx.y;
  const int64_t m0 = bx * GBM;
  const int64_t n0 = by * GBN;
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
    TileAcc<R> acc;
    acc.init();
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
        AC v = czero(R());
        if (am[i] >= 0 && ak[kk] >= 0) v = cvt<R>(__ldg(A + za + am[i] + ak[kk]));
        As[kk][i] = v;
      }
#pragma unroll
      for (int r = 0; r < (GBK * GBN) / GTHREADS; ++r) {
        int e = tid + r * GTHREADS;
        int j = e % GBN, kk = e / GBN;
        AC v = czero(R());
        if (bn[j] >= 0 && bk[kk] >= 0) v = cvt<R>(__ldg(B + zb + bn[j] + bk[kk]));
        Bs[kk][j] = v;
      }
      __syncthreads();
#pragma unroll 4
      for (int kk = 0; kk < GBK; ++kk) {
        AC a[4], b[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) a[r] = As[kk][ty + 16 * r];
#pragma unroll
        for (int s = 0; s < 4; ++s) b[s] = Bs[kk][tx + 16 * s];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int s = 0; s < 4; ++s) cfma(acc.part(r, s), a[r], b[s]);
      }
      acc.fold();
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      int i = ty + 16 * r;
      if (cm[i] < 0) continue;
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        int j = tx + 16 * s;
        if (cn[j] < 0) continue;
        C[zc + cm[i] + cn[j]] = store_as<TC>(acc.value(r, s));
      }
    }
  }
}

template <typename TA, typename TB, typename TC>
static cudaError_t gemm_launch(const void* A, const void* B, void* C, const GemmDesc& d, cudaStream_t s) {
  using R = typename std::conditional<std::is_same<TC, double2>::value, double, float>::type;
  int64_t gm = (d.M + GBM - 1) / GBM, gn = (d.N + GBN - 1) / GBN;
  int swap = 0;
  if (gn > 65535) {  // put the long side on x
    if (gm > 65535) return cudaErrorInvalidConfiguration;
    std::swap(gm, gn);
    swap = 1;
  }
  if (gm > 2147483647LL) return cudaErrorInvalidConfiguration;
  dim3 grid((unsigned)gm, (unsigned)gn, (unsigned)(d.Z < 65535 ? d.Z : 65535));
  k_gemm<TA, TB, TC, R><<<grid, GTHREADS, 0, s>>>((const TA*)A, (const TB*)B, (TC*)C, d, swap);
  return cudaGetLastError();
}

template <typename TA, typename TB>
static cudaError_t gemm_launch_c(int tc, const void* A, const void* B, void* C, const GemmDesc& d, cudaStream_t s) {
  if (tc == PQ_C128) return gemm_launch<TA, TB, double2>(A, B, C, d, s);
  return gemm_launch<TA, TB, float2>(A, B, C, d, s);
}

cudaError_t launch_gemm(int ta, int tb, int tc, const void* A, const void* B, void* C, const GemmDesc& d,
                        cudaStream_t stream) {
  if (d.M * d.N * d.Z == 0) return cudaSuccess;
  if (ta == PQ_C128 && tb == PQ_C128) return gemm_launch_c<double2, double2>(tc, A, B, C, d, stream);
  if (ta == PQ_C128) return gemm_launch_c<double2, float2>(tc, A, B, C, d, stream);
  if (tb == PQ_C128) return gemm_launch_c<float2, double2>(tc, A, B, C, d, stream);
  return gemm_launch_c<float2, float2>(tc, A, B, C, d, stream);
}

}  // namespace pq
