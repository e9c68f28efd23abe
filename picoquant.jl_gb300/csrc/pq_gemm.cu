// Tiled SIMT complex GEMM with the index permutation folded into gathered tile
// loads (any mode order in A, B and C), for sm_103a.
//
// Complex128 results accumulate in FP64 (the plain FP64 path).  Complex64
// results accumulate each 16-deep K tile in FP32 and fold the tile sums into a
// Kahan-compensated accumulator, so the rounding error does not grow with K.
//
// Three tile shapes (256 threads, each owning R x S results):
//   square  BM=64,  BN=64,  R=4,  S=4   general pairs
//   tall    BM=256, BN=16,  R=16, S=1   narrow N (e.g. a big boundary absorbing
//                                        a qubit with few open bonds)
//   wide    BM=16,  BN=256, R=1,  S=16  narrow M
// The next K tile's gathered global loads are issued into registers before
// the current tile is consumed from shared memory (double buffering).
#include "pq_types.cuh"

namespace pq {

constexpr int GBK = 16, GTHREADS = 256;
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

template <typename R, int NACC>
struct TileAcc;
template <int NACC>
struct TileAcc<double, NACC> {
  double2 v[NACC];
  __device__ __forceinline__ void init() {
#pragma unroll
    for (int i = 0; i < NACC; ++i) v[i] = make_double2(0.0, 0.0);
  }
  __device__ __forceinline__ double2& part(int i) { return v[i]; }
  __device__ __forceinline__ void fold() {}
  __device__ __forceinline__ double2 value(int i) const { return v[i]; }
};
template <int NACC>
struct TileAcc<float, NACC> {
  float2 p[NACC];
  KahanC k[NACC];
  __device__ __forceinline__ void init() {
#pragma unroll
    for (int i = 0; i < NACC; ++i) {
      p[i] = make_float2(0.f, 0.f);
      kahan_init(k[i]);
    }
  }
  __device__ __forceinline__ float2& part(int i) { return p[i]; }
  __device__ __forceinline__ void fold() {
#pragma unroll
    for (int i = 0; i < NACC; ++i) {
      kahan_add(k[i], p[i]);
      p[i] = make_float2(0.f, 0.f);
    }
  }
  __device__ __forceinline__ float2 value(int i) const { return kahan_value(k[i]); }
};

template <typename TA, typename TB, typename TC, typename R, int BM, int BN, int RR, int SS>
__global__ void __launch_bounds__(GTHREADS)
    k_gemm(const TA* __restrict__ A, const TB* __restrict__ B, TC* __restrict__ C, const __grid_constant__ GemmDesc d,
           int swap_xy) {
  using AC = typename Acc<R>::C;
  constexpr int TX = BN / SS, TY = BM / RR;  // thread grid
  static_assert(TX * TY == GTHREADS, "thread grid");
  constexpr int LA = (GBK * BM) / GTHREADS, LB = (GBK * BN) / GTHREADS;  // loads per thread
  static_assert(LA * GTHREADS == GBK * BM && LB * GTHREADS == GBK * BN, "tile loads");
  __shared__ AC As[GBK][BM];
  __shared__ AC Bs[GBK][BN];
  __shared__ int64_t am[BM], cm[BM], bn[BN], cn[BN], ak[2][GBK], bk[2][GBK];
  const int tid = threadIdx.x;
  const int tx = tid % TX, ty = tid / TX;
  const int64_t bx = swap_xy ? blockIdx.y : blockIdx.x;
  const int64_t by = swap_xy ? blockIdx.x : blockIdx.y;
  const int64_t m0 = bx * BM;
  const int64_t n0 = by * BN;
  for (int i = tid; i < BM + BN; i += GTHREADS) {
    if (i < BM) {
      int64_t m = m0 + i;
      if (m < d.M) {
        int64_t o2;
        am[i] = decode_off(m, d.nm, d.mdim, d.msa, d.msc, o2);
        cm[i] = o2;
      } else {
        am[i] = -1;
        cm[i] = -1;
      }
    } else {
      int j = i - BM;
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
  }
  auto k_offsets = [&](int buf, int64_t k0) {
    if (tid < GBK) {
      int64_t k = k0 + tid;
      if (k < d.K) {
        int64_t o2;
        ak[buf][tid] = decode_off(k, d.nk, d.kdim, d.ksa, d.ksb, o2);
        bk[buf][tid] = o2;
      } else {
        ak[buf][tid] = -1;
        bk[buf][tid] = -1;
      }
    }
  };
  const int64_t nkt = (d.K + GBK - 1) / GBK;
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
    TileAcc<R, RR * SS> acc;
    acc.init();
    AC ra[LA], rb[LB];  // next tile, staged in registers
    __syncthreads();    // previous z iteration done with the offsets / tiles
    k_offsets(0, 0);
    __syncthreads();
    auto fetch = [&](int buf) {
#pragma unroll
      for (int r = 0; r < LA; ++r) {
        int e = tid + r * GTHREADS;
        int i = e % BM, kk = e / BM;
        ra[r] = (am[i] >= 0 && ak[buf][kk] >= 0) ? cvt<R>(__ldg(A + za + am[i] + ak[buf][kk])) : czero(R());
      }
#pragma unroll
      for (int r = 0; r < LB; ++r) {
        int e = tid + r * GTHREADS;
        int j = e % BN, kk = e / BN;
        rb[r] = (bn[j] >= 0 && bk[buf][kk] >= 0) ? cvt<R>(__ldg(B + zb + bn[j] + bk[buf][kk])) : czero(R());
      }
    };
    fetch(0);
    for (int64_t t = 0; t < nkt; ++t) {
      const int buf = (int)(t & 1);
      // registers -> shared tile
#pragma unroll
      for (int r = 0; r < LA; ++r) {
        int e = tid + r * GTHREADS;
        As[e / BM][e % BM] = ra[r];
      }
#pragma unroll
      for (int r = 0; r < LB; ++r) {
        int e = tid + r * GTHREADS;
        Bs[e / BN][e % BN] = rb[r];
      }
      if (t + 1 < nkt) k_offsets(buf ^ 1, (t + 1) * GBK);
      __syncthreads();
      if (t + 1 < nkt) fetch(buf ^ 1);  // global loads of the next tile overlap the math below
#pragma unroll 4
      for (int kk = 0; kk < GBK; ++kk) {
        AC a[RR], b[SS];
#pragma unroll
        for (int r = 0; r < RR; ++r) a[r] = As[kk][ty + TY * r];
#pragma unroll
        for (int s = 0; s < SS; ++s) b[s] = Bs[kk][tx + TX * s];
#pragma unroll
        for (int r = 0; r < RR; ++r)
#pragma unroll
          for (int s = 0; s < SS; ++s) cfma(acc.part(r * SS + s), a[r], b[s]);
      }
      acc.fold();
      __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < RR; ++r) {
      int i = ty + TY * r;
      if (cm[i] < 0) continue;
#pragma unroll
      for (int s = 0; s < SS; ++s) {
        int j = tx + TX * s;
        if (cn[j] < 0) continue;
        C[zc + cm[i] + cn[j]] = store_as<TC>(acc.value(r * SS + s));
      }
    }
  }
}

template <typename TA, typename TB, typename TC, int BM, int BN, int RR, int SS>
static cudaError_t gemm_launch(const void* A, const void* B, void* C, const GemmDesc& d, cudaStream_t s) {
  using R = typename std::conditional<std::is_same<TC, double2>::value, double, float>::type;
  int64_t gm = (d.M + BM - 1) / BM, gn = (d.N + BN - 1) / BN;
  int swap = 0;
  if (gn > 65535) {  // put the long side on x
    if (gm > 65535) return cudaErrorInvalidConfiguration;
    std::swap(gm, gn);
    swap = 1;
  }
  if (gm > 2147483647LL) return cudaErrorInvalidConfiguration;
  dim3 grid((unsigned)gm, (unsigned)gn, (unsigned)(d.Z < 65535 ? d.Z : 65535));
  k_gemm<TA, TB, TC, R, BM, BN, RR, SS><<<grid, GTHREADS, 0, s>>>((const TA*)A, (const TB*)B, (TC*)C, d, swap);
  return cudaGetLastError();
}

template <typename TA, typename TB, typename TC>
static cudaError_t gemm_shape(int shape, const void* A, const void* B, void* C, const GemmDesc& d, cudaStream_t s) {
  // the narrow tiles need 32 KiB of complex64 staging; complex128 results
  // (FP64 accumulation, twice the tile bytes) always use the square tile
  if constexpr (std::is_same<TC, float2>::value) {
    if (shape == GEMM_TALL) return gemm_launch<TA, TB, TC, 256, 16, 16, 1>(A, B, C, d, s);
    if (shape == GEMM_WIDE) return gemm_launch<TA, TB, TC, 16, 256, 1, 16>(A, B, C, d, s);
  }
  return gemm_launch<TA, TB, TC, 64, 64, 4, 4>(A, B, C, d, s);
}

template <typename TA, typename TB>
static cudaError_t gemm_launch_c(int tc, int shape, const void* A, const void* B, void* C, const GemmDesc& d,
                                 cudaStream_t s) {
  if (tc == PQ_C128) return gemm_shape<TA, TB, double2>(shape, A, B, C, d, s);
  return gemm_shape<TA, TB, float2>(shape, A, B, C, d, s);
}

int gemm_tile_shape(const GemmDesc& d) {
  if (d.N < 32 && d.M >= 4 * d.N) return GEMM_TALL;
  if (d.M < 32 && d.N >= 4 * d.M) return GEMM_WIDE;
  return GEMM_SQUARE;
}

cudaError_t launch_gemm(int ta, int tb, int tc, const void* A, const void* B, void* C, const GemmDesc& d,
                        cudaStream_t stream) {
  if (d.M * d.N * d.Z == 0) return cudaSuccess;
  const int shape = gemm_tile_shape(d);
  if (ta == PQ_C128 && tb == PQ_C128) return gemm_launch_c<double2, double2>(tc, shape, A, B, C, d, stream);
  if (ta == PQ_C128) return gemm_launch_c<double2, float2>(tc, shape, A, B, C, d, stream);
  if (tb == PQ_C128) return gemm_launch_c<float2, double2>(tc, shape, A, B, C, d, stream);
  return gemm_launch_c<float2, float2>(tc, shape, A, B, C, d, stream);
}

}  // namespace pq
