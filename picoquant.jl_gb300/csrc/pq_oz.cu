// Exact-accumulation split-precision complex contraction on the tcgen05 tensor
// cores (sm_103a, PQ_PREC_OZAKI): the Ozaki scheme (Ozaki, Ogita, Oishi, Rump,
// "Error-free transformations of matrix multiplication by using fast routines
// of matrix multiplication and its applicability", Numer. Algorithms 59, 2012)
// with bf16 slices and FP32 accumulation in TMEM.
//
// Scaling.  Every row m of A (over K, per batch index) gets the power of two
// 2^ea[m] with every |Re|, |Im| of the row below it (frexp exponent of the row
// maximum); likewise every column n of B gets 2^eb[n].  A scaled value
// x = a 2^-ea in (-1, 1) is cut into five slices on fixed grids
//   s0 = rint(x 2^7) 2^-7,  s_i = rint((x - s0 - .. - s_{i-1}) 2^{7(i+1)}) 2^{-7(i+1)}
// (|s0| <= 1, |s_i| <= 2^{-7i-1}), each an integer of at most 8 bits times a
// power of two, hence exact in bf16; x - (s0 + .. + s4) is below 2^-36, so a
// value 2^-10 below its row maximum still keeps 26 significant bits.
//
// Products.  s_i t_j is an integer multiple of 2^{-7(i+j+2)} of magnitude at
// most 2^{-7(i+j)}.  The 15 slice pairs with i + j <= 4 are accumulated by
// level l = i + j into three accumulators per real output (Cr, Ci):
//   level 0   (0,0)             multiples of 2^-14, |sum| <= 2K
//   level 1   (0,1) (1,0)       multiples of 2^-21, |sum| <= 4K 2^-8
//   levels 2-4 (the other 12)   |sum| <= 2^-14 relative
// For K <= 512 the level-0 and level-1 sums fit the 24-bit FP32 significand
// on their grids, so the tensor core accumulates them EXACTLY (its rounding
// of an accumulation never drops a bit); only the small levels 2-4 round
// (truncation, about 2^-30 relative after K).  The result is
// (L0 + L1 + L2) 2^(ea+eb) rounded once to the output type, so the error is
// the output rounding plus the dropped pairs and slice residuals, at most
// 2^-33 K 2^(ea+eb) per component.  (Dropping level 4 -- four slices, ten
// pairs -- was measured to double the amplitude error of deep circuits:
// their rows span many binades.)
//   Cr = Ar.Br + (-Ai).Bi   (the negation is the MMA's negate-A bit)
//   Ci = Ar.Bi + Ai.Br
//
// Kernels (one launch each, in stream order):
//   k_oz_exp      row / column scale exponents of A and B
//   k_oz_pack     slices into planes [z][row tile][k tile][plane][ROWS*16 bf16]
//                 in the canonical no-swizzle K-major UMMA layout (8-row x
//                 16-byte core matrices: 8 rows x 8 bf16), planes
//                 {Re s0..s4, Im s0..s4}; rows and K beyond the operand are 0
//   k_result_index result offsets of every row and column of C
//   k_oz_gemm     persistent, one CTA per SM over 128 x TN output tiles (TN =
//                 64, or 32 / 16 for narrow pairs; a pair whose A side is the
//                 narrow one runs as B x A):
//     warp 0     producer: cp.async.bulk of the 20 plane tiles of one 16-deep
//                K tile into a 3- or 4-stage shared-memory ring;
//     warp 1     TMEM owner and MMA issuer: 60 tcgen05.mma (kind::f16, bf16,
//                M=128, N=TN, K=16) per K tile into six TN-column
//                accumulators (L0r L0i L1r L1i L2r L2i);
//     warps 2-9  epilogue, once per tile: warp w reads TMEM lanes 32*(w%4)..
//                and half of the TN columns, combines the levels with an
//                error-free two-sum, scales by 2^(ea+eb) and scatters C
//                through the result index map.
// Every mbarrier wait is bounded; on expiry the kernel records an error in the
// context's status word and runs to the end (TMEM is always released).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "pq_tcgen05.cuh"
#include "pq_types.cuh"

namespace pq {

namespace {

using namespace tcg;

constexpr int TM = 128, TK = 16;
constexpr int kSlices = 5;                       // bf16 slices per real value
constexpr int kPlanes = 2 * kSlices;             // per operand: Re s0..s4, Im s0..s4
constexpr int kPairs = 15;                       // slice pairs (i, j) with i + j <= 4
constexpr int kThreads = 320;                    // producer, MMA, 8 epilogue warps
constexpr int kEpiWarps = 8;
constexpr int kATile = TM * TK;                  // bf16 per A plane tile (4 KiB)

// Tile width N: 64 for general pairs, 32 and 16 for narrow ones.
template <int TN>
struct OzCfg {
  static constexpr int kBTile = TN * TK;                                   // bf16 per B plane tile
  static constexpr uint32_t stage_bytes = kPlanes * (kATile + kBTile) * 2;
  static constexpr int stages = TN == 64 ? 3 : 4;
  static constexpr uint32_t tmem_cols = TN == 64 ? 512 : (TN == 32 ? 256 : 128);  // >= 6 TN, power of 2
  static constexpr int cw = TN / (kEpiWarps / 4);                           // columns per epilogue warp
  static_assert(6 * TN <= (int)tmem_cols && cw % 8 == 0, "tile width");
};
constexpr int kExpZero = -4096;                  // exponent of an all-zero row
constexpr int64_t kMaxK = 512;                   // exact level-0/1 sums up to this K

// slice pairs, level 0 first, then level 1, then levels 4, 3, 2 (the inexact
// accumulator takes its small terms first)
//   i: 0 0 1 0 1 2 3 4 0 1 2 3 0 1 2
//   j: 0 1 0 4 3 2 1 0 3 2 1 0 2 1 0
// (4-bit fields, pair p in bits [4p, 4p + 4))
__host__ __device__ constexpr int pair_i(int p) { return (int)((uint64_t)0x210321043210100ull >> (4 * p)) & 15; }
__host__ __device__ constexpr int pair_j(int p) { return (int)((uint64_t)0x12012301234010ull >> (4 * p)) & 15; }

__host__ __device__ constexpr int level_of(int p) { return p == 0 ? 0 : (p < 3 ? 1 : 2); }
__host__ __device__ constexpr bool first_of_level(int p) { return p == 0 || p == 1 || p == 3; }

template <typename T>
struct Real;
template <>
struct Real<float2> {
  using R = float;
};
template <>
struct Real<double2> {
  using R = double;
};

__device__ __forceinline__ float absmax(float a, float b) { return fmaxf(fabsf(a), fabsf(b)); }
__device__ __forceinline__ double absmax(double a, double b) { return fmax(fabs(a), fabs(b)); }
__device__ __forceinline__ float scale2(float x, int e) { return ldexpf(x, e); }
__device__ __forceinline__ double scale2(double x, int e) { return ldexp(x, e); }
__device__ __forceinline__ float round_int(float x) { return rintf(x); }
__device__ __forceinline__ double round_int(double x) { return rint(x); }

__device__ __forceinline__ int exp_of(float v) {
  int e;
  frexpf(v, &e);
  return v == 0.f ? kExpZero : e;
}
__device__ __forceinline__ int exp_of(double v) {
  int e;
  frexp(v, &e);
  return v == 0.0 ? kExpZero : e;
}

// Row (side 0: A rows m) or column (side 1: B columns n) scale exponents:
// e[z * rows + r] = max over k of the frexp exponent of max(|Re|, |Im|).
// One block per (ROWS-row tile, z); every K offset is staged in shared memory.
template <typename T, int ROWS>
__global__ void __launch_bounds__(256) k_oz_exp(const T* __restrict__ X, const __grid_constant__ GemmDesc d, int side,
                                                int64_t rows, int* __restrict__ e_out) {
  __shared__ int64_t roff[ROWS];
  __shared__ int64_t koff[kMaxK];
  __shared__ int emax[ROWS];
  const int64_t rt = blockIdx.x, z = blockIdx.y;
  const int nrm = side == 0 ? d.nm : d.nn;
  const int64_t* rdim = side == 0 ? d.mdim : d.ndim;
  const int64_t* rstr = side == 0 ? d.msa : d.nsb;
  const int64_t* kstr = side == 0 ? d.ksa : d.ksb;
  const int64_t* zstr = side == 0 ? d.zsa : d.zsb;
  for (int t = threadIdx.x; t < ROWS; t += blockDim.x) {
    const int64_t r = rt * ROWS + t;
    roff[t] = r < rows ? decode(r, nrm, rdim, rstr) : -1;
    emax[t] = kExpZero;
  }
  for (int t = threadIdx.x; t < d.K; t += blockDim.x) koff[t] = decode(t, d.nk, d.kdim, kstr);
  __syncthreads();
  const int64_t zo = decode(z, d.nz, d.zdim, zstr);
  using R = typename Real<T>::R;
  const int64_t n = (int64_t)ROWS * d.K;
  for (int64_t o = threadIdx.x; o < n; o += blockDim.x) {
    const int r = (int)(o % ROWS);
    const int64_t k = o / ROWS;
    if (roff[r] < 0) continue;
    const T v = X[zo + roff[r] + koff[k]];
    const R m = absmax((R)v.x, (R)v.y);
    atomicMax(&emax[r], exp_of(m));
  }
  __syncthreads();
  for (int t = threadIdx.x; t < ROWS; t += blockDim.x) {
    const int64_t r = rt * ROWS + t;
    if (r < rows) e_out[z * rows + r] = emax[t];
  }
}

// The slices of x (|x| < 1 after scaling); every step is exact in R.
template <typename R>
__device__ __forceinline__ void slices(R x, float* s) {
  R r = x;
  R g = (R)128.0;  // 2^7(i+1)
#pragma unroll
  for (int i = 0; i < kSlices; ++i) {
    const R si = round_int(r * g) / g;
    s[i] = (float)si;
    r -= si;
    g *= (R)128.0;
  }
}

template <typename T, int ROWS>
__global__ void __launch_bounds__(256) k_oz_pack(const T* __restrict__ X, __nv_bfloat16* __restrict__ planes,
                                                 const __grid_constant__ GemmDesc d, int side, int64_t rows,
                                                 int64_t rtiles, int64_t ktiles, const int* __restrict__ e_in) {
  constexpr int TILE = ROWS * TK, GROUPS = ROWS / 8;
  __shared__ int64_t roff[ROWS];
  __shared__ int rexp[ROWS];
  __shared__ int64_t koff[TK];
  const int64_t kt = blockIdx.x, rt = blockIdx.y, z = blockIdx.z;
  const int nrm = side == 0 ? d.nm : d.nn;
  const int64_t* rdim = side == 0 ? d.mdim : d.ndim;
  const int64_t* rstr = side == 0 ? d.msa : d.nsb;
  const int64_t* kstr = side == 0 ? d.ksa : d.ksb;
  const int64_t* zstr = side == 0 ? d.zsa : d.zsb;
  for (int t = threadIdx.x; t < ROWS + TK; t += blockDim.x) {
    if (t < ROWS) {
      const int64_t r = rt * ROWS + t;
      roff[t] = r < rows ? decode(r, nrm, rdim, rstr) : -1;
      rexp[t] = r < rows ? e_in[z * rows + r] : kExpZero;
    } else {
      const int64_t k = kt * TK + (t - ROWS);
      koff[t - ROWS] = k < d.K ? decode(k, d.nk, d.kdim, kstr) : -1;
    }
  }
  __syncthreads();
  const int64_t zo = decode(z, d.nz, d.zdim, zstr);
  using R = typename Real<T>::R;
  __nv_bfloat16* tile = planes + (((z * rtiles + rt) * ktiles + kt) * kPlanes) * (int64_t)TILE;
  for (int o = threadIdx.x; o < TILE; o += blockDim.x) {
    // o = ((kc * GROUPS + g) * 8 + r8) * 8 + k8: core matrix (kc, g), row r8, K k8
    const int core = o >> 6, within = o & 63;
    const int kc = core / GROUPS, g = core - kc * GROUPS;
    const int r = g * 8 + (within >> 3), k = kc * 8 + (within & 7);
    float re[kSlices], im[kSlices];
#pragma unroll
    for (int i = 0; i < kSlices; ++i) re[i] = im[i] = 0.f;
    if (roff[r] >= 0 && koff[k] >= 0 && rexp[r] != kExpZero) {
      const T v = X[zo + roff[r] + koff[k]];
      slices<R>(scale2((R)v.x, -rexp[r]), re);
      slices<R>(scale2((R)v.y, -rexp[r]), im);
    }
#pragma unroll
    for (int i = 0; i < kSlices; ++i) {
      tile[(0 * kSlices + i) * TILE + o] = __float2bfloat16_rn(re[i]);
      tile[(1 * kSlices + i) * TILE + o] = __float2bfloat16_rn(im[i]);
    }
  }
}

template <int TN>
struct alignas(1024) OzSmem {
  __nv_bfloat16 stage[OzCfg<TN>::stages][kPlanes * (kATile + OzCfg<TN>::kBTile)];  // A planes, then B planes
  uint64_t full[OzCfg<TN>::stages];
  uint64_t empty[OzCfg<TN>::stages];
  uint64_t accf;
  uint64_t acce;
  uint64_t drain;
  uint32_t tmem_base;
};

// a + b = s + e exactly (Knuth's two-sum).
__device__ __forceinline__ float two_sum(float a, float b, float& e) {
  const float s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
  return s;
}
__device__ __forceinline__ float combine(float l0, float l1, float l2, int ex, float) {
  float e;
  const float s = two_sum(l0, l1, e);
  return ldexpf(s + (e + l2), ex);
}
__device__ __forceinline__ double combine(float l0, float l1, float l2, int ex, double) {
  return ldexp(((double)l0 + (double)l1) + (double)l2, ex);
}

template <typename TC, int TN>
__global__ void __launch_bounds__(kThreads, 1)
    k_oz_gemm(const __nv_bfloat16* __restrict__ pa, const __nv_bfloat16* __restrict__ pb, TC* __restrict__ C,
              const __grid_constant__ GemmDesc d, const int64_t* __restrict__ cm_tab,
              const int64_t* __restrict__ cn_tab, const int* __restrict__ ea, const int* __restrict__ eb,
              int64_t mtiles, int64_t ntiles, int64_t ktiles, int* status) {
  using CF = OzCfg<TN>;
  constexpr int kStages = CF::stages, kBTile = CF::kBTile;
  constexpr uint32_t kTmemCols = CF::tmem_cols;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  OzSmem<TN>& sm = *reinterpret_cast<OzSmem<TN>*>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ntot = ntiles * mtiles * d.Z;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&sm.full[s], 1);
      mbar_init(&sm.empty[s], 1);
    }
    mbar_init(&sm.accf, 1);
    mbar_init(&sm.acce, kEpiWarps);  // one arrival per epilogue warp
    mbar_init(&sm.drain, 1);
    mbar_init_fence();
  }
  if (warp == 1) tmem_alloc(&sm.tmem_base, kTmemCols);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = sm.tmem_base;
  bool ok = true;

  if (warp == 0) {
    if (lane == 0) {
      int64_t g = 0;  // K tiles issued so far (all tiles)
      for (int64_t tile = blockIdx.x; tile < ntot && ok; tile += gridDim.x) {
        const int64_t nt = tile % ntiles, r = tile / ntiles, mt = r % mtiles, z = r / mtiles;
        const __nv_bfloat16* atile = pa + ((z * mtiles + mt) * ktiles) * (int64_t)(kPlanes * kATile);
        const __nv_bfloat16* btile = pb + ((z * ntiles + nt) * ktiles) * (int64_t)(kPlanes * kBTile);
        for (int64_t kt = 0; kt < ktiles; ++kt, ++g) {
          const int s = (int)(g % kStages);
          const uint32_t ph = (uint32_t)((g / kStages) & 1);
          if (!mbar_wait(&sm.empty[s], ph ^ 1)) {
            ok = false;
            break;
          }
          mbar_expect_tx(&sm.full[s], CF::stage_bytes);
          const __nv_bfloat16* a = atile + kt * (kPlanes * kATile);
          const __nv_bfloat16* b = btile + kt * (kPlanes * kBTile);
          __nv_bfloat16* dst = sm.stage[s];
#pragma unroll
          for (int p = 0; p < kPlanes; ++p) {
            bulk_g2s(dst + p * kATile, a + p * kATile, kATile * 2, &sm.full[s]);
            bulk_g2s(dst + kPlanes * kATile + p * kBTile, b + p * kBTile, kBTile * 2, &sm.full[s]);
          }
        }
      }
      // the copies of the last stages are in flight until their full barrier
      // completes: wait (bounded) so none lands after the CTA has exited
      for (int64_t i = g - 1; i >= 0 && i >= g - kStages; --i)
        if (!mbar_wait(&sm.full[i % kStages], (uint32_t)((i / kStages) & 1))) ok = false;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_bf16(TM, TN), idesc_neg = idesc_bf16(TM, TN, true);
      constexpr uint32_t ALBO = (TM / 8) * 128, BLBO = (TN / 8) * 128, SBO = 128;
      int64_t g = 0;  // K tiles consumed so far
      int64_t t = 0;  // tiles of this CTA
      for (int64_t tile = blockIdx.x; tile < ntot && ok; tile += gridDim.x, ++t) {
        // the epilogue of the previous tile has read the accumulators
        if (!mbar_wait(&sm.acce, (uint32_t)((t & 1) ^ 1))) {
          ok = false;
          break;
        }
        fence_after();
        for (int64_t kt = 0; kt < ktiles; ++kt, ++g) {
          const int s = (int)(g % kStages);
          const uint32_t ph = (uint32_t)((g / kStages) & 1);
          if (!mbar_wait(&sm.full[s], ph)) {
            ok = false;
            break;
          }
          fence_after();
          const uint32_t sa = smem_u32(sm.stage[s]);
          const uint64_t a0 = smem_desc(sa, ALBO, SBO);
          const uint64_t b0 = smem_desc(sa + kPlanes * kATile * 2, BLBO, SBO);
#pragma unroll
          for (int p = 0; p < kPairs; ++p) {
            const int i = pair_i(p), j = pair_j(p);
            const uint32_t acc = (kt == 0 && first_of_level(p)) ? 0u : 1u;
            const uint32_t dr = tmem + (uint32_t)(level_of(p) * 2 * TN), di = dr + TN;
            const uint64_t ar = a0 + (uint64_t)(((0 * kSlices + i) * kATile * 2) >> 4);
            const uint64_t ai = a0 + (uint64_t)(((1 * kSlices + i) * kATile * 2) >> 4);
            const uint64_t br = b0 + (uint64_t)(((0 * kSlices + j) * kBTile * 2) >> 4);
            const uint64_t bi = b0 + (uint64_t)(((1 * kSlices + j) * kBTile * 2) >> 4);
            mma_bf16(dr, ar, br, idesc, acc);     // + Ar.Br
            mma_bf16(di, ar, bi, idesc, acc);     // + Ar.Bi
            mma_bf16(dr, ai, bi, idesc_neg, 1u);  // - Ai.Bi
            mma_bf16(di, ai, br, idesc, 1u);      // + Ai.Br
          }
          mma_commit(&sm.empty[s]);  // smem stage free once these MMAs finish
        }
        if (!ok) break;
        mma_commit(&sm.accf);  // tile accumulators ready for the epilogue
      }
      // every MMA issued has finished once this arrives (TMEM is freed below)
      mma_commit(&sm.drain);
      if (!mbar_wait(&sm.drain, 0)) ok = false;
    }
  } else {
    // epilogue: warp w reads TMEM lanes of quadrant w % 4, columns [32h, 32h+32)
    constexpr int CW = CF::cw;
    const int q = warp & 3, h = (warp - 2) >> 2;
    const int row = q * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
    using R = typename std::conditional<std::is_same<TC, double2>::value, double, float>::type;
    int64_t t = 0;
    for (int64_t tile = blockIdx.x; tile < ntot && ok; tile += gridDim.x, ++t) {
      const int64_t nt = tile % ntiles, r = tile / ntiles, mt = r % mtiles, z = r / mtiles;
      bool got = mbar_wait(&sm.accf, (uint32_t)(t & 1));
      got = __all_sync(0xffffffffu, got);  // the TMEM loads below are warp-collective
      if (!got) {
        ok = false;
        break;
      }
      fence_after();
      const int64_t m = mt * TM + row;
      const bool mrow = m < d.M;
      const int64_t base = mrow ? decode(z, d.nz, d.zdim, d.zsc) + cm_tab[m] : 0;
      const int exa = mrow ? ea[z * d.M + m] : 0;
#pragma unroll 1
      for (int piece = 0; piece < CW / 8; ++piece) {
        __syncwarp();  // the TMEM loads are warp-collective
        const uint32_t col = (uint32_t)(h * CW + piece * 8);
        float l0r[8], l0i[8], l1r[8], l1i[8], l2r[8], l2i[8];
        tmem_ld8(lane_base + col + 0 * TN, l0r);
        tmem_ld8(lane_base + col + 1 * TN, l0i);
        tmem_ld8(lane_base + col + 2 * TN, l1r);
        tmem_ld8(lane_base + col + 3 * TN, l1i);
        tmem_ld8(lane_base + col + 4 * TN, l2r);
        tmem_ld8(lane_base + col + 5 * TN, l2i);
        tmem_wait_ld();
        if (piece == CW / 8 - 1) {  // every value of this tile is in registers
          fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&sm.acce);
        }
        const int64_t n0 = nt * TN + col;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          if (!mrow || n0 + j >= d.N) break;
          const int ex = exa + eb[z * d.N + n0 + j];
          R vr, vi;
          if (exa == kExpZero || ex < -2 * 1100) {
            vr = vi = (R)0;  // an all-zero row or column
          } else {
            vr = combine(l0r[j], l1r[j], l2r[j], ex, R());
            vi = combine(l0i[j], l1i[j], l2i[j], ex, R());
          }
          TC out;
          out.x = vr;
          out.y = vi;
          C[base + cn_tab[n0 + j]] = out;
        }
      }
    }
  }
  if (!ok && status) atomicExch(status, kStatusTcTimeout);
  fence_before();
  __syncthreads();
  if (warp == 1) {
    fence_after();
    tmem_dealloc(tmem, kTmemCols);
  }
}

int oz_tile_n(int64_t n) { return n <= 16 ? 16 : (n <= 32 ? 32 : 64); }

struct OzLayout {
  int tn;
  int64_t mt, nt, kt;
  size_t pa, pb, cm, cn, ea, eb, total;  // byte offsets from the aligned base
};

OzLayout layout(const GemmDesc& d) {
  OzLayout L;
  L.tn = oz_tile_n(d.N);
  L.mt = ceil_div(d.M, TM);
  L.nt = ceil_div(d.N, L.tn);
  L.kt = ceil_div(d.K, TK);
  auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  L.pa = 0;
  L.pb = up(L.pa + (size_t)(d.Z * L.mt * L.kt) * kPlanes * kATile * 2);
  L.cm = up(L.pb + (size_t)(d.Z * L.nt * L.kt) * kPlanes * (L.tn * TK) * 2);
  L.cn = up(L.cm + (size_t)d.M * 8);
  L.ea = up(L.cn + (size_t)d.N * 8);
  L.eb = up(L.ea + (size_t)(d.Z * d.M) * 4);
  L.total = up(L.eb + (size_t)(d.Z * d.N) * 4) + 256;
  return L;
}

// The kernels keep the long side on M (the 128 TMEM lanes): a pair whose A
// side is the narrow one is run as C = B x A with the roles swapped.
GemmDesc swapped(const GemmDesc& d) {
  GemmDesc s = d;
  s.M = d.N;
  s.N = d.M;
  s.nm = d.nn;
  s.nn = d.nm;
  for (int i = 0; i < kMaxModes; ++i) {
    s.mdim[i] = d.ndim[i];
    s.msa[i] = d.nsb[i];
    s.msc[i] = d.nsc[i];
    s.ndim[i] = d.mdim[i];
    s.nsb[i] = d.msa[i];
    s.nsc[i] = d.msc[i];
    s.ksa[i] = d.ksb[i];
    s.ksb[i] = d.ksa[i];
    s.zsa[i] = d.zsb[i];
    s.zsb[i] = d.zsa[i];
  }
  return s;
}
bool needs_swap(const GemmDesc& d) { return d.M < 64 && d.N > d.M; }

template <typename T, int ROWS>
void prep_rows(const void* X, int side, __nv_bfloat16* planes, int* e, const GemmDesc& d, int64_t rtiles, int64_t kt,
               cudaStream_t s) {
  const int64_t rows = side == 0 ? d.M : d.N;
  k_oz_exp<T, ROWS><<<dim3((unsigned)rtiles, (unsigned)d.Z), 256, 0, s>>>((const T*)X, d, side, rows, e);
  k_oz_pack<T, ROWS><<<dim3((unsigned)kt, (unsigned)rtiles, (unsigned)d.Z), 256, 0, s>>>((const T*)X, planes, d, side,
                                                                                       rows, rtiles, kt, e);
}

template <typename T>
void prep_operand(const void* X, int side, int rows_per_tile, __nv_bfloat16* planes, int* e, const GemmDesc& d,
                  int64_t rtiles, int64_t kt, cudaStream_t s) {
  if (rows_per_tile == TM) prep_rows<T, TM>(X, side, planes, e, d, rtiles, kt, s);
  else if (rows_per_tile == 64) prep_rows<T, 64>(X, side, planes, e, d, rtiles, kt, s);
  else if (rows_per_tile == 32) prep_rows<T, 32>(X, side, planes, e, d, rtiles, kt, s);
  else prep_rows<T, 16>(X, side, planes, e, d, rtiles, kt, s);
}

template <typename TC, int TN>
cudaError_t oz_gemm_launch(const __nv_bfloat16* pa, const __nv_bfloat16* pb, void* C, const GemmDesc& d,
                           const int64_t* cm, const int64_t* cn, const int* ea, const int* eb, const OzLayout& L,
                           int* status, cudaStream_t s) {
  static_assert(sizeof(OzSmem<TN>) + 1024 <= 232448, "shared memory layout exceeds 227 KiB");
  const size_t smem = sizeof(OzSmem<TN>) + 1024;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_oz_gemm<TC, TN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const int64_t tiles = L.mt * L.nt * d.Z;
  const unsigned grid = (unsigned)std::min<int64_t>(tiles, sm_count());
  k_oz_gemm<TC, TN><<<grid, kThreads, smem, s>>>(pa, pb, (TC*)C, d, cm, cn, ea, eb, L.mt, L.nt, L.kt, status);
  return cudaGetLastError();
}

template <typename TC>
cudaError_t oz_gemm_tn(const __nv_bfloat16* pa, const __nv_bfloat16* pb, void* C, const GemmDesc& d,
                       const int64_t* cm, const int64_t* cn, const int* ea, const int* eb, const OzLayout& L,
                       int* status, cudaStream_t s) {
  if (L.tn == 64) return oz_gemm_launch<TC, 64>(pa, pb, C, d, cm, cn, ea, eb, L, status, s);
  if (L.tn == 32) return oz_gemm_launch<TC, 32>(pa, pb, C, d, cm, cn, ea, eb, L, status, s);
  return oz_gemm_launch<TC, 16>(pa, pb, C, d, cm, cn, ea, eb, L, status, s);
}

bool eligible_oriented(const GemmDesc& d) {
  if (d.M < 64 || d.N < 8 || d.K < 16 || d.K > kMaxK) return false;
  if (d.Z > 65535 || ceil_div(d.M, TM) > 65535 || ceil_div(d.N, oz_tile_n(d.N)) > 65535) return false;
  return layout(d).total <= (size_t(24) << 30);
}

}  // namespace

bool oz_eligible(const GemmDesc& d) { return eligible_oriented(needs_swap(d) ? swapped(d) : d); }

size_t oz_scratch_bytes(const GemmDesc& d) { return layout(needs_swap(d) ? swapped(d) : d).total; }

cudaError_t launch_oz(int ta, int tb, int tc, const void* A, const void* B, void* C, const GemmDesc& d0, void* scratch,
                      size_t scratch_bytes, int* status, cudaStream_t stream) {
  if (!oz_eligible(d0)) return cudaErrorNotSupported;
  const bool swap = needs_swap(d0);
  const GemmDesc d = swap ? swapped(d0) : d0;
  if (swap) {
    std::swap(A, B);
    std::swap(ta, tb);
  }
  const OzLayout L = layout(d);
  if (!scratch || scratch_bytes < L.total) return cudaErrorInvalidValue;
  char* base = (char*)(((uintptr_t)scratch + 255) & ~(uintptr_t)255);
  auto* pa = (__nv_bfloat16*)(base + L.pa);
  auto* pb = (__nv_bfloat16*)(base + L.pb);
  auto* cm = (int64_t*)(base + L.cm);
  auto* cn = (int64_t*)(base + L.cn);
  auto* ea = (int*)(base + L.ea);
  auto* eb = (int*)(base + L.eb);
  if (ta == PQ_C128)
    prep_operand<double2>(A, 0, TM, pa, ea, d, L.mt, L.kt, stream);
  else
    prep_operand<float2>(A, 0, TM, pa, ea, d, L.mt, L.kt, stream);
  if (tb == PQ_C128)
    prep_operand<double2>(B, 1, L.tn, pb, eb, d, L.nt, L.kt, stream);
  else
    prep_operand<float2>(B, 1, L.tn, pb, eb, d, L.nt, L.kt, stream);
  const int64_t idx_blocks = std::min<int64_t>(ceil_div(d.M + d.N, 256), 152 * 8);
  k_result_index<<<(unsigned)idx_blocks, 256, 0, stream>>>(d, cm, cn);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return tc == PQ_C128 ? oz_gemm_tn<double2>(pa, pb, C, d, cm, cn, ea, eb, L, status, stream)
                       : oz_gemm_tn<float2>(pa, pb, C, d, cm, cn, ea, eb, L, status, stream);
}

}  // namespace pq
