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
// Complex arithmetic on real tensor cores: a tile of 64 complex rows of A is
// held as the 192-row stack [Ar; Ai; -Ar] of each slice, so that
//   X1 = rows 0..127   = [Ar; Ai]
//   X2 = rows 64..191  = [Ai; -Ar]  (issued with the MMA's negate-A bit: [-Ai; Ar])
// and one accumulator of 128 TMEM lanes receives
//   X1 . Br + X2' . Bi = [Ar.Br - Ai.Bi ; Ai.Br + Ar.Bi] = [Cr ; Ci]
// for the 64 rows: 2 MMAs (M=128, N=TN, K=16) per slice pair and K tile.
//
// Kernels (one launch each, in stream order):
//   k_oz_exp        row scale exponents of A (k_oz_exp_k when A is contiguous
//                   along K), column scale exponents of B
//   k_oz_pack       B's slices into planes [z][col tile][k tile][plane][TN*16
//                   bf16] in the canonical no-swizzle K-major UMMA layout
//                   (8-row x 16-byte core matrices), planes {Re s0..s4, Im
//                   s0..s4}; columns and K beyond the operand are 0
//   k_result_index  result offsets of every row and column of C
//   k_oz_gemm       persistent, one CTA per SM over 64 x TN complex output
//                   tiles (TN = 128, or 64 / 32 / 16 for narrow pairs; a pair
//                   whose A side is the narrow one runs as B x A):
//     warp 0       producer: cp.async.bulk of B's 10 plane tiles of one
//                  16-deep K tile into the shared-memory ring;
//     warp 1       TMEM owner and MMA issuer: 30 tcgen05.mma (kind::f16,
//                  bf16) per K tile into three TN-column accumulators (levels
//                  0, 1, 2-4); narrow tiles (TN <= 64) alternate between two
//                  such sets, so a tile's MMAs do not wait for the epilogue
//                  of the one before; 16-wide tiles issue one MMA per A slice
//                  i against B's slices 0 .. 4-i side by side (N = 16 (5-i),
//                  10 MMAs per K tile), each slice pair into its own exact
//                  16-column region;
//     warps 2-9    A converters: gather A's 64 x 16 complex values of the K
//                  tile through its index map straight from HBM (the group's
//                  next K tile in flight while this one is sliced), slice
//                  them and store the [Ar; Ai; -Ar] stacks into the ring (no
//                  slice planes of A ever reach HBM); for complex64 A two
//                  groups of four warps take alternate K tiles, each thread
//                  8 consecutive k of one row, so every store is a whole
//                  16-byte core-matrix row;
//     warps 10-17  epilogue, once per tile: Cr from TMEM lanes 0-63, Ci from
//                  lanes 64-127; the levels are combined with an error-free
//                  two-sum, scaled by 2^(ea+eb) and scattered through the
//                  result index map.
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

constexpr int TK = 16;
constexpr int kThreads = 576;                    // producer, MMA, 8 converter + 8 epilogue warps
constexpr int kConvWarps = 8, kEpiWarps = 8;
constexpr int kRows = 64;                        // complex rows of A per tile
constexpr int kStackBytes = 3 * kRows * TK * 2;  // one slice's [Ar; Ai; -Ar] stack (6 KiB)
constexpr int kExpZero = -4096;                  // exponent of an all-zero row
constexpr int64_t kMaxK = 512;                   // exact level-0/1 sums up to this K

// Tile width N: 128 for general pairs, 64 / 32 / 16 for narrow ones.
// Slices per real value: 5 for PQ_PREC_OZAKI (15 slice pairs, i + j <= 4),
// 4 for PQ_PREC_OZAKI4 (10 pairs, i + j <= 3), 3 for PQ_PREC_3XBF16 (6
// pairs, i + j <= 2).
template <int NSL>
struct Sl {
  static_assert(NSL == 5 || NSL == 4 || NSL == 3, "slice count");
  static constexpr int planes = 2 * NSL;  // per operand: Re s0.., Im s0..
  static constexpr int pairs = NSL == 5 ? 15 : (NSL == 4 ? 10 : 6);
};

template <int TN, int NSL>
struct OzCfg {
  static constexpr int kBTile = TN * TK;                                   // bf16 per B plane tile
  static constexpr uint32_t b_bytes = Sl<NSL>::planes * kBTile * 2;        // B planes of one K tile
  static constexpr uint32_t stage_bytes = NSL * kStackBytes + b_bytes;
  static constexpr int stages = (TN == 128 && NSL >= 4) ? 3 : 4;
  // 16-wide tiles: one MMA per A slice i against B slices 0 .. NSL-1-i side
  // by side (N = 16 (NSL - i)), every slice pair in its own TMEM region
  static constexpr bool narrow = TN == 16;
  // accumulator columns of one tile: three levels of TN columns, or the
  // NSL (NSL + 1) / 2 pair regions of 16 columns
  static constexpr int set_cols = narrow ? 8 * NSL * (NSL + 1) : 3 * TN;
  // accumulator sets: two for TN <= 64, so that the MMAs of the next tile
  // run while the epilogue drains this one
  static constexpr int acc_sets = TN <= 64 ? 2 : 1;
  static constexpr uint32_t tmem_cols =
      TN == 128 ? 512 : (TN == 64 ? 512 : (TN == 32 ? 256 : (2 * set_cols > 256 ? 512 : 256)));
  static constexpr int cw = TN / 2;                                         // columns per epilogue warp
  static_assert(acc_sets * set_cols <= (int)tmem_cols && cw % 8 == 0 && stage_bytes % 1024 == 0, "tile width");
};

// First TMEM column of A slice i's region in a narrow tile: the regions of
// slices 0 .. i-1 hold NSL, NSL - 1, ... pair blocks of 16 columns.
template <int NSL>
__host__ __device__ constexpr int narrow_col(int i) {
  return 16 * (i * NSL - i * (i - 1) / 2);
}
// The slice pairs of level >= 2, smallest level first: the p-th is
// (rest_i, rest_level - rest_i); level l holds the l + 1 pairs i = 0 .. l.
template <int NSL>
__host__ __device__ constexpr int rest_level(int p) {
  int l = NSL - 1;
  while (p > l) {
    p -= l + 1;
    --l;
  }
  return l;
}
template <int NSL>
__host__ __device__ constexpr int rest_i(int p) {
  int l = NSL - 1;
  while (p > l) {
    p -= l + 1;
    --l;
  }
  return p;
}

// slice pairs, level 0 first, then level 1, then the higher levels (the
// inexact accumulator takes its small terms first).  Five slices:
//   i: 0 0 1 0 1 2 3 4 0 1 2 3 0 1 2
//   j: 0 1 0 4 3 2 1 0 3 2 1 0 2 1 0
// four slices (levels 0 to 3, ten pairs):
//   i: 0 0 1 0 1 2 3 0 1 2
//   j: 0 1 0 3 2 1 0 2 1 0
// three slices:
//   i: 0 0 1 0 1 2
//   j: 0 1 0 2 1 0
// (4-bit fields, pair p in bits [4p, 4p + 4))
template <int NSL>
__host__ __device__ constexpr int pair_i(int p) {
  return (int)((NSL == 5 ? 0x210321043210100ull : (NSL == 4 ? 0x2103210100ull : 0x210100ull)) >> (4 * p)) & 15;
}
template <int NSL>
__host__ __device__ constexpr int pair_j(int p) {
  return (int)((NSL == 5 ? 0x12012301234010ull : (NSL == 4 ? 0x0120123010ull : 0x12010ull)) >> (4 * p)) & 15;
}

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
// e[z * rows + r] = frexp exponent of the largest |Re|, |Im| over k.
// One block per (ROWS-row tile, z); thread t always reads row t % ROWS (K
// offsets staged in shared memory), keeps a running maximum with four loads
// in flight, and the 256 / ROWS threads of a row combine at the end.
template <typename T, int ROWS>
__global__ void __launch_bounds__(256) k_oz_exp(const T* __restrict__ X, const __grid_constant__ GemmDesc d, int side,
                                                int64_t rows, int* __restrict__ e_out) {
  static_assert(256 % ROWS == 0, "rows per block");
  constexpr int KS = 256 / ROWS;  // threads per row
  __shared__ int64_t koff[kMaxK];
  __shared__ int emax[ROWS];
  const int64_t rt = blockIdx.x, z = blockIdx.y;
  const int nrm = side == 0 ? d.nm : d.nn;
  const int64_t* rdim = side == 0 ? d.mdim : d.ndim;
  const int64_t* rstr = side == 0 ? d.msa : d.nsb;
  const int64_t* kstr = side == 0 ? d.ksa : d.ksb;
  const int64_t* zstr = side == 0 ? d.zsa : d.zsb;
  for (int t = threadIdx.x; t < ROWS; t += blockDim.x) emax[t] = kExpZero;
  for (int t = threadIdx.x; t < d.K; t += blockDim.x) koff[t] = decode(t, d.nk, d.kdim, kstr);
  __syncthreads();
  using R = typename Real<T>::R;
  const int r = threadIdx.x % ROWS, k0 = threadIdx.x / ROWS;
  const int64_t row = rt * ROWS + r;
  if (row < rows) {
    const T* xr = X + decode(z, d.nz, d.zdim, zstr) + decode(row, nrm, rdim, rstr);
    R mx = 0;
    int64_t k = k0;
    for (; k + 3 * KS < d.K; k += 4 * KS) {
      const T v0 = xr[koff[k]], v1 = xr[koff[k + KS]], v2 = xr[koff[k + 2 * KS]], v3 = xr[koff[k + 3 * KS]];
      mx = fmax(mx, fmax(fmax(absmax((R)v0.x, (R)v0.y), absmax((R)v1.x, (R)v1.y)),
                         fmax(absmax((R)v2.x, (R)v2.y), absmax((R)v3.x, (R)v3.y))));
    }
    for (; k < d.K; k += KS) {
      const T v = xr[koff[k]];
      mx = fmax(mx, absmax((R)v.x, (R)v.y));
    }
    atomicMax(&emax[r], exp_of(mx));
  }
  __syncthreads();
  for (int t = threadIdx.x; t < ROWS; t += blockDim.x) {
    const int64_t rr = rt * ROWS + t;
    if (rr < rows) e_out[z * rows + rr] = emax[t];
  }
}

// Row scale exponents of A when A is contiguous along K (its first K mode
// has stride 1 and extent >= 2) but not along M: KL consecutive lanes read
// consecutive k of one row (KL = the first K mode's extent, a power of two,
// at most 32), combine their maxima with shuffles, and the RS = 32 / KL row
// groups of a warp take consecutive rows -- when A's first M mode follows its
// first K mode in memory, every load of a warp is one contiguous 256-byte
// run.  A warp takes four such steps at a time, twice; one block of 8 warps
// per 64 RS rows and batch index z.
template <typename T>
__global__ void __launch_bounds__(256) k_oz_exp_k(const T* __restrict__ X, const __grid_constant__ GemmDesc d,
                                                  int64_t rows, int KL, int* __restrict__ e_out) {
  using R = typename Real<T>::R;
  __shared__ int64_t koff[kMaxK];
  const int64_t z = blockIdx.y;
  for (int t = threadIdx.x; t < d.K; t += blockDim.x) koff[t] = decode(t, d.nk, d.kdim, d.ksa);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int RS = 32 / KL;
  const int sub = lane / KL, kl = lane % KL;
  const int64_t zo = decode(z, d.nz, d.zdim, d.zsa);
  const int64_t r0 = (int64_t)blockIdx.x * 64 * RS + warp * 8 * RS;
#pragma unroll 1
  for (int rr = 0; rr < 8 * RS; rr += 4 * RS) {
    const T* xr[4];
    bool v[4];
    R mx[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int64_t row = r0 + rr + i * RS + sub;
      v[i] = row < rows;
      xr[i] = X + zo + (v[i] ? decode(row, d.nm, d.mdim, d.msa) : 0);
      mx[i] = 0;
    }
#pragma unroll 2
    for (int k = kl; k < d.K; k += KL) {
      const int64_t o = koff[k];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        if (v[i]) {
          const T x = xr[i][o];
          mx[i] = fmax(mx[i], absmax((R)x.x, (R)x.y));
        }
      }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      for (int s = KL / 2; s > 0; s >>= 1) mx[i] = fmax(mx[i], __shfl_xor_sync(0xffffffffu, mx[i], s));
      if (kl == 0 && v[i]) e_out[z * rows + r0 + rr + i * RS + sub] = exp_of(mx[i]);
    }
  }
}

// A's row exponents: the K-major kernel when A's first K mode has stride 1
// (and its first M mode does not), else the row-per-thread kernel.
template <typename T>
void row_exponents(const T* A, const GemmDesc& d, int* ea, cudaStream_t s) {
  int KL = 1;
  if (d.nk > 0 && d.ksa[0] == 1 && !(d.nm > 0 && d.msa[0] == 1))
    while (KL < 32 && 2 * KL <= d.kdim[0]) KL *= 2;
  if (KL >= 2) {
    const int64_t rows_per_block = 64 * (32 / KL);
    k_oz_exp_k<T><<<dim3((unsigned)ceil_div(d.M, rows_per_block), (unsigned)d.Z), 256, 0, s>>>(A, d, d.M, KL, ea);
  } else {
    k_oz_exp<T, 128><<<dim3((unsigned)ceil_div(d.M, 128), (unsigned)d.Z), 256, 0, s>>>(A, d, 0, d.M, ea);
  }
}

// The slices of x (|x| < 1 after scaling); every step is exact in R.
template <typename R, int NSL>
__device__ __forceinline__ void slices(R x, float* s) {
  R r = x;
  R g = (R)128.0, gi = (R)(1.0 / 128.0);  // 2^7(i+1) and its inverse (exact)
#pragma unroll
  for (int i = 0; i < NSL; ++i) {
    const R si = round_int(r * g) * gi;
    s[i] = (float)si;
    r -= si;
    g *= (R)128.0;
    gi *= (R)(1.0 / 128.0);
  }
}

// 2^k as a float for -126 <= k <= 127.
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((k + 127) << 23); }
// Two factors whose product is 2^-e (|e| <= 252), each a normal float: x 2^-e
// is (x f.x) f.y, exact unless the result underflows (far below any slice).
__device__ __forceinline__ float2 inv_scale(int e) {
  const int a = (-e) / 2;
  return make_float2(pow2f(a), pow2f(-e - a));
}
// x 2^-e: complex64 rows (|e| <= 149) by the two factors f, complex128 rows
// (any exponent) by ldexp.
__device__ __forceinline__ float scale_row(float x, int, float2 f) { return (x * f.x) * f.y; }
__device__ __forceinline__ double scale_row(double x, int e, float2) { return ldexp(x, -e); }

// One plane tile (ROWS x 16) is shared by PARTS blocks (blockIdx.x = kt PARTS
// + part), each slicing TILE / PARTS values: complex128 B is sliced in FP64,
// whose GB300 rate is low, so the work is spread over many SMs.
template <typename T, int ROWS, int NSL>
__host__ __device__ constexpr int pack_parts() {
  return ROWS * TK / 256 > 0 ? ROWS * TK / 256 : 1;
}
template <typename T, int ROWS, int NSL>
__global__ void __launch_bounds__(256) k_oz_pack(const T* __restrict__ X, __nv_bfloat16* __restrict__ planes,
                                                 const __grid_constant__ GemmDesc d, int side, int64_t rows,
                                                 int64_t rtiles, int64_t ktiles, const int* __restrict__ e_in) {
  constexpr int TILE = ROWS * TK, GROUPS = ROWS / 8, PARTS = pack_parts<T, ROWS, NSL>(), PER = TILE / PARTS;
  __shared__ int64_t roff[ROWS];
  __shared__ int rexp[ROWS];
  __shared__ int64_t koff[TK];
  const int64_t kt = blockIdx.x / PARTS, rt = blockIdx.y, z = blockIdx.z;
  const int part = (int)(blockIdx.x % PARTS);
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
  __nv_bfloat16* tile = planes + (((z * rtiles + rt) * ktiles + kt) * Sl<NSL>::planes) * (int64_t)TILE;
  for (int o = part * PER + threadIdx.x; o < (part + 1) * PER; o += blockDim.x) {
    // o = ((kc * GROUPS + g) * 8 + r8) * 8 + k8: core matrix (kc, g), row r8, K k8
    const int core = o >> 6, within = o & 63;
    const int kc = core / GROUPS, g = core - kc * GROUPS;
    const int r = g * 8 + (within >> 3), k = kc * 8 + (within & 7);
    float re[NSL], im[NSL];
#pragma unroll
    for (int i = 0; i < NSL; ++i) re[i] = im[i] = 0.f;
    if (roff[r] >= 0 && koff[k] >= 0 && rexp[r] != kExpZero) {
      const T v = X[zo + roff[r] + koff[k]];
      slices<R, NSL>(scale2((R)v.x, -rexp[r]), re);
      slices<R, NSL>(scale2((R)v.y, -rexp[r]), im);
    }
    if constexpr (ROWS == 16) {
      // 16-wide tiles: per part (Re, Im) one block of the NSL slices side by
      // side along N (slice i = rows 16 i .. 16 i + 15, row groups 2 i and
      // 2 i + 1), so that slices 0 .. m form one operand of 16 (m + 1) rows
      const int r8 = within >> 3, k8 = within & 7;
#pragma unroll
      for (int i = 0; i < NSL; ++i) {
        const int q = ((kc * (NSL * GROUPS) + i * GROUPS + g) * 8 + r8) * 8 + k8;
        tile[0 * NSL * TILE + q] = __float2bfloat16_rn(re[i]);
        tile[1 * NSL * TILE + q] = __float2bfloat16_rn(im[i]);
      }
    } else {
#pragma unroll
      for (int i = 0; i < NSL; ++i) {
        tile[(0 * NSL + i) * TILE + o] = __float2bfloat16_rn(re[i]);
        tile[(1 * NSL + i) * TILE + o] = __float2bfloat16_rn(im[i]);
      }
    }
  }
}

template <int TN, int NSL>
struct alignas(1024) OzSmem {
  unsigned char stage[OzCfg<TN, NSL>::stages][OzCfg<TN, NSL>::stage_bytes];  // A stacks, then B planes
  int64_t koff[kMaxK];                                                        // A's K offsets
  uint64_t full[OzCfg<TN, NSL>::stages];
  uint64_t empty[OzCfg<TN, NSL>::stages];
  uint64_t accf[2];  // accumulator set b holds a finished tile
  uint64_t acce[2];  // the epilogue has read accumulator set b
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
// (l0 + l1 + l2) rounded once (before scaling): l0 + l1 by an error-free
// two-sum, the small l2 added to its error term.
__device__ __forceinline__ float level_sum(float l0, float l1, float l2) {
  float e;
  const float s = two_sum(l0, l1, e);
  return s + (e + l2);
}
// x 2^ex with one rounding, the same value as ldexpf(x, ex): a multiply by an
// exact power of two when 2^ex is a normal float.
__device__ __forceinline__ float scale_pow2(float x, int ex) {
  return (ex >= -126 && ex <= 127) ? x * __int_as_float((ex + 127) << 23) : ldexpf(x, ex);
}
__device__ __forceinline__ float combine(float l0, float l1, float l2, int ex, float) {
  return scale_pow2(level_sum(l0, l1, l2), ex);
}
__device__ __forceinline__ double combine(float l0, float l1, float l2, int ex, double) {
  return ldexp(((double)l0 + (double)l1) + (double)l2, ex);
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // exact: slices have <= 8 bits
  return *reinterpret_cast<const uint32_t*>(&v);
}
__device__ __forceinline__ void sts64(uint32_t addr, uint32_t a, uint32_t b) {
  asm volatile("st.shared.v2.b32 [%0], {%1, %2};" ::"r"(addr), "r"(a), "r"(b) : "memory");
}
__device__ __forceinline__ void sts128(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}

// A values per converter thread and K tile: 8 for complex64 A (whole 16-byte
// core-matrix rows), 4 for complex128 A.
constexpr int kConvThreads = 32 * kConvWarps;
template <typename TA>
__host__ __device__ constexpr int conv_values() {
  return sizeof(TA) == 8 ? 8 : 4;
}
// Generic-proxy shared-memory writes made visible to the tensor core's reads.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

template <typename TA, typename TC, int TN, int NSL>
__global__ void __launch_bounds__(kThreads, 1)
    k_oz_gemm(const TA* __restrict__ A, const __nv_bfloat16* __restrict__ pb, TC* __restrict__ C,
              const __grid_constant__ GemmDesc d, const int64_t* __restrict__ cm_tab,
              const int64_t* __restrict__ cn_tab, const int* __restrict__ ea, const int* __restrict__ eb,
              int64_t mtiles, int64_t ntiles, int64_t ktiles, int* status) {
  using CF = OzCfg<TN, NSL>;
  constexpr int kSlices = NSL, kPlanes = Sl<NSL>::planes, kPairs = Sl<NSL>::pairs;
  constexpr int kStages = CF::stages;
  constexpr uint32_t kTmemCols = CF::tmem_cols;
  constexpr int kSets = CF::acc_sets;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  OzSmem<TN, NSL>& sm = *reinterpret_cast<OzSmem<TN, NSL>*>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ntot = ntiles * mtiles * d.Z;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      // producer's expect_tx + one arrival per warp of the converter group of the K tile
      mbar_init(&sm.full[s], 1 + kConvWarps * 4 / conv_values<TA>());
      mbar_init(&sm.empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&sm.accf[b], 1);
      mbar_init(&sm.acce[b], kEpiWarps);  // one arrival per epilogue warp
    }
    mbar_init(&sm.drain, 1);
    mbar_init_fence();
  }
  for (int t = threadIdx.x; t < d.K; t += blockDim.x) sm.koff[t] = decode(t, d.nk, d.kdim, d.ksa);
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
        const int64_t nt = tile % ntiles, z = tile / (ntiles * mtiles);
        const __nv_bfloat16* btile = pb + ((z * ntiles + nt) * ktiles) * (int64_t)(kPlanes * CF::kBTile);
        for (int64_t kt = 0; kt < ktiles; ++kt, ++g) {
          const int s = (int)(g % kStages);
          const uint32_t ph = (uint32_t)((g / kStages) & 1);
          if (!mbar_wait(&sm.empty[s], ph ^ 1)) {
            ok = false;
            break;
          }
          mbar_expect_tx(&sm.full[s], CF::b_bytes);
          bulk_g2s(sm.stage[s] + kSlices * kStackBytes, btile + kt * (kPlanes * CF::kBTile), CF::b_bytes,
                   &sm.full[s]);
        }
      }
      // the copies of the last stages are in flight until their full barrier
      // completes: wait (bounded) so none lands after the CTA has exited
      for (int64_t i = g - 1; i >= 0 && i >= g - kStages; --i)
        if (!mbar_wait(&sm.full[i % kStages], (uint32_t)((i / kStages) & 1))) ok = false;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_bf16(128, TN), idesc_neg = idesc_bf16(128, TN, true);
      constexpr uint32_t ALBO = 24 * 128, BLBO = (TN / 8) * 128, SBO = 128;
      int64_t g = 0;  // K tiles consumed so far
      int64_t t = 0;  // tiles of this CTA
      for (int64_t tile = blockIdx.x; tile < ntot && ok; tile += gridDim.x, ++t) {
        // the epilogue has read this accumulator set's previous tile
        const int b = (int)(t % kSets);
        if (!mbar_wait(&sm.acce[b], (uint32_t)(((t / kSets) & 1) ^ 1))) {
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
          if constexpr (CF::narrow) {
            // B block per part: NSL slices x 2 row groups per K half
            const uint64_t bn = smem_desc(sa + kSlices * kStackBytes, NSL * 2 * 128, SBO);
#pragma unroll
            for (int i = 0; i < NSL; ++i) {
              const uint32_t dl = tmem + (uint32_t)(b * CF::set_cols + narrow_col<NSL>(i));
              const uint64_t x1 = a0 + (uint64_t)((i * kStackBytes) >> 4);            // [Ar; Ai]
              const uint64_t x2 = a0 + (uint64_t)((i * kStackBytes + 8 * 128) >> 4);  // [Ai; -Ar]
              const uint64_t bi = bn + (uint64_t)((NSL * CF::kBTile * 2) >> 4);       // the Im block
              const uint32_t acc = kt == 0 ? 0u : 1u;
              mma_bf16(dl, x1, bn, idesc_bf16(128, 16 * (NSL - i)), acc);   // [Ar.Br ; Ai.Br], slices 0..NSL-1-i
              mma_bf16(dl, x2, bi, idesc_bf16(128, 16 * (NSL - i), true), 1u);
            }
            mma_commit(&sm.empty[s]);
            continue;
          }
          const uint64_t b0 = smem_desc(sa + kSlices * kStackBytes, BLBO, SBO);
#pragma unroll
          for (int p = 0; p < kPairs; ++p) {
            const int i = pair_i<NSL>(p), j = pair_j<NSL>(p);
            const uint32_t acc = (kt == 0 && first_of_level(p)) ? 0u : 1u;
            const uint32_t dl = tmem + (uint32_t)((b * 3 + level_of(p)) * TN);
            const uint64_t x1 = a0 + (uint64_t)((i * kStackBytes) >> 4);             // [Ar; Ai]
            const uint64_t x2 = a0 + (uint64_t)((i * kStackBytes + 8 * 128) >> 4);   // [Ai; -Ar]
            const uint64_t br = b0 + (uint64_t)(((0 * kSlices + j) * CF::kBTile * 2) >> 4);
            const uint64_t bi = b0 + (uint64_t)(((1 * kSlices + j) * CF::kBTile * 2) >> 4);
            mma_bf16(dl, x1, br, idesc, acc);     // [Ar.Br ; Ai.Br]
            mma_bf16(dl, x2, bi, idesc_neg, 1u);  // [-Ai.Bi ; Ar.Bi]
          }
          mma_commit(&sm.empty[s]);  // smem stage free once these MMAs finish
        }
        if (!ok) break;
        mma_commit(&sm.accf[b]);  // tile accumulators ready for the epilogue
      }
      // every MMA issued has finished once this arrives (TMEM is freed below)
      mma_commit(&sm.drain);
      if (!mbar_wait(&sm.drain, 0)) ok = false;
    }
  } else if (warp < 2 + kConvWarps) {
    // converters: with NV values per thread and K tile, the converter warps
    // form NV / 4 groups that take alternate K tiles; thread ch of a group
    // handles row r = ch % 64 and the NV consecutive K values from
    // kq = (ch / 64) NV of its K tiles.  Complex64 A: NV = 8, a whole 16-byte
    // core-matrix row per stack block, stored without bank conflicts;
    // complex128 A: NV = 4 (half rows; fewer registers), one group.
    constexpr int NV = conv_values<TA>(), H = NV / 4, GT = kConvThreads / H;
    const int c = threadIdx.x - 64;
    const int grp = c / GT, ch = c % GT;
    const int r = ch & (kRows - 1), kq = (ch >> 6) * NV;
    using R = typename Real<TA>::R;
    // byte offset of (slice 0, block 0, row r, K value kq) in the stacks
    const uint32_t row_off = (uint32_t)((((kq >> 3) * 24 + (r >> 3)) * 8 + (r & 7)) * 16 + (kq & 7) * 2);
    // This CTA's K tiles form one sequence g = tile number * ktiles + kt; the
    // group takes g = grp, grp + H, ...  The next one's A values and row
    // exponent are loaded while this one is sliced, across tile boundaries
    // (a tile's rows and exponent are looked up once per tile).
    const int64_t ntl = blockIdx.x < ntot ? (ntot - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const int64_t items = ntl * ktiles;
    int64_t ptl = -1;  // tile (number within this CTA) whose row pointer and exponent are cached
    const TA* prow = A;
    bool pm = false;
    int en = kExpZero;  // exponent of the prefetched K tile's row (a load in flight)
    auto row_info = [&](int64_t tl) {
      const int64_t tile = blockIdx.x + tl * gridDim.x;
      const int64_t rr = tile / ntiles, mt = rr % mtiles, z = rr / mtiles;
      const int64_t m = mt * kRows + r;
      pm = m < d.M;
      en = pm ? ea[z * d.M + m] : kExpZero;
      prow = A + (pm ? decode(z, d.nz, d.zdim, d.zsa) + decode(m, d.nm, d.mdim, d.msa) : 0);
      ptl = tl;
    };
    // zeros past the operand (and for rows outside it); an all-zero row's
    // values are zeros themselves, whatever its exponent
    auto load = [&](int64_t kt, TA* v) {
#pragma unroll
      for (int q = 0; q < NV; ++q) {
        const int64_t k = kt * TK + kq + q;
        if (pm && k < d.K) {
          v[q] = prow[sm.koff[k]];
        } else {
          v[q].x = 0;
          v[q].y = 0;
        }
      }
    };
    TA nxt[NV];
    if (grp < items) {
      row_info(grp / ktiles);
      load(grp % ktiles, nxt);
    }
    for (int64_t gk = grp; gk < items && ok; gk += H) {
      const int e = en;
      TA cur[NV];
#pragma unroll
      for (int q = 0; q < NV; ++q) cur[q] = nxt[q];
      if (gk + H < items) {  // in flight while this K tile is sliced
        const int64_t gp = gk + H, tl = gp / ktiles;
        if (tl != ptl) row_info(tl);
        load(gp - tl * ktiles, nxt);
      }
      const float2 f = inv_scale(e != kExpZero ? e : 0);
      {
        const int s = (int)(gk % kStages);
        const uint32_t ph = (uint32_t)((gk / kStages) & 1);
        uint32_t pr[kSlices][NV / 2], pim[kSlices][NV / 2];  // bf16 pairs (k, k + 1) of Ar, Ai
#pragma unroll
        for (int q = 0; q < NV; q += 2) {
          float a0[kSlices], b0[kSlices], a1[kSlices], b1[kSlices];
          slices<R, NSL>(scale_row((R)cur[q].x, e, f), a0);
          slices<R, NSL>(scale_row((R)cur[q].y, e, f), b0);
          slices<R, NSL>(scale_row((R)cur[q + 1].x, e, f), a1);
          slices<R, NSL>(scale_row((R)cur[q + 1].y, e, f), b1);
#pragma unroll
          for (int i = 0; i < kSlices; ++i) {
            pr[i][q / 2] = pack_bf16x2(a0[i], a1[i]);
            pim[i][q / 2] = pack_bf16x2(b0[i], b1[i]);
          }
        }
        bool got = mbar_wait(&sm.empty[s], ph ^ 1);
        got = __all_sync(0xffffffffu, got);
        if (!got) {
          ok = false;
          break;
        }
        const uint32_t base = smem_u32(sm.stage[s]) + row_off;
#pragma unroll
        for (int i = 0; i < kSlices; ++i) {
          const uint32_t slice = base + (uint32_t)(i * kStackBytes);
          constexpr uint32_t kNeg = 0x80008000u;
          if constexpr (NV == 8) {
            sts128(slice, pr[i][0], pr[i][1], pr[i][2], pr[i][3]);                              // Ar
            sts128(slice + 8 * 128, pim[i][0], pim[i][1], pim[i][2], pim[i][3]);                // Ai
            sts128(slice + 16 * 128, pr[i][0] ^ kNeg, pr[i][1] ^ kNeg, pr[i][2] ^ kNeg, pr[i][3] ^ kNeg);  // -Ar
          } else {
            sts64(slice, pr[i][0], pr[i][1]);                        // Ar
            sts64(slice + 8 * 128, pim[i][0], pim[i][1]);            // Ai
            sts64(slice + 16 * 128, pr[i][0] ^ kNeg, pr[i][1] ^ kNeg);  // -Ar
          }
        }
        fence_proxy_async();
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.full[s]);
      }
    }
  } else {
    // epilogue: warp w reads TMEM lanes of quadrant w % 4 (0, 1: Cr of rows
    // 0..63; 2, 3: Ci), columns [h TN/2, (h+1) TN/2)
    constexpr int CW = CF::cw;
    const int q = warp & 3, h = (warp - 2 - kConvWarps) >> 2;
    const int part = q >> 1;               // 0: real parts, 1: imaginary parts
    const int r = (q & 1) * 32 + lane;     // complex row within the tile
    const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
    using R = typename std::conditional<std::is_same<TC, double2>::value, double, float>::type;
    R* Cr = reinterpret_cast<R*>(C);
    constexpr int PW = CW >= 16 ? 16 : 8;   // columns per TMEM load
    // One accumulator set and complex64 results: the combined levels are
    // parked in the unused fourth TMEM block so that the accumulators are
    // released before the scaling and the scattered stores.
    constexpr bool kStash = kSets == 1 && std::is_same<TC, float2>::value && 4 * TN <= (int)kTmemCols &&
                            CW % 16 == 0;
    constexpr int NU = (CW + 31) / 32;       // columns of the warp's range per lane
    // per-tile offsets and scales, loaded one tile ahead: the row's from
    // this lane, the warp's columns spread over the lanes
    struct Meta {
      int64_t base, c0;
      int exa;
      bool mrow;
      int ebl[NU];
      long long cnl[NU];
    };
    auto meta = [&](int64_t tile, Meta& M) {
      const int64_t nt = tile % ntiles, rr = tile / ntiles, mt = rr % mtiles, z = rr / mtiles;
      const int64_t m = mt * kRows + r;
      M.mrow = m < d.M;
      M.base = M.mrow ? decode(z, d.nz, d.zdim, d.zsc) + cm_tab[m] : 0;
      M.exa = M.mrow ? ea[z * d.M + m] : kExpZero;
      M.c0 = nt * TN + h * CW;
#pragma unroll
      for (int u = 0; u < NU; ++u) {
        const int64_t col = M.c0 + lane + 32 * u;
        const bool valid = lane + 32 * u < CW && col < d.N;
        M.ebl[u] = valid ? eb[z * d.N + col] : kExpZero;
        M.cnl[u] = valid ? (long long)cn_tab[col] : 0;
      }
    };
    Meta nm;
    if (blockIdx.x < ntot) meta(blockIdx.x, nm);
    int64_t t = 0;
    for (int64_t tile = blockIdx.x; tile < ntot && ok; tile += gridDim.x, ++t) {
      const Meta M = nm;
      if (tile + gridDim.x < ntot) meta(tile + gridDim.x, nm);  // in flight during this tile
      const bool mrow = M.mrow;
      const int64_t base = M.base, c0 = M.c0;
      const int exa = M.exa;
      const int b = (int)(t % kSets);
      bool got = mbar_wait(&sm.accf[b], (uint32_t)((t / kSets) & 1));
      got = __all_sync(0xffffffffu, got);  // the TMEM loads below are warp-collective
      if (!got) {
        ok = false;
        break;
      }
      fence_after();
      if constexpr (kStash) {
        // Phase 1 (holds the accumulators): the three levels of each element
        // summed into one float, parked in the spare TMEM block (columns
        // 3 TN .. 4 TN, the same lanes); then the accumulators are released.
#pragma unroll
        for (int piece = 0; piece < CW / 16; ++piece) {
          __syncwarp();
          const uint32_t col = (uint32_t)(h * CW + piece * 16);
          float l0[16], l1[16], l2[16];
          tmem_ld16(lane_base + col + 0 * TN, l0);
          tmem_ld16(lane_base + col + 1 * TN, l1);
          tmem_ld16(lane_base + col + 2 * TN, l2);
          tmem_wait_ld();
#pragma unroll
          for (int j = 0; j < 16; ++j) l0[j] = level_sum(l0[j], l1[j], l2[j]);
          tmem_st16(lane_base + 3 * TN + col, l0);
        }
        tmem_wait_st();
        fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.acce[b]);
        // Phase 2 (overlaps the next tile's MMAs): scale by 2^(ea + eb) and
        // scatter through the result index map.
#pragma unroll
        for (int piece = 0; piece < CW / 16; ++piece) {
          __syncwarp();
          float v[16];
          tmem_ld16(lane_base + 3 * TN + (uint32_t)(h * CW + piece * 16), v);
          tmem_wait_ld();
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int cc = piece * 16 + j;
            const int ebj = __shfl_sync(0xffffffffu, M.ebl[cc / 32], cc % 32);
            const long long cnj = __shfl_sync(0xffffffffu, M.cnl[cc / 32], cc % 32);
            if (mrow && c0 + cc < d.N) {
              const int ex = exa + ebj;
              const R val = (exa == kExpZero || ex < -2 * 1100) ? (R)0 : (R)scale_pow2(v[j], ex);
              Cr[2 * (base + cnj) + part] = val;
            }
          }
        }
        continue;
      }
#pragma unroll
      for (int piece = 0; piece < CW / PW; ++piece) {
        __syncwarp();  // the TMEM loads are warp-collective
        const uint32_t col = (uint32_t)(b * 3 * TN + h * CW + piece * PW);
        float l0[PW], l1[PW], l2[PW];
        if constexpr (CF::narrow) {
          // the slice-pair regions (each an exact sum over K): level 0 =
          // (0,0); level 1 = (0,1) + (1,0), exact; levels 2 .. NSL-1 summed
          // in FP32, the smallest first, four regions per TMEM wait
          static_assert(PW == 8, "narrow tiles: 8 columns per epilogue warp");
          const uint32_t rb = lane_base + (uint32_t)(b * CF::set_cols + h * CW + piece * PW);
          float t0[PW], t1[PW];
          tmem_ld8(rb + narrow_col<NSL>(0), l0);
          tmem_ld8(rb + narrow_col<NSL>(0) + 16, t0);
          tmem_ld8(rb + narrow_col<NSL>(1), t1);
          tmem_wait_ld();
#pragma unroll
          for (int q = 0; q < PW; ++q) {
            l1[q] = t0[q] + t1[q];
            l2[q] = 0.f;
          }
          constexpr int NR = NSL * (NSL + 1) / 2 - 3;
#pragma unroll
          for (int p0 = 0; p0 < NR; p0 += 4) {
            float tb[4][PW];
#pragma unroll
            for (int u = 0; u < 4; ++u)
              if (p0 + u < NR)
                tmem_ld8(rb + narrow_col<NSL>(rest_i<NSL>(p0 + u)) +
                             16 * (rest_level<NSL>(p0 + u) - rest_i<NSL>(p0 + u)),
                         tb[u]);
            tmem_wait_ld();
#pragma unroll
            for (int u = 0; u < 4; ++u)
              if (p0 + u < NR)
#pragma unroll
                for (int q = 0; q < PW; ++q) l2[q] += tb[u][q];
          }
        } else if constexpr (PW == 16) {
          tmem_ld16(lane_base + col + 0 * TN, l0);
          tmem_ld16(lane_base + col + 1 * TN, l1);
          tmem_ld16(lane_base + col + 2 * TN, l2);
        } else {
          tmem_ld8(lane_base + col + 0 * TN, l0);
          tmem_ld8(lane_base + col + 1 * TN, l1);
          tmem_ld8(lane_base + col + 2 * TN, l2);
        }
        tmem_wait_ld();
        if (piece == CW / PW - 1) {  // every value of this tile is in registers
          fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&sm.acce[b]);
        }
#pragma unroll
        for (int j = 0; j < PW; ++j) {
          const int cc = piece * PW + j;  // column within the warp's range
          const int ebj = __shfl_sync(0xffffffffu, M.ebl[cc / 32], cc % 32);
          const long long cnj = __shfl_sync(0xffffffffu, M.cnl[cc / 32], cc % 32);
          if (mrow && c0 + cc < d.N) {
            const int ex = exa + ebj;
            const R v = (exa == kExpZero || ex < -2 * 1100) ? (R)0 : combine(l0[j], l1[j], l2[j], ex, R());
            Cr[2 * (base + cnj) + part] = v;
          }
        }
      }
    }
  }
  if (!ok) report_timeout(status);
  fence_before();
  __syncthreads();
  if (warp == 1) {
    fence_after();
    tmem_dealloc(tmem, kTmemCols);
  }
}

int oz_tile_n(int64_t n) { return n <= 16 ? 16 : (n <= 32 ? 32 : (n <= 64 ? 64 : 128)); }
// Tile width of an oriented pair: the autotuner's choice when it set one,
// else the narrowest tile that covers N (at most 128).
int oz_tile_of(const GemmDesc& d) {
  return (d.tile_n == 16 || d.tile_n == 32 || d.tile_n == 64 || d.tile_n == 128) ? d.tile_n : oz_tile_n(d.N);
}

struct OzLayout {
  int tn;
  int64_t mt, nt, kt;
  size_t pb, cm, cn, ea, eb, total;  // byte offsets from the aligned base
};

OzLayout layout(const GemmDesc& d, int nsl) {
  OzLayout L;
  L.tn = oz_tile_of(d);
  L.mt = ceil_div(d.M, kRows);
  L.nt = ceil_div(d.N, L.tn);
  L.kt = ceil_div(d.K, TK);
  auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  L.pb = 0;
  L.cm = up(L.pb + (size_t)(d.Z * L.nt * L.kt) * (2 * nsl) * (L.tn * TK) * 2);
  L.cn = up(L.cm + (size_t)d.M * 8);
  L.ea = up(L.cn + (size_t)d.N * 8);
  L.eb = up(L.ea + (size_t)(d.Z * d.M) * 4);
  L.total = up(L.eb + (size_t)(d.Z * d.N) * 4) + 256;
  return L;
}

// The kernels keep the long side on M (the TMEM lanes): a pair whose A side
// is the narrow one is run as C = B x A with the roles swapped.
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
// Orientation: the autotuner's choice (orient 1 = as given, 2 = swapped) when
// it set one, else swap when A is the narrow side.
bool needs_swap(const GemmDesc& d) {
  if (d.orient == 1) return false;
  if (d.orient == 2) return true;
  return d.M < 64 && d.N > d.M;
}

// B's column exponents (16 columns per block, 16 threads on each: B is the
// small side, so its pass needs many blocks to be short), then its slices.
template <typename T, int ROWS, int NSL>
void prep_b(const void* X, __nv_bfloat16* planes, int* e, const GemmDesc& d, int64_t rtiles, int64_t kt,
            cudaStream_t s) {
  k_oz_exp<T, 16><<<dim3((unsigned)ceil_div(d.N, 16), (unsigned)d.Z), 256, 0, s>>>((const T*)X, d, 1, d.N, e);
  constexpr int parts = pack_parts<T, ROWS, NSL>();
  k_oz_pack<T, ROWS, NSL><<<dim3((unsigned)(kt * parts), (unsigned)rtiles, (unsigned)d.Z), 256, 0, s>>>(
      (const T*)X, planes, d, 1, d.N, rtiles, kt, e);
}

template <typename T, int NSL>
void prep_b_tn(const void* X, int tn, __nv_bfloat16* planes, int* e, const GemmDesc& d, int64_t rtiles, int64_t kt,
               cudaStream_t s) {
  if (tn == 128) prep_b<T, 128, NSL>(X, planes, e, d, rtiles, kt, s);
  else if (tn == 64) prep_b<T, 64, NSL>(X, planes, e, d, rtiles, kt, s);
  else if (tn == 32) prep_b<T, 32, NSL>(X, planes, e, d, rtiles, kt, s);
  else prep_b<T, 16, NSL>(X, planes, e, d, rtiles, kt, s);
}

template <typename TA, typename TC, int TN, int NSL>
cudaError_t oz_gemm_launch(const void* A, const __nv_bfloat16* pb, void* C, const GemmDesc& d, const int64_t* cm,
                           const int64_t* cn, const int* ea, const int* eb, const OzLayout& L, int* status,
                           cudaStream_t s) {
  static_assert(sizeof(OzSmem<TN, NSL>) + 1024 <= 232448, "shared memory layout exceeds 227 KiB");
  const size_t smem = sizeof(OzSmem<TN, NSL>) + 1024;
  static bool attr = false;
  if (!attr) {
    cudaError_t e =
        cudaFuncSetAttribute(k_oz_gemm<TA, TC, TN, NSL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const int64_t tiles = L.mt * L.nt * d.Z;
  const unsigned grid = (unsigned)std::min<int64_t>(tiles, sm_count());
  k_oz_gemm<TA, TC, TN, NSL><<<grid, kThreads, smem, s>>>((const TA*)A, pb, (TC*)C, d, cm, cn, ea, eb, L.mt, L.nt, L.kt,
                                                     status);
  return cudaGetLastError();
}

template <typename TA, typename TC, int NSL>
cudaError_t oz_gemm_tn(const void* A, const __nv_bfloat16* pb, void* C, const GemmDesc& d, const int64_t* cm,
                       const int64_t* cn, const int* ea, const int* eb, const OzLayout& L, int* status,
                       cudaStream_t s) {
  if (L.tn == 128) return oz_gemm_launch<TA, TC, 128, NSL>(A, pb, C, d, cm, cn, ea, eb, L, status, s);
  if (L.tn == 64) return oz_gemm_launch<TA, TC, 64, NSL>(A, pb, C, d, cm, cn, ea, eb, L, status, s);
  if (L.tn == 32) return oz_gemm_launch<TA, TC, 32, NSL>(A, pb, C, d, cm, cn, ea, eb, L, status, s);
  return oz_gemm_launch<TA, TC, 16, NSL>(A, pb, C, d, cm, cn, ea, eb, L, status, s);
}

bool eligible_oriented(const GemmDesc& d) {
  if (d.M < 64 || d.N < 8 || d.K < 16 || d.K > kMaxK) return false;
  // fewer than 512 complex products per output (e.g. a tall operand absorbing
  // a 16-column gate tensor over K = 16): memory-bound work whose per-tile
  // costs here exceed a plain FP32 pass, and whose FP32 sums have <= 32 terms
  if (d.N * d.K < 512) return false;
  if (d.Z > 65535 || ceil_div(d.N, oz_tile_of(d)) > 65535) return false;  // grid y / z of the B passes
  return layout(d, 5).total <= (size_t(24) << 30);
}

}  // namespace

bool oz_eligible(const GemmDesc& d) { return eligible_oriented(needs_swap(d) ? swapped(d) : d); }

size_t oz_scratch_bytes(int slices, const GemmDesc& d) { return layout(needs_swap(d) ? swapped(d) : d, slices).total; }

template <int NSL>
static cudaError_t launch_oz_n(int ta, int tb, int tc, const void* A, const void* B, void* C, const GemmDesc& d,
                               char* base, const OzLayout& L, int* status, cudaStream_t stream) {
  auto* pb = (__nv_bfloat16*)(base + L.pb);
  auto* cm = (int64_t*)(base + L.cm);
  auto* cn = (int64_t*)(base + L.cn);
  auto* ea = (int*)(base + L.ea);
  auto* eb = (int*)(base + L.eb);
  if (ta == PQ_C128)
    row_exponents((const double2*)A, d, ea, stream);
  else
    row_exponents((const float2*)A, d, ea, stream);
  if (tb == PQ_C128)
    prep_b_tn<double2, NSL>(B, L.tn, pb, eb, d, L.nt, L.kt, stream);
  else
    prep_b_tn<float2, NSL>(B, L.tn, pb, eb, d, L.nt, L.kt, stream);
  const int64_t idx_blocks = std::min<int64_t>(ceil_div(d.M + d.N, 256), 152 * 8);
  k_result_index<<<(unsigned)idx_blocks, 256, 0, stream>>>(d, cm, cn);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (ta == PQ_C128)
    return tc == PQ_C128 ? oz_gemm_tn<double2, double2, NSL>(A, pb, C, d, cm, cn, ea, eb, L, status, stream)
                         : oz_gemm_tn<double2, float2, NSL>(A, pb, C, d, cm, cn, ea, eb, L, status, stream);
  return tc == PQ_C128 ? oz_gemm_tn<float2, double2, NSL>(A, pb, C, d, cm, cn, ea, eb, L, status, stream)
                       : oz_gemm_tn<float2, float2, NSL>(A, pb, C, d, cm, cn, ea, eb, L, status, stream);
}

cudaError_t launch_oz(int slices, int ta, int tb, int tc, const void* A, const void* B, void* C,
                      const GemmDesc& d0, void* scratch, size_t scratch_bytes, int* status, cudaStream_t stream) {
  if (!oz_eligible(d0) || (slices != 5 && slices != 4 && slices != 3)) return cudaErrorNotSupported;
  const bool swap = needs_swap(d0);
  const GemmDesc d = swap ? swapped(d0) : d0;
  if (swap) {
    std::swap(A, B);
    std::swap(ta, tb);
  }
  const OzLayout L = layout(d, slices);
  if (!scratch || scratch_bytes < L.total) return cudaErrorInvalidValue;
  char* base = (char*)(((uintptr_t)scratch + 255) & ~(uintptr_t)255);
  if (slices == 5) return launch_oz_n<5>(ta, tb, tc, A, B, C, d, base, L, status, stream);
  if (slices == 4) return launch_oz_n<4>(ta, tb, tc, A, B, C, d, base, L, status, stream);
  return launch_oz_n<3>(ta, tb, tc, A, B, C, d, base, L, status, stream);
}

}  // namespace pq
