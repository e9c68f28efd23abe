// Split-precision complex contraction on the 5th-generation tensor cores
// (tcgen05, sm_103a): TF32 split products, FP32 accumulation in TMEM over
// 16-deep K chunks, chunk sums folded into Kahan-compensated FP32 registers.
//
//   C = A x B (complex), two real accumulators per output tile
//     Cr = Ar.Br + (-Ai).Bi   (the negation is the MMA's negate-A bit)
//     Ci = Ar.Bi + Ai.Br
//   Every real value is split into NS TF32 terms x = x0 + x1 (+ x2), each the
//   round-to-nearest TF32 value of the remainder, and a real product is the
//   sum of the term products with i + j < NS:
//     NS = 2 (PQ_PREC_3XTF32): x0y0 + x0y1 + x1y0                (3 products)
//     NS = 3 (PQ_PREC_6XTF32): x0y0 + x0y1 + x1y0 + x0y2 + x2y0 + x1y1  (6)
//
// k_tc_pack gathers an operand through its index map (any mode order, batch
// modes) into 2*NS planes {re terms, im terms} laid out tile by tile; a tile is
// ROWS (128 for A, 48 for B) x 16 K values in the canonical no-swizzle
// K-major UMMA layout: 8-row x 16-byte core matrices (128 contiguous bytes),
// row-adjacent core matrices 128 bytes apart, K-adjacent ones ROWS*16 bytes
// apart.  One bulk copy moves one plane tile.  Rows and K beyond the operand
// are zero.
//
// k_tc_gemm: one CTA per 128 x 48 output tile (x batch), 14 warps.
//   warp 0   producer: cp.async.bulk of the 4*NS plane tiles of one 16-deep K
//            tile into a shared-memory ring (mbarrier complete_tx);
//   warp 1   allocates TMEM and issues tcgen05.mma (M=128, N=48, K=8); every
//            16-deep K tile is one chunk, rotating over four sets of two
//            48-column FP32 accumulators, committed to the epilogue per chunk;
//   warps 2-13 epilogue: warp w reads TMEM lanes 32*(w%4).. and 16 of the 48
//            columns, folds each chunk's (Cr, Ci) into Kahan sums, hands the
//            accumulator set back, and finally scatters C through the result
//            index map.
// The tensor core rounds accumulations toward zero.  The small correction
// products of a chunk go in first, the hi x hi products last, so each chunk
// takes its few truncations at (partial) full magnitude; chunks are summed
// with compensation, which keeps the bias from growing with K, and the
// expected shrinkage of those truncations is added back in the final store.
// Every mbarrier wait is bounded; on expiry the kernel records an error in the
// context's status word and runs to the end (TMEM is always released), so the
// host sees PQ_ERR_DEVICE, not a hang.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "pq_tcgen05.cuh"
#include "pq_types.cuh"

namespace pq {

namespace {

using namespace tcg;

constexpr int TM = 128, TN = 48, TK = 16;
constexpr int kThreads = 448;                  // producer, MMA, 12 epilogue warps
constexpr int kEpiWarps = 12;
constexpr int kSets = 4;                       // TMEM accumulator sets in rotation
constexpr uint32_t kTmemCols = 512;            // 4 sets x 2 accumulators x 48 columns = 384 used
// Expected relative shrinkage of a value truncated (rounded toward zero) to
// FP32: half an ulp over a log-uniform mantissa, 2^-24 * ln 2 ...
constexpr float kTruncUnit = 4.13145e-8f;
// ... times the effective number of full-magnitude truncations per chunk: the
// four hi x hi additions into an accumulator land on partial sums of about
// 1/4, 1/2, 3/4 and all of the chunk value (random-sign terms), 2.5 in all;
// measured on random complex operands the shrinkage is 2.2 units (the
// partial sums' mantissas are not log-uniform).
constexpr float kTruncBias = 2.2f * kTruncUnit;
constexpr int kATile = TM * TK;                // floats per A plane tile (8 KiB)
constexpr int kBTile = TN * TK;                // floats per B plane tile (3 KiB)

template <int NS>
struct Cfg {
  static constexpr int planes = 2 * NS;                                  // per operand
  static constexpr uint32_t stage_bytes = planes * (kATile + kBTile) * 4;
  static constexpr int stages = NS == 2 ? 5 : 3;
  static constexpr int products = NS == 2 ? 3 : 6;
};

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

template <int NS>
__device__ __forceinline__ void split(float x, float* t) {
  t[0] = tf32_rna(x);
  float r = x - t[0];
  t[1] = tf32_rna(r);
  if (NS == 3) t[2] = tf32_rna(r - t[1]);
}
template <int NS>
__device__ __forceinline__ void split(double x, float* t) {
  t[0] = tf32_rna((float)x);
  double r = x - (double)t[0];
  t[1] = tf32_rna((float)r);
  if (NS == 3) t[2] = tf32_rna((float)(r - (double)t[1]));
}

// Pack operand X (side 0: A with m modes, side 1: B with n modes) into planes
// laid out [z][row tile][k tile][plane][ROWS*16 floats].
template <typename T, int NS, int ROWS>
__global__ void __launch_bounds__(256) k_tc_pack(const T* __restrict__ X, float* __restrict__ planes,
                                                 const __grid_constant__ GemmDesc d, int side, int64_t rows,
                                                 int64_t rtiles, int64_t ktiles) {
  constexpr int TILE = ROWS * TK, GROUPS = ROWS / 8;
  __shared__ int64_t roff[ROWS];
  __shared__ int64_t koff[TK];
  const int64_t kt = blockIdx.x, rt = blockIdx.y, z = blockIdx.z;
  const int nrm = side == 0 ? d.nm : d.nn;
  const int64_t* rdim = side == 0 ? d.mdim : d.ndim;
  const int64_t* rstr = side == 0 ? d.msa : d.nsb;
  const int64_t* kstr = side == 0 ? d.ksa : d.ksb;
  const int64_t* zstr = side == 0 ? d.zsa : d.zsb;
  for (int t = threadIdx.x; t < ROWS + TK; t += blockDim.x) {
    if (t < ROWS) {
      int64_t r = rt * ROWS + t;
      roff[t] = r < rows ? decode(r, nrm, rdim, rstr) : -1;
    } else {
      int64_t k = kt * TK + (t - ROWS);
      koff[t - ROWS] = k < d.K ? decode(k, d.nk, d.kdim, kstr) : -1;
    }
  }
  __syncthreads();
  const int64_t zo = decode(z, d.nz, d.zdim, zstr);
  float* tile = planes + (((z * rtiles + rt) * ktiles + kt) * (2 * NS)) * (int64_t)TILE;
  for (int o = threadIdx.x; o < TILE; o += blockDim.x) {
    // o = ((kc * GROUPS + g) * 32) + r8 * 4 + k4
    const int core = o >> 5, within = o & 31;
    const int kc = core / GROUPS, g = core - kc * GROUPS;
    const int r = g * 8 + (within >> 2), k = kc * 4 + (within & 3);
    float re[3] = {0.f, 0.f, 0.f}, im[3] = {0.f, 0.f, 0.f};
    if (roff[r] >= 0 && koff[k] >= 0) {
      T v = X[zo + roff[r] + koff[k]];
      split<NS>(v.x, re);
      split<NS>(v.y, im);
    }
#pragma unroll
    for (int t = 0; t < NS; ++t) {
      tile[(0 * NS + t) * TILE + o] = re[t];
      tile[(1 * NS + t) * TILE + o] = im[t];
    }
  }
}

template <int NS>
struct alignas(1024) TcSmem {
  float stage[Cfg<NS>::stages][Cfg<NS>::planes * (kATile + kBTile)];  // A planes, then B planes
  uint64_t full[Cfg<NS>::stages];
  uint64_t empty[Cfg<NS>::stages];
  uint64_t accf[kSets];
  uint64_t acce[kSets];
  uint64_t drain;
  uint32_t tmem_base;
};

// Persistent: each CTA walks output tiles blockIdx.x, +gridDim.x, ... (n tile
// fastest, so the CTAs working on one row block at a time share its A planes
// in L2).  The producer and the MMA issuer run ahead across tile boundaries;
// the epilogue of one tile overlaps the MMAs of the next.
template <typename TC, int NS>
__global__ void __launch_bounds__(kThreads, 1)
    k_tc_gemm(const float* __restrict__ pa, const float* __restrict__ pb, TC* __restrict__ C,
              const __grid_constant__ GemmDesc d, const int64_t* __restrict__ cm_tab,
              const int64_t* __restrict__ cn_tab, int64_t mtiles, int64_t ntiles, int64_t ktiles, int* status) {
  using CF = Cfg<NS>;
  constexpr int S = CF::stages, P = CF::planes;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TcSmem<NS>& sm = *reinterpret_cast<TcSmem<NS>*>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ntot = ntiles * mtiles * d.Z;

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&sm.full[s], 1);
      mbar_init(&sm.empty[s], 1);
    }
    for (int b = 0; b < kSets; ++b) {
      mbar_init(&sm.accf[b], 1);
      mbar_init(&sm.acce[b], kEpiWarps);  // one arrival per epilogue warp
    }
    mbar_init(&sm.drain, 1);
    mbar_init_fence();
  }
  if (warp == 1) {
    tmem_alloc(&sm.tmem_base, kTmemCols);
  }
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
        const float* atile = pa + ((z * mtiles + mt) * ktiles) * (int64_t)(P * kATile);
        const float* btile = pb + ((z * ntiles + nt) * ktiles) * (int64_t)(P * kBTile);
        for (int64_t kt = 0; kt < ktiles; ++kt, ++g) {
          const int s = (int)(g % S);
          const uint32_t ph = (uint32_t)((g / S) & 1);
          if (!mbar_wait(&sm.empty[s], ph ^ 1)) {
            ok = false;
            break;
          }
          mbar_expect_tx(&sm.full[s], CF::stage_bytes);
          const float* a = atile + kt * (P * kATile);
          const float* b = btile + kt * (P * kBTile);
          float* dst = sm.stage[s];
#pragma unroll
          for (int p = 0; p < P; ++p) {
            bulk_g2s(dst + p * kATile, a + p * kATile, kATile * 4, &sm.full[s]);
            bulk_g2s(dst + P * kATile + p * kBTile, b + p * kBTile, kBTile * 4, &sm.full[s]);
          }
        }
      }
      // the copies of the last stages are in flight until their full barrier
      // completes: wait (bounded) so none lands after the CTA has exited
      for (int64_t i = g - 1; i >= 0 && i >= g - S; --i)
        if (!mbar_wait(&sm.full[i % S], (uint32_t)((i / S) & 1))) ok = false;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_tf32(TM, TN), idesc_neg = idesc_tf32(TM, TN, true);
      constexpr uint32_t ALBO = (TM / 8) * 128, BLBO = (TN / 8) * 128, SBO = 128;
      int64_t g = 0;  // K tiles (= chunks) consumed so far
      for (int64_t tile = blockIdx.x; tile < ntot && ok; tile += gridDim.x) {
        for (int64_t kt = 0; kt < ktiles; ++kt, ++g) {
          const int s = (int)(g % S);
          const uint32_t ph = (uint32_t)((g / S) & 1);
          const int b = (int)(g % kSets);
          const uint32_t use = (uint32_t)((g / kSets) & 1);
          if (!mbar_wait(&sm.full[s], ph) || !mbar_wait(&sm.acce[b], use ^ 1)) {
            ok = false;
            break;
          }
          fence_after();
          const uint32_t sa = smem_u32(sm.stage[s]);
          const uint32_t sb = sa + P * kATile * 4;
          const uint32_t dr = tmem + (uint32_t)b * (2 * TN), di = dr + TN;
          // The tensor core rounds an accumulation toward zero.  The small
          // correction products go in first (the first one overwrites), the
          // large hi x hi products last.
#pragma unroll
          for (int q = 1; q <= CF::products; ++q) {
            const int qq = q == CF::products ? 0 : q;  // hi x hi last
            // term pairs (i, j) with i + j < NS: (0,0) (0,1) (1,0) (0,2) (2,0) (1,1)
            const int ti = (qq == 2) ? 1 : (qq == 4) ? 2 : (qq == 5) ? 1 : 0;
            const int tj = (qq == 1) ? 1 : (qq == 3) ? 2 : (qq == 5) ? 1 : 0;
#pragma unroll
            for (int j = 0; j < TK / 8; ++j) {  // the two 8-deep halves of the tile
              const uint32_t acc = (q == 1 && j == 0) ? 0u : 1u;
              const uint32_t oa = (uint32_t)j * 2 * ALBO, ob = (uint32_t)j * 2 * BLBO;
              const uint64_t ar = smem_desc(sa + (0 * NS + ti) * kATile * 4 + oa, ALBO, SBO);
              const uint64_t ai = smem_desc(sa + (1 * NS + ti) * kATile * 4 + oa, ALBO, SBO);
              const uint64_t br = smem_desc(sb + (0 * NS + tj) * kBTile * 4 + ob, BLBO, SBO);
              const uint64_t bi = smem_desc(sb + (1 * NS + tj) * kBTile * 4 + ob, BLBO, SBO);
              mma_tf32(dr, ar, br, idesc, acc);     // + Ar.Br
              mma_tf32(di, ar, bi, idesc, acc);     // + Ar.Bi
              mma_tf32(dr, ai, bi, idesc_neg, 1u);  // - Ai.Bi
              mma_tf32(di, ai, br, idesc, 1u);      // + Ai.Br
            }
          }
          mma_commit(&sm.accf[b]);   // chunk accumulators ready for the epilogue
          mma_commit(&sm.empty[s]);  // smem stage free once these MMAs finish
        }
      }
      // every MMA issued has finished once this arrives (TMEM is freed below)
      mma_commit(&sm.drain);
      if (!mbar_wait(&sm.drain, 0)) ok = false;
    }
  } else {
    // epilogue: warp w reads TMEM lanes of quadrant w % 4, columns [16h, 16h+16)
    constexpr int CW = TN / (kEpiWarps / 4);  // columns per epilogue warp
    static_assert(CW == 16, "one 16-column load per accumulator");
    const int q = warp & 3, h = (warp - 2) >> 2;
    const int row = q * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
    int64_t g = 0;
    for (int64_t tile = blockIdx.x; tile < ntot && ok; tile += gridDim.x) {
      const int64_t nt = tile % ntiles, r = tile / ntiles, mt = r % mtiles, z = r / mtiles;
      KahanC acc[CW];
#pragma unroll
      for (int j = 0; j < CW; ++j) kahan_init(acc[j]);
      for (int64_t kt = 0; kt < ktiles; ++kt, ++g) {
        const int b = (int)(g % kSets);
        const uint32_t use = (uint32_t)((g / kSets) & 1);
        bool got = mbar_wait(&sm.accf[b], use);
        got = __all_sync(0xffffffffu, got);  // the TMEM loads below are warp-collective
        if (!got) {
          ok = false;
          break;
        }
        fence_after();
        const uint32_t col = (uint32_t)(b * 2 * TN + h * CW);
        float vr[16], vi[16];
        tmem_ld16(lane_base + col, vr);
        tmem_ld16(lane_base + col + TN, vi);
        tmem_wait_ld();
        fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.acce[b]);  // values are in registers: hand the set back
#pragma unroll
        for (int j = 0; j < CW; ++j) kahan_add(acc[j], make_float2(vr[j], vi[j]));
      }
      if (!ok) break;
      const int64_t m = mt * TM + row;
      if (m < d.M) {
        const int64_t base = decode(z, d.nz, d.zdim, d.zsc) + cm_tab[m];
        const int64_t n0 = nt * TN + h * CW;
#pragma unroll
        for (int j = 0; j < CW; ++j) {
          if (n0 + j >= d.N) break;
          // the truncations of every chunk shrink it by kTruncBias relative
          // on average; the sum is linear in the chunks, so the expectation
          // is added back once here
          const float2 v = kahan_value(acc[j]);
          C[base + cn_tab[n0 + j]] = store_as<TC>(make_float2(fmaf(kTruncBias, v.x, v.x), fmaf(kTruncBias, v.y, v.y)));
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

int splits_of(int precision) { return precision == PQ_PREC_6XTF32 ? 3 : 2; }

template <typename T, int NS>
void pack_both(const void* A, int ta, const void* B, int tb, float* pa, float* pb, const GemmDesc& d, int64_t mt,
               int64_t nt, int64_t kt, cudaStream_t s) {
  dim3 ga((unsigned)kt, (unsigned)mt, (unsigned)d.Z), gb((unsigned)kt, (unsigned)nt, (unsigned)d.Z);
  (void)sizeof(T);
  if (ta == PQ_C128)
    k_tc_pack<double2, NS, TM><<<ga, 256, 0, s>>>((const double2*)A, pa, d, 0, d.M, mt, kt);
  else
    k_tc_pack<float2, NS, TM><<<ga, 256, 0, s>>>((const float2*)A, pa, d, 0, d.M, mt, kt);
  if (tb == PQ_C128)
    k_tc_pack<double2, NS, TN><<<gb, 256, 0, s>>>((const double2*)B, pb, d, 1, d.N, nt, kt);
  else
    k_tc_pack<float2, NS, TN><<<gb, 256, 0, s>>>((const float2*)B, pb, d, 1, d.N, nt, kt);
}

template <typename TC, int NS>
cudaError_t gemm_launch(const float* pa, const float* pb, void* C, const GemmDesc& d, const int64_t* cm,
                        const int64_t* cn, int64_t mt, int64_t nt, int64_t kt, int* status, cudaStream_t s) {
  static_assert(sizeof(TcSmem<NS>) + 1024 <= 232448, "shared memory layout exceeds 227 KiB");
  // the whole opt-in shared memory (one CTA per SM either way): the ring plus
  // slack past the last stage
  const size_t smem = 232448;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_tc_gemm<TC, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const int64_t tiles = mt * nt * d.Z;
  const unsigned grid = (unsigned)std::min<int64_t>(tiles, sm_count());
  k_tc_gemm<TC, NS><<<grid, kThreads, smem, s>>>(pa, pb, (TC*)C, d, cm, cn, mt, nt, kt, status);
  return cudaGetLastError();
}

}  // namespace

// PQ_PREC_OZAKI / PQ_PREC_OZAKI4 / PQ_PREC_3XBF16 run the exact-accumulation
// kernels (pq_oz.cu, 5 / 4 / 3 bf16 slices) where their limits allow
// (K <= 512) and the 6xTF32 (the first two) / 3xTF32 kernels otherwise.
static bool tf32_eligible(const GemmDesc& d) {
  if (d.M < 64 || d.N < 64 || d.K < 16) return false;
  return d.Z <= 65535 && ceil_div(d.N, TN) <= 65535 && ceil_div(d.M, TM) <= 65535;
}
static int tf32_precision(int precision) {
  return (precision == PQ_PREC_OZAKI || precision == PQ_PREC_OZAKI4)
             ? PQ_PREC_6XTF32
             : (precision == PQ_PREC_3XBF16 ? PQ_PREC_3XTF32 : precision);
}
static bool sliced_bf16(int precision) {
  return precision == PQ_PREC_OZAKI || precision == PQ_PREC_OZAKI4 || precision == PQ_PREC_3XBF16;
}
static int bf16_slices(int precision) {
  return precision == PQ_PREC_OZAKI ? 5 : (precision == PQ_PREC_OZAKI4 ? 4 : 3);
}

size_t tc_scratch_bytes(int precision, const GemmDesc& d) {
  if (sliced_bf16(precision) && oz_eligible(d)) return oz_scratch_bytes(bf16_slices(precision), d);
  const int P = 2 * splits_of(tf32_precision(precision));
  const int64_t mt = ceil_div(d.M, TM), nt = ceil_div(d.N, TN), kt = ceil_div(d.K, TK);
  return (size_t)(d.Z * (mt * kATile + nt * kBTile) * kt * P * 4) + (size_t)(d.M + d.N) * 8 + 1024;
}

bool tc_eligible(int precision, const GemmDesc& d) {
  if (precision != PQ_PREC_3XTF32 && precision != PQ_PREC_6XTF32 && !sliced_bf16(precision)) return false;
  if (sliced_bf16(precision) && oz_eligible(d)) return true;
  return tf32_eligible(d) && tc_scratch_bytes(precision, d) <= (size_t(24) << 30);
}

int tc_launch_count(int precision, const GemmDesc& d) {
  // exponents of A and B, slices of B, result index table, GEMM (A is sliced
  // inside it); or the TF32 path's index table, two packs, GEMM
  return (sliced_bf16(precision) && oz_eligible(d)) ? 5 : 4;
}

cudaError_t launch_tc(int precision, int ta, int tb, int tc, const void* A, const void* B, void* C, const GemmDesc& d,
                      void* scratch, size_t scratch_bytes, int* status, cudaStream_t stream) {
  if (!tc_eligible(precision, d)) return cudaErrorNotSupported;
  if (!scratch || scratch_bytes < tc_scratch_bytes(precision, d)) return cudaErrorInvalidValue;
  if (sliced_bf16(precision) && oz_eligible(d))
    return launch_oz(bf16_slices(precision), ta, tb, tc, A, B, C, d, scratch, scratch_bytes, status, stream);
  const int NS = splits_of(tf32_precision(precision));
  const int64_t mt = ceil_div(d.M, TM), nt = ceil_div(d.N, TN), kt = ceil_div(d.K, TK);
  float* pa = (float*)(((uintptr_t)scratch + 255) & ~(uintptr_t)255);
  float* pb = pa + d.Z * mt * kt * (int64_t)(2 * NS * kATile);
  int64_t* cm = (int64_t*)(pb + d.Z * nt * kt * (int64_t)(2 * NS * kBTile));
  int64_t* cn = cm + d.M;
  const int64_t idx_blocks = std::min<int64_t>(ceil_div(d.M + d.N, 256), 152 * 8);
  k_result_index<<<(unsigned)idx_blocks, 256, 0, stream>>>(d, cm, cn);
  cudaError_t e;
  if (NS == 2) {
    pack_both<float, 2>(A, ta, B, tb, pa, pb, d, mt, nt, kt, stream);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return tc == PQ_C128 ? gemm_launch<double2, 2>(pa, pb, C, d, cm, cn, mt, nt, kt, status, stream)
                         : gemm_launch<float2, 2>(pa, pb, C, d, cm, cn, mt, nt, kt, status, stream);
  }
  pack_both<float, 3>(A, ta, B, tb, pa, pb, d, mt, nt, kt, stream);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  return tc == PQ_C128 ? gemm_launch<double2, 3>(pa, pb, C, d, cm, cn, mt, nt, kt, status, stream)
                       : gemm_launch<float2, 3>(pa, pb, C, d, cm, cn, mt, nt, kt, status, stream);
}

}  // namespace pq
