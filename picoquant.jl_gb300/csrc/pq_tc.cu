// Split-precision complex contraction on the 5th-generation tensor cores
// (tcgen05, sm_103a): TF32 split products, FP32 accumulation in TMEM over
// short K chunks, chunk sums folded into Kahan-compensated FP32 registers.
//
//   C = A x B (complex), four real accumulators per output tile
//     P1 = Ar.Br,  P2 = Ai.Bi,  P3 = Ar.Bi,  P4 = Ai.Br  (Cr = P1 - P2, Ci = P3 + P4)
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
//   warp 0   producer: cp.async.bulk of the 4*NS plane tiles of one K step
//            into a shared-memory ring (mbarrier complete_tx);
//   warp 1   allocates TMEM and issues tcgen05.mma (M=128, N=48, K=8); every
//            8-deep K step is one chunk, alternating between two sets of four
//            48-column FP32 accumulators, committed to the epilogue per chunk;
//   warps 2-13 epilogue: warp w reads TMEM lanes 32*(w%4).. and 16 of the 48
//            columns, folds each chunk's (P1 - P2, P3 + P4) into Kahan sums,
//            hands the accumulator set back, and finally scatters C through
//            the result index map.
// The tensor core rounds accumulations toward zero; each chunk takes one such
// rounding at full magnitude (its hi x hi product is issued last) and chunks
// are summed with compensation, which keeps the bias from growing with K; the
// expected shrinkage of that rounding is added back in the final store.
// Every mbarrier wait is bounded; on expiry the
// kernel records an error in the context's status word and runs to the end
// (TMEM is always released), so the host sees PQ_ERR_DEVICE, not a hang.
#include <cuda_runtime.h>

#include <cstdint>

#include "pq_types.cuh"

namespace pq {

namespace {

constexpr int TM = 128, TN = 48, TK = 16;
constexpr int kThreads = 448;                  // producer, MMA, 12 epilogue warps
constexpr int kEpiWarps = 12;
constexpr uint32_t kTmemCols = 512;            // 2 sets x 4 accumulators x 48 columns = 384 used
constexpr uint32_t kWaitLimit = 1u << 22;      // mbarrier polls before giving up
constexpr int kStatusTcTimeout = 0x7c01;
// Expected relative shrinkage of a value truncated (rounded toward zero) to
// FP32: half an ulp over a log-uniform mantissa, 2^-24 * ln 2.
constexpr float kTruncBias = 4.13145e-8f;
constexpr int kATile = TM * TK;                // floats per A plane tile (8 KiB)
constexpr int kBTile = TN * TK;                // floats per B plane tile (3 KiB)

template <int NS>
struct Cfg {
  static constexpr int planes = 2 * NS;                                  // per operand
  static constexpr uint32_t stage_bytes = planes * (kATile + kBTile) * 4;
  static constexpr int stages = NS == 2 ? 4 : 3;
  static constexpr int products = NS == 2 ? 3 : 6;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

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

__device__ __forceinline__ int64_t decode(int64_t x, int n, const int64_t* dim, const int64_t* s1) {
  int64_t o = 0;
#pragma unroll 1
  for (int i = 0; i < n; ++i) {
    int64_t q = x / dim[i];
    o += (x - q * dim[i]) * s1[i];
    x = q;
  }
  return o;
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

// ---- PTX wrappers -----------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < kWaitLimit; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
// Shared-memory matrix descriptor: no swizzle, K-major canonical layout.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for sm_100-family tcgen05
  return d;                // base offset 0, no swizzle (layout type 0)
}
// Instruction descriptor for kind::tf32, FP32 accumulation, both K-major.
__host__ __device__ constexpr uint32_t idesc_tf32(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

template <int NS>
struct alignas(1024) TcSmem {
  float stage[Cfg<NS>::stages][Cfg<NS>::planes * (kATile + kBTile)];  // A planes, then B planes
  uint64_t full[Cfg<NS>::stages];
  uint64_t empty[Cfg<NS>::stages];
  uint64_t accf[2];
  uint64_t acce[2];
  uint32_t tmem_base;
  int64_t cm[TM];
  int64_t cn[TN];
};

template <typename TC, int NS>
__global__ void __launch_bounds__(kThreads, 1)
    k_tc_gemm(const float* __restrict__ pa, const float* __restrict__ pb, TC* __restrict__ C,
              const __grid_constant__ GemmDesc d, int64_t mtiles, int64_t ntiles, int64_t ktiles, int* status) {
  using CF = Cfg<NS>;
  constexpr int S = CF::stages, P = CF::planes;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TcSmem<NS>& sm = *reinterpret_cast<TcSmem<NS>*>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t nt = blockIdx.x, mt = blockIdx.y, z = blockIdx.z;
  const int64_t nchunks = ktiles * (TK / 8);  // one chunk per 8-deep K step

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&sm.full[s], 1);
      mbar_init(&sm.empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&sm.accf[b], 1);
      mbar_init(&sm.acce[b], kEpiWarps);  // one arrival per epilogue warp
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int i = threadIdx.x; i < TM + TN; i += blockDim.x) {
    if (i < TM) {
      int64_t m = mt * TM + i;
      sm.cm[i] = m < d.M ? decode(m, d.nm, d.mdim, d.msc) : -1;
    } else {
      int64_t n = nt * TN + (i - TM);
      sm.cn[i - TM] = n < d.N ? decode(n, d.nn, d.ndim, d.nsc) : -1;
    }
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.tmem_base)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = sm.tmem_base;
  bool ok = true;

  const float* atile = pa + ((z * mtiles + mt) * ktiles) * (int64_t)(P * kATile);
  const float* btile = pb + ((z * ntiles + nt) * ktiles) * (int64_t)(P * kBTile);

  if (warp == 0) {
    if (lane == 0) {
      for (int64_t kt = 0; kt < ktiles; ++kt) {
        const int s = (int)(kt % S);
        const uint32_t ph = (uint32_t)((kt / S) & 1);
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
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_tf32(TM, TN);
      constexpr uint32_t ALBO = (TM / 8) * 128, BLBO = (TN / 8) * 128, SBO = 128;
      int64_t c = 0;  // chunk = one 8-deep K step
      for (int64_t kt = 0; kt < ktiles && ok; ++kt) {
        const int s = (int)(kt % S);
        const uint32_t ph = (uint32_t)((kt / S) & 1);
        if (!mbar_wait(&sm.full[s], ph)) {
          ok = false;
          break;
        }
        fence_after();
        const uint32_t sa = smem_u32(sm.stage[s]);
        const uint32_t sb = sa + P * kATile * 4;
#pragma unroll
        for (int j = 0; j < TK / 8; ++j, ++c) {
          const int b = (int)(c & 1);
          const uint32_t use = (uint32_t)((c >> 1) & 1);
          if (!mbar_wait(&sm.acce[b], use ^ 1)) {
            ok = false;
            break;
          }
          fence_after();
          const uint32_t d1 = tmem + (uint32_t)b * (4 * TN), d2 = d1 + TN, d3 = d1 + 2 * TN, d4 = d1 + 3 * TN;
          const uint32_t oa = (uint32_t)j * 2 * ALBO, ob = (uint32_t)j * 2 * BLBO;
          // The tensor core rounds an accumulation toward zero.  The small
          // correction products go in first (the first one overwrites), the
          // large hi x hi product last, so each accumulator takes exactly one
          // rounding at its full magnitude per chunk.
#pragma unroll
          for (int q = 1; q <= CF::products; ++q) {
            const int qq = q == CF::products ? 0 : q;  // hi x hi last
            // term pairs (i, j) with i + j < NS: (0,0) (0,1) (1,0) (0,2) (2,0) (1,1)
            const int ti = (qq == 2) ? 1 : (qq == 4) ? 2 : (qq == 5) ? 1 : 0;
            const int tj = (qq == 1) ? 1 : (qq == 3) ? 2 : (qq == 5) ? 1 : 0;
            const uint32_t acc = q == 1 ? 0u : 1u;
            const uint64_t ar = smem_desc(sa + (0 * NS + ti) * kATile * 4 + oa, ALBO, SBO);
            const uint64_t ai = smem_desc(sa + (1 * NS + ti) * kATile * 4 + oa, ALBO, SBO);
            const uint64_t br = smem_desc(sb + (0 * NS + tj) * kBTile * 4 + ob, BLBO, SBO);
            const uint64_t bi = smem_desc(sb + (1 * NS + tj) * kBTile * 4 + ob, BLBO, SBO);
            mma_tf32(d1, ar, br, idesc, acc);  // Ar.Br
            mma_tf32(d2, ai, bi, idesc, acc);  // Ai.Bi
            mma_tf32(d3, ar, bi, idesc, acc);  // Ar.Bi
            mma_tf32(d4, ai, br, idesc, acc);  // Ai.Br
          }
          mma_commit(&sm.accf[b]);  // chunk accumulators ready for the epilogue
        }
        mma_commit(&sm.empty[s]);  // smem stage free once these MMAs finish
      }
    }
  } else {
    // epilogue: warp w reads TMEM lanes of quadrant w % 4, columns [16h, 16h+16)
    constexpr int CW = TN / (kEpiWarps / 4);  // columns per epilogue warp
    const int q = warp & 3, h = (warp - 2) >> 2;
    const int row = q * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
    KahanC acc[CW];
#pragma unroll
    for (int j = 0; j < CW; ++j) kahan_init(acc[j]);
    for (int64_t c = 0; c < nchunks; ++c) {
      const int b = (int)(c & 1);
      const uint32_t use = (uint32_t)((c >> 1) & 1);
      bool got = mbar_wait(&sm.accf[b], use);
      got = __all_sync(0xffffffffu, got);  // the TMEM loads below are warp-collective
      if (!got) {
        ok = false;
        break;
      }
      fence_after();
#pragma unroll
      for (int piece = 0; piece < CW / 8; ++piece) {
        const uint32_t col = (uint32_t)(b * 4 * TN + h * CW + piece * 8);
        float p1[8], p2[8], p3[8], p4[8];
        tmem_ld8(lane_base + col, p1);
        tmem_ld8(lane_base + col + TN, p2);
        tmem_ld8(lane_base + col + 2 * TN, p3);
        tmem_ld8(lane_base + col + 3 * TN, p4);
        tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 8; ++j) kahan_add(acc[piece * 8 + j], make_float2(p1[j] - p2[j], p3[j] + p4[j]));
      }
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.acce[b]);
    }
    if (ok) {
      const int64_t cmr = sm.cm[row];
      const int64_t zc = decode(z, d.nz, d.zdim, d.zsc);
      if (cmr >= 0) {
#pragma unroll
        for (int j = 0; j < CW; ++j) {
          const int64_t cnj = sm.cn[h * CW + j];
          if (cnj < 0) continue;
          // every chunk value came out of one round-toward-zero at full
          // magnitude, which shrinks it by 2^-24 ln 2 relative on average
          // (mantissas log-uniform within a binade); the sum is linear in the
          // chunks, so the expectation is added back once here
          const float2 v = kahan_value(acc[j]);
          C[zc + cmr + cnj] = store_as<TC>(make_float2(fmaf(kTruncBias, v.x, v.x), fmaf(kTruncBias, v.y, v.y)));
        }
      }
    }
  }
  if (!ok && status) atomicExch(status, kStatusTcTimeout);
  fence_before();
  __syncthreads();
  if (warp == 1) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

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
cudaError_t gemm_launch(const float* pa, const float* pb, void* C, const GemmDesc& d, int64_t mt, int64_t nt,
                        int64_t kt, int* status, cudaStream_t s) {
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
  dim3 grid((unsigned)nt, (unsigned)mt, (unsigned)d.Z);
  k_tc_gemm<TC, NS><<<grid, kThreads, smem, s>>>(pa, pb, (TC*)C, d, mt, nt, kt, status);
  return cudaGetLastError();
}

}  // namespace

bool tc_eligible(int precision, const GemmDesc& d) {
  if (precision != PQ_PREC_3XTF32 && precision != PQ_PREC_6XTF32) return false;
  if (d.M < 64 || d.N < 64 || d.K < 16) return false;
  if (d.Z > 65535 || ceil_div(d.N, TN) > 2147483647LL || ceil_div(d.M, TM) > 65535) return false;
  return tc_scratch_bytes(precision, d) <= (size_t(24) << 30);
}

size_t tc_scratch_bytes(int precision, const GemmDesc& d) {
  const int P = 2 * splits_of(precision);
  const int64_t mt = ceil_div(d.M, TM), nt = ceil_div(d.N, TN), kt = ceil_div(d.K, TK);
  return (size_t)(d.Z * (mt * kATile + nt * kBTile) * kt * P * 4) + 1024;
}

cudaError_t launch_tc(int precision, int ta, int tb, int tc, const void* A, const void* B, void* C, const GemmDesc& d,
                      void* scratch, size_t scratch_bytes, int* status, cudaStream_t stream) {
  if (!tc_eligible(precision, d)) return cudaErrorNotSupported;
  if (!scratch || scratch_bytes < tc_scratch_bytes(precision, d)) return cudaErrorInvalidValue;
  const int NS = splits_of(precision);
  const int64_t mt = ceil_div(d.M, TM), nt = ceil_div(d.N, TN), kt = ceil_div(d.K, TK);
  float* pa = (float*)(((uintptr_t)scratch + 255) & ~(uintptr_t)255);
  float* pb = pa + d.Z * mt * kt * (int64_t)(2 * NS * kATile);
  cudaError_t e;
  if (NS == 2) {
    pack_both<float, 2>(A, ta, B, tb, pa, pb, d, mt, nt, kt, stream);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return tc == PQ_C128 ? gemm_launch<double2, 2>(pa, pb, C, d, mt, nt, kt, status, stream)
                         : gemm_launch<float2, 2>(pa, pb, C, d, mt, nt, kt, status, stream);
  }
  pack_both<float, 3>(A, ta, B, tb, pa, pb, d, mt, nt, kt, stream);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  return tc == PQ_C128 ? gemm_launch<double2, 3>(pa, pb, C, d, mt, nt, kt, status, stream)
                       : gemm_launch<float2, 3>(pa, pb, C, d, mt, nt, kt, status, stream);
}

}  // namespace pq
