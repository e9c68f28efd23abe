// Split-precision complex contraction on the 5th-generation tensor cores
// (tcgen05, sm_103a): 3xTF32 products with FP32 accumulation in TMEM.
//
//   C = A x B (complex), computed as three real accumulators per output tile
//     P1 = Ar.Br,  P2 = Ai.Bi,  P3 = Ar.Bi + Ai.Br     (Cr = P1 - P2, Ci = P3)
//   with every real product split as  x.y ~ xh.yh + xh.yl + xl.yh
//   where xh = tf32(x) and xl = tf32(x - xh) (round to nearest).
//
// Step 1 (k_tc_pack): each operand is gathered through its index map (any
// mode order, batch modes) into four planes {re_hi, re_lo, im_hi, im_lo} of
// FP32 values with TF32 precision, laid out tile by tile: a tile is 128 rows
// (M or N) x 16 K values, stored in the canonical no-swizzle K-major UMMA
// layout (8-row x 16-byte core matrices, 128 contiguous bytes each; core
// matrices along K are 2048 bytes apart, along rows 128 bytes apart), so one
// 8 KiB bulk copy moves one plane tile.  Rows and K past the operand are zero.
//
// Step 2 (k_tc_gemm): one CTA per 128 x 128 output tile (x batch), 6 warps:
//   warp 0  producer: cp.async.bulk of 8 plane tiles per K step into a
//           3-stage shared-memory ring (mbarrier complete_tx);
//   warp 1  TMEM owner + MMA issuer: 24 tcgen05.mma (M=128, N=128, K=8) per
//           16-deep K step into three 128-column FP32 accumulators, then
//           tcgen05.commit to release the stage;
//   warps 2-5 epilogue: tcgen05.ld of the accumulators (each warp its 32-lane
//           quadrant), Cr = P1 - P2, Ci = P3, scattered to C through the
//           result index map.
// Every mbarrier wait is bounded; on expiry the kernel records an error in the
// context's status word and runs to completion, so the host sees
// PQ_ERR_DEVICE instead of a hang.
#include <cuda_runtime.h>

#include <cstdint>

#include "pq_types.cuh"

namespace pq {

namespace {

constexpr int TM = 128, TN = 128, TK = 16;      // tile extents
constexpr int kStages = 3;
constexpr int kPlanes = 4;                       // re_hi, re_lo, im_hi, im_lo
constexpr int kTileFloats = TM * TK;             // 2048 floats = 8 KiB per plane tile
constexpr uint32_t kTileBytes = kTileFloats * 4;
constexpr uint32_t kStageBytes = 2 * kPlanes * kTileBytes;  // A and B planes
constexpr int kThreads = 192;
constexpr uint32_t kTmemCols = 512;              // three 128-column accumulators
constexpr uint32_t kWaitLimit = 1u << 22;        // mbarrier polls before giving up
constexpr int kStatusTcTimeout = 0x7c01;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// hi/lo TF32 split of a real value held in FP32 or FP64.
__device__ __forceinline__ void split(float x, float& hi, float& lo) {
  hi = tf32_rna(x);
  lo = tf32_rna(x - hi);
}
__device__ __forceinline__ void split(double x, float& hi, float& lo) {
  hi = tf32_rna((float)x);
  lo = tf32_rna((float)(x - (double)hi));
}

// Offset (in floats) of element (row r, k) inside one plane tile.
__device__ __forceinline__ int tile_off(int r, int k) { return ((k >> 2) * 16 + (r >> 3)) * 32 + (r & 7) * 4 + (k & 3); }

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

// Pack operand X (side 0: A with m modes, side 1: B with n modes) into planes.
// planes layout: [z][row tile][k tile][plane][2048 floats].
template <typename T>
__global__ void __launch_bounds__(256) k_tc_pack(const T* __restrict__ X, float* __restrict__ planes,
                                                 const __grid_constant__ GemmDesc d, int side, int64_t rows,
                                                 int64_t rtiles, int64_t ktiles) {
  __shared__ int64_t roff[TM];
  __shared__ int64_t koff[TK];
  const int64_t kt = blockIdx.x, rt = blockIdx.y;
  const int64_t z = blockIdx.z;
  const int nrm = side == 0 ? d.nm : d.nn;
  const int64_t* rdim = side == 0 ? d.mdim : d.ndim;
  const int64_t* rstr = side == 0 ? d.msa : d.nsb;
  const int64_t* kstr = side == 0 ? d.ksa : d.ksb;
  const int64_t* zstr = side == 0 ? d.zsa : d.zsb;
  const int t = threadIdx.x;
  if (t < TM) {
    int64_t r = rt * TM + t;
    roff[t] = r < rows ? decode(r, nrm, rdim, rstr) : -1;
  } else if (t < TM + TK) {
    int64_t k = kt * TK + (t - TM);
    koff[t - TM] = k < d.K ? decode(k, d.nk, d.kdim, kstr) : -1;
  }
  __syncthreads();
  const int64_t zo = decode(z, d.nz, d.zdim, zstr);
  float* tile = planes + (((z * rtiles + rt) * ktiles + kt) * kPlanes) * (int64_t)kTileFloats;
  for (int o = t; o < kTileFloats; o += blockDim.x) {
    // invert tile_off: o = ((kc*16 + g)*32) + r8*4 + k4
    const int core = o >> 5, within = o & 31;
    const int kc = core >> 4, g = core & 15;
    const int r = g * 8 + (within >> 2), k = kc * 4 + (within & 3);
    float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
    if (roff[r] >= 0 && koff[k] >= 0) {
      T v = X[zo + roff[r] + koff[k]];
      split(v.x, rh, rl);
      split(v.y, ih, il);
    }
    tile[0 * kTileFloats + o] = rh;
    tile[1 * kTileFloats + o] = rl;
    tile[2 * kTileFloats + o] = ih;
    tile[3 * kTileFloats + o] = il;
  }
}

// ---- PTX wrappers -----------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
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
  return (1u << 4)                        // D: F32
         | (2u << 7)                      // A: TF32
         | (2u << 10)                     // B: TF32
         | ((uint32_t)(n >> 3) << 17)     // N / 8
         | ((uint32_t)(m >> 4) << 24);    // M / 16
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
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

struct alignas(1024) TcSmem {
  float stage[kStages][2 * kPlanes][kTileFloats];  // A planes then B planes
  uint64_t full[kStages];
  uint64_t empty[kStages];
  uint64_t accum;
  uint32_t tmem_base;
  int64_t cm[TM];
  int64_t cn[TN];
};

template <typename TC>
__global__ void __launch_bounds__(kThreads, 1)
    k_tc_gemm(const float* __restrict__ pa, const float* __restrict__ pb, TC* __restrict__ C,
              const __grid_constant__ GemmDesc d, int64_t mtiles, int64_t ntiles, int64_t ktiles, int* status) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TcSmem& S = *reinterpret_cast<TcSmem*>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t nt = blockIdx.x, mt = blockIdx.y, z = blockIdx.z;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&S.full[s], 1);
      mbar_init(&S.empty[s], 1);
    }
    mbar_init(&S.accum, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // result offsets of this tile's rows / columns
  for (int i = threadIdx.x; i < TM + TN; i += blockDim.x) {
    if (i < TM) {
      int64_t m = mt * TM + i;
      S.cm[i] = m < d.M ? decode(m, d.nm, d.mdim, d.msc) : -1;
    } else {
      int64_t n = nt * TN + (i - TM);
      S.cn[i - TM] = n < d.N ? decode(n, d.nn, d.ndim, d.nsc) : -1;
    }
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem_base)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = S.tmem_base;
  bool ok = true;

  const float* atile = pa + ((z * mtiles + mt) * ktiles) * (int64_t)(kPlanes * kTileFloats);
  const float* btile = pb + ((z * ntiles + nt) * ktiles) * (int64_t)(kPlanes * kTileFloats);

  if (warp == 0) {
    if (lane == 0) {
      for (int64_t kt = 0; kt < ktiles && ok; ++kt) {
        const int s = (int)(kt % kStages);
        const uint32_t ph = (uint32_t)((kt / kStages) & 1);
        if (!mbar_wait(&S.empty[s], ph ^ 1)) {
          ok = false;
          break;
        }
        mbar_expect_tx(&S.full[s], kStageBytes);
        const float* a = atile + kt * (kPlanes * kTileFloats);
        const float* b = btile + kt * (kPlanes * kTileFloats);
#pragma unroll
        for (int p = 0; p < kPlanes; ++p) {
          bulk_g2s(S.stage[s][p], a + p * kTileFloats, kTileBytes, &S.full[s]);
          bulk_g2s(S.stage[s][kPlanes + p], b + p * kTileFloats, kTileBytes, &S.full[s]);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_tf32(TM, TN);
      constexpr uint32_t LBO = 2048, SBO = 128;  // K-direction / row-direction core matrix strides
      const uint32_t d1 = tmem, d2 = tmem + 128, d3 = tmem + 256;
      for (int64_t kt = 0; kt < ktiles && ok; ++kt) {
        const int s = (int)(kt % kStages);
        const uint32_t ph = (uint32_t)((kt / kStages) & 1);
        if (!mbar_wait(&S.full[s], ph)) {
          ok = false;
          break;
        }
        fence_after();
#pragma unroll
        for (int j = 0; j < TK / 8; ++j) {
          const uint32_t off = (uint32_t)j * 2 * LBO;
          const uint64_t arh = smem_desc(smem_u32(S.stage[s][0]) + off, LBO, SBO);
          const uint64_t arl = smem_desc(smem_u32(S.stage[s][1]) + off, LBO, SBO);
          const uint64_t aih = smem_desc(smem_u32(S.stage[s][2]) + off, LBO, SBO);
          const uint64_t ail = smem_desc(smem_u32(S.stage[s][3]) + off, LBO, SBO);
          const uint64_t brh = smem_desc(smem_u32(S.stage[s][4]) + off, LBO, SBO);
          const uint64_t brl = smem_desc(smem_u32(S.stage[s][5]) + off, LBO, SBO);
          const uint64_t bih = smem_desc(smem_u32(S.stage[s][6]) + off, LBO, SBO);
          const uint64_t bil = smem_desc(smem_u32(S.stage[s][7]) + off, LBO, SBO);
          const uint32_t acc = (kt > 0 || j > 0) ? 1u : 0u;
          // P1 = Ar.Br
          mma_tf32(d1, arh, brh, idesc, acc);
          mma_tf32(d1, arh, brl, idesc, 1u);
          mma_tf32(d1, arl, brh, idesc, 1u);
          // P2 = Ai.Bi
          mma_tf32(d2, aih, bih, idesc, acc);
          mma_tf32(d2, aih, bil, idesc, 1u);
          mma_tf32(d2, ail, bih, idesc, 1u);
          // P3 = Ar.Bi + Ai.Br
          mma_tf32(d3, arh, bih, idesc, acc);
          mma_tf32(d3, arh, bil, idesc, 1u);
          mma_tf32(d3, arl, bih, idesc, 1u);
          mma_tf32(d3, aih, brh, idesc, 1u);
          mma_tf32(d3, aih, brl, idesc, 1u);
          mma_tf32(d3, ail, brh, idesc, 1u);
        }
        mma_commit(&S.empty[s]);  // stage reusable once these MMAs finish
      }
      mma_commit(&S.accum);  // accumulators complete
    }
  } else {
    // epilogue warps 2..5: TMEM lane quadrant = warp % 4
    const int q = warp & 3;
    const int row = q * 32 + lane;
    if (!mbar_wait(&S.accum, 0)) ok = false;
    ok = __all_sync(0xffffffffu, ok);  // the TMEM loads below are warp-collective
    fence_after();
    if (ok) {
      const int64_t cmr = S.cm[row];
      const int64_t zc = decode(z, d.nz, d.zdim, d.zsc);
      const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
#pragma unroll 1
      for (int c0 = 0; c0 < TN; c0 += 16) {
        float p1[16], p2[16], p3[16];
        tmem_ld16(lane_base + c0, p1);
        tmem_ld16(lane_base + 128 + c0, p2);
        tmem_ld16(lane_base + 256 + c0, p3);
        tmem_wait_ld();
        if (cmr >= 0) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int64_t cnj = S.cn[c0 + j];
            if (cnj >= 0) C[zc + cmr + cnj] = store_as<TC>(make_float2(p1[j] - p2[j], p3[j]));
          }
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

}  // namespace

bool tc_eligible(int precision, const GemmDesc& d) {
  if (precision != PQ_PREC_3XTF32) return false;
  if (d.M < 64 || d.N < 64 || d.K < 16) return false;
  if (d.Z > 65535 || ceil_div(d.N, TN) > 2147483647LL || ceil_div(d.M, TM) > 65535) return false;
  // packed planes (16 bytes per complex element of A and B) stay below 24 GiB
  return tc_scratch_bytes(precision, d) <= (size_t(24) << 30);
}

size_t tc_scratch_bytes(int precision, const GemmDesc& d) {
  (void)precision;
  const int64_t mt = ceil_div(d.M, TM), nt = ceil_div(d.N, TN), kt = ceil_div(d.K, TK);
  const int64_t per_tile = (int64_t)kPlanes * kTileFloats * 4;
  return (size_t)(d.Z * (mt + nt) * kt * per_tile) + 1024;
}

cudaError_t launch_tc(int precision, int ta, int tb, int tc, const void* A, const void* B, void* C, const GemmDesc& d,
                      void* scratch, size_t scratch_bytes, int* status, cudaStream_t stream) {
  if (!tc_eligible(precision, d)) return cudaErrorNotSupported;
  if (!scratch || scratch_bytes < tc_scratch_bytes(precision, d)) return cudaErrorInvalidValue;
  const int64_t mt = ceil_div(d.M, TM), nt = ceil_div(d.N, TN), kt = ceil_div(d.K, TK);
  float* pa = (float*)(((uintptr_t)scratch + 255) & ~(uintptr_t)255);
  float* pb = pa + d.Z * mt * kt * (int64_t)(kPlanes * kTileFloats);
  dim3 ga((unsigned)kt, (unsigned)mt, (unsigned)d.Z), gb((unsigned)kt, (unsigned)nt, (unsigned)d.Z);
  if (ta == PQ_C128)
    k_tc_pack<double2><<<ga, 256, 0, stream>>>((const double2*)A, pa, d, 0, d.M, mt, kt);
  else
    k_tc_pack<float2><<<ga, 256, 0, stream>>>((const float2*)A, pa, d, 0, d.M, mt, kt);
  if (tb == PQ_C128)
    k_tc_pack<double2><<<gb, 256, 0, stream>>>((const double2*)B, pb, d, 1, d.N, nt, kt);
  else
    k_tc_pack<float2><<<gb, 256, 0, stream>>>((const float2*)B, pb, d, 1, d.N, nt, kt);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // the whole opt-in shared memory (one CTA per SM either way): the ring plus
  // slack past the last stage
  static_assert(sizeof(TcSmem) + 1024 <= 232448, "shared memory layout exceeds 227 KiB");
  const size_t smem = 232448;
  dim3 grid((unsigned)nt, (unsigned)mt, (unsigned)d.Z);
  if (tc == PQ_C128) {
    static bool attr = false;
    if (!attr) {
      e = cudaFuncSetAttribute(k_tc_gemm<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      attr = true;
    }
    k_tc_gemm<double2><<<grid, kThreads, smem, stream>>>(pa, pb, (double2*)C, d, mt, nt, kt, status);
  } else {
    static bool attr = false;
    if (!attr) {
      e = cudaFuncSetAttribute(k_tc_gemm<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      attr = true;
    }
    k_tc_gemm<float2><<<grid, kThreads, smem, stream>>>(pa, pb, (float2*)C, d, mt, nt, kt, status);
  }
  return cudaGetLastError();
}

}  // namespace pq
