// Skinny pairs on the SIMT cores (sm_103a): a large operand X (R rows over
// its free modes, K <= 16 contracted) against a small operand W (K x N, N <=
// 16), C[r, n] = sum_k X[r, k] W[k, n].  This is a gate of up to four qubits
// applied to a state vector or a boundary tensor absorbing a gate column:
// memory-bound work whose bytes are X read once and C written once.
//
// One thread per row: it decodes the row's offsets in X and C (the modes are
// merged, so a state-vector row has at most a few), loads its K values of X
// (all in flight at once), multiplies them by W from shared memory (a
// broadcast read) and writes its N results.  Consecutive threads take
// consecutive rows, so each load and store of a warp is coalesced whenever the
// row's first mode has unit stride; when X's unit-stride mode is contracted,
// a thread's K loads cover whole sectors instead.
//
// Accumulation: FP32 for complex64 results (K <= 16 terms, the generic
// kernel's single chunk), FP64 for complex128 results.
#include <algorithm>
#include <cstring>
#include <type_traits>

#include "pq_types.cuh"

namespace pq {

namespace {

constexpr int kSkThreads = 256;

struct SkinnyDesc {
  int64_t R, K, N;
  int nr, nk, nn;
  int64_t rdim[kMaxModes], rsx[kMaxModes], rsc[kMaxModes];
  int32_t rlog[kMaxModes];  // log2 of rdim, or -1
  int64_t kdim[kMaxModes], ksx[kMaxModes], ksw[kMaxModes];
  int64_t ndim[kMaxModes], nsw[kMaxModes], nsc[kMaxModes];
};

__device__ __forceinline__ int64_t dec(int64_t x, int n, const int64_t* dim, const int64_t* s) {
  int64_t o = 0;
  for (int i = 0; i < n; ++i) {
    const int64_t q = x / dim[i];
    o += (x - q * dim[i]) * s[i];
    x = q;
  }
  return o;
}

template <typename TX, typename TW, typename TC, typename R, int KMAX>
__global__ void __launch_bounds__(kSkThreads)
    k_skinny(const TX* __restrict__ X, const TW* __restrict__ W, TC* __restrict__ C,
             const __grid_constant__ SkinnyDesc d) {
  using R2 = typename Acc<R>::C;
  __shared__ R2 w[KMAX][kSkinnyN];  // W[k][n], zero past K and N
  __shared__ int64_t kx[KMAX];
  __shared__ int64_t cn[kSkinnyN];
  for (int t = threadIdx.x; t < KMAX * kSkinnyN; t += blockDim.x) {
    const int k = t / kSkinnyN, n = t % kSkinnyN;
    R2 v = czero(R());
    if (k < d.K && n < d.N) v = cvt<R>(W[dec(k, d.nk, d.kdim, d.ksw) + dec(n, d.nn, d.ndim, d.nsw)]);
    w[k][n] = v;
  }
  for (int t = threadIdx.x; t < KMAX; t += blockDim.x) kx[t] = t < d.K ? dec(t, d.nk, d.kdim, d.ksx) : 0;
  for (int t = threadIdx.x; t < kSkinnyN; t += blockDim.x) cn[t] = t < d.N ? dec(t, d.nn, d.ndim, d.nsc) : 0;
  __syncthreads();
  const int K = (int)d.K, N = (int)d.N;
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < d.R; r += step) {
    int64_t xo = 0, co = 0, x = r;
    for (int i = 0; i < d.nr; ++i) {
      int64_t q, rem;
      if (d.rlog[i] >= 0) {
        rem = x & (d.rdim[i] - 1);
        q = x >> d.rlog[i];
      } else {
        q = x / d.rdim[i];
        rem = x - q * d.rdim[i];
      }
      xo += rem * d.rsx[i];
      co += rem * d.rsc[i];
      x = q;
    }
    R2 a[KMAX];
#pragma unroll
    for (int k = 0; k < KMAX; ++k) a[k] = k < K ? cvt<R>(__ldg(X + xo + kx[k])) : czero(R());
#pragma unroll
    for (int n0 = 0; n0 < kSkinnyN; n0 += 4) {
      if (n0 >= N) break;
      R2 acc[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[j] = czero(R());
#pragma unroll
      for (int k = 0; k < KMAX; ++k) {
#pragma unroll
        for (int j = 0; j < 4; ++j) cfma(acc[j], a[k], w[k][n0 + j]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (n0 + j < N) C[co + cn[n0 + j]] = store_as<TC>(acc[j]);
    }
  }
}

template <typename TX, typename TW, typename TC>
cudaError_t launch_typed(const void* X, const void* W, void* C, const SkinnyDesc& d, cudaStream_t s) {
  using R = typename std::conditional<std::is_same<TC, double2>::value, double, float>::type;
  const int grid = grid_for(d.R, kSkThreads);
  if (d.K <= 4)
    k_skinny<TX, TW, TC, R, 4><<<grid, kSkThreads, 0, s>>>((const TX*)X, (const TW*)W, (TC*)C, d);
  else
    k_skinny<TX, TW, TC, R, kSkinnyK><<<grid, kSkThreads, 0, s>>>((const TX*)X, (const TW*)W, (TC*)C, d);
  return cudaGetLastError();
}

int log2_exact(int64_t v) {
  int l = 0;
  while ((int64_t(1) << l) < v) ++l;
  return (int64_t(1) << l) == v ? l : -1;
}

}  // namespace

bool skinny_eligible(const GemmDesc& g) {
  return g.Z == 1 && std::max(g.M, g.N) >= kSkinnyMinRows && std::min(g.M, g.N) <= kSkinnyN && g.K <= kSkinnyK;
}

cudaError_t launch_skinny(int ta, int tb, int tc, const void* A, const void* B, void* C, const GemmDesc& g,
                          cudaStream_t stream) {
  if (!skinny_eligible(g)) return cudaErrorInvalidValue;
  // the large side is X (rows), the small side W
  const bool a_big = g.M >= g.N;
  SkinnyDesc d;
  std::memset(&d, 0, sizeof(d));
  d.R = a_big ? g.M : g.N;
  d.N = a_big ? g.N : g.M;
  d.K = g.K;
  d.nr = a_big ? g.nm : g.nn;
  d.nn = a_big ? g.nn : g.nm;
  d.nk = g.nk;
  for (int i = 0; i < d.nr; ++i) {
    d.rdim[i] = a_big ? g.mdim[i] : g.ndim[i];
    d.rsx[i] = a_big ? g.msa[i] : g.nsb[i];
    d.rsc[i] = a_big ? g.msc[i] : g.nsc[i];
    d.rlog[i] = log2_exact(d.rdim[i]);
  }
  for (int i = 0; i < d.nk; ++i) {
    d.kdim[i] = g.kdim[i];
    d.ksx[i] = a_big ? g.ksa[i] : g.ksb[i];
    d.ksw[i] = a_big ? g.ksb[i] : g.ksa[i];
  }
  for (int i = 0; i < d.nn; ++i) {
    d.ndim[i] = a_big ? g.ndim[i] : g.mdim[i];
    d.nsw[i] = a_big ? g.nsb[i] : g.msa[i];
    d.nsc[i] = a_big ? g.nsc[i] : g.msc[i];
  }
  if (d.R == 0) return cudaSuccess;
  const void* X = a_big ? A : B;
  const void* W = a_big ? B : A;
  const int tx = a_big ? ta : tb, tw = a_big ? tb : ta;
  const bool x64 = tx == PQ_C128, w64 = tw == PQ_C128, c64 = tc == PQ_C128;
  if (!x64 && !w64 && !c64) return launch_typed<float2, float2, float2>(X, W, C, d, stream);
  if (!x64 && w64 && !c64) return launch_typed<float2, double2, float2>(X, W, C, d, stream);
  if (!x64 && !w64 && c64) return launch_typed<float2, float2, double2>(X, W, C, d, stream);
  if (!x64 && w64 && c64) return launch_typed<float2, double2, double2>(X, W, C, d, stream);
  if (x64 && !w64 && !c64) return launch_typed<double2, float2, float2>(X, W, C, d, stream);
  if (x64 && w64 && !c64) return launch_typed<double2, double2, float2>(X, W, C, d, stream);
  if (x64 && !w64 && c64) return launch_typed<double2, float2, double2>(X, W, C, d, stream);
  return launch_typed<double2, double2, double2>(X, W, C, d, stream);
}

}  // namespace pq
