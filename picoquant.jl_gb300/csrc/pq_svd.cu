// Singular value decomposition on the device for the bond splits of the
// compressed (MPS) path: decompose_tensor! (src/layer1.jl:146-184, reached
// from src/layer2.jl:487-560 and compress_bond!).
//
// One-sided (Hestenes) Jacobi (Demmel & Veselic, "Jacobi's method is more
// accurate than QR", SIAM J. Matrix Anal. Appl. 13, 1992): the columns of W
// (R x Cn, R >= Cn, column-major) are orthogonalised by plane rotations
// applied in place, accumulated in V; at convergence the column norms are
// the singular values, the normalised columns the left singular vectors.  A
// matrix with fewer rows than columns is decomposed through W = A^H.
//
// The pairs of a round (the circle method over the columns) are disjoint, so
// the one CTA rotates all of them at once; each pair's three inner products
// are reductions over the lanes that hold it.  A pair (x, y) with inner product
// g = x^H y = |g| e^{i phi} is rotated as the real pair (x, y e^{-i phi}) by
// the classical angle and y's phase restored.
//
// The arithmetic follows the element type of the backend, as LAPACK's does
// for the reference: complex FP32 (complex64 contexts) or complex FP64
// (complex128 contexts).  W, and V where room is left, live in shared memory
// for the whole iteration; the bond splits of the compressed path are small
// matrices (2 chi x 2 chi), which one CTA holds.  The sweep count is bounded
// by the caller's max_sweeps.
#include <cuda_runtime.h>

#include <cmath>

#include "pq_types.cuh"

namespace pq {

namespace {

constexpr int kSvdThreads = 1024;
constexpr int kSvdWarps = kSvdThreads / 32;
constexpr size_t kSvdSmemCap = 220 * 1024;  // of the 227 KB a CTA may hold

template <typename Rl>
struct Cx;
template <>
struct Cx<float> {
  using T = float2;
};
template <>
struct Cx<double> {
  using T = double2;
};

template <typename C, typename Rl>
__device__ __forceinline__ C mk(Rl a, Rl b) {
  C r;
  r.x = a;
  r.y = b;
  return r;
}
template <typename C>
__device__ __forceinline__ C cmul(C a, C b) {
  return mk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename C>
__device__ __forceinline__ C cconj(C a) {
  return mk<C>(a.x, -a.y);
}
template <typename Rl>
__device__ __forceinline__ Rl wsum(Rl v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Columns a and b of the round-robin pairing of N (even) players in round r
// (r < N - 1, k < N / 2: each sum below wraps at most once).
__device__ __forceinline__ void pair_of(int r, int k, int N, int& a, int& b) {
  if (k == 0) {
    a = r;
    b = N - 1;
  } else {
    a = r + k;
    if (a >= N - 1) a -= N - 1;
    b = r - k + N - 1;
    if (b >= N - 1) b -= N - 1;
  }
}

// 1 / sqrt(x) for x > 0 to about one ulp: the hardware estimate and one
// Newton-Raphson step y <- y (3 - x y^2) / 2.
__device__ __forceinline__ float rsqrt_nr(float x) {
  const float y = rsqrtf(x);
  return y * fmaf(-0.5f * x * y, y, 1.5f);
}

// The rotation of a pair from its Gram entries al = |x|^2, be = |y|^2,
// g = gr + i gi = x^H y: false when the pair is orthogonal to tol (or its
// inner product below the floor), else c, s (c^2 + s^2 = 1) and the unit
// phase e = g / |g|.  Only c, s and e need full precision (they make the
// rotation unitary); the angle itself may be approximate, which Jacobi's
// next sweep absorbs.
template <typename Rl>
__device__ __forceinline__ bool rot_params(Rl al, Rl be, Rl gr, Rl gi, Rl floor2, Rl tol2, Rl& c, Rl& s,
                                           typename Cx<Rl>::T& e);
template <>
__device__ __forceinline__ bool rot_params<float>(float al, float be, float gr, float gi, float floor2, float tol2,
                                                  float& c, float& s, float2& e) {
  const float g2 = fmaf(gr, gr, gi * gi);
  if (!(g2 > floor2) || al == 0.f || be == 0.f || g2 < tol2 * al * be) return false;
  const float ig = rsqrt_nr(g2);
  e = make_float2(gr * ig, gi * ig);
  const float zeta = (be - al) * 0.5f * ig;
  const float az = fabsf(zeta);
  const float q = fmaf(az, az, 1.f);
  const float t = az < 1e18f ? __fdividef(1.f, az + q * rsqrtf(q)) : __fdividef(0.5f, az);
  c = rsqrt_nr(fmaf(t, t, 1.f));
  s = zeta >= 0.f ? c * t : -c * t;
  return true;
}
template <>
__device__ __forceinline__ bool rot_params<double>(double al, double be, double gr, double gi, double floor2,
                                                   double tol2, double& c, double& s, double2& e) {
  const double g2 = fma(gr, gr, gi * gi);
  if (!(g2 > floor2) || al == 0.0 || be == 0.0 || g2 < tol2 * al * be) return false;
  const double g = sqrt(g2);
  e = make_double2(gr / g, gi / g);
  const double zeta = (be - al) / (2.0 * g);
  const double az = fabs(zeta);
  const double t = az < 1e150 ? 1.0 / (az + sqrt(fma(az, az, 1.0))) : 0.5 / az;
  c = 1.0 / sqrt(fma(t, t, 1.0));
  s = zeta >= 0.0 ? c * t : -c * t;
  return true;
}

// A (m x n, column-major) -> W (R x Cn) = A, or A^H when m < n; V = I;
// Jacobi sweeps; sig = the column norms of W.  W and V are worked on in
// shared memory when w_sm / v_sm are set, and written to Wg / Vg at the end.
//
// Every pair of a round is in flight at once: a warp holds G = 32 / L pairs,
// L lanes each (L = 32, 16 or 8 for up to 64, 128 or 256 columns), so that a
// round costs one pair's chain of dependent steps (inner products, a
// reduction over L lanes, the rotation's scalars, the rotation).  Lanes of a
// pair that has nothing to do (the padding column, an orthogonal pair) still
// take part in the reduction, which every lane of the warp executes.
template <typename Rl>
__global__ void __launch_bounds__(kSvdThreads)
    k_jacobi_svd(const typename Cx<Rl>::T* __restrict__ A, int m, int n, typename Cx<Rl>::T* Wg,
                 typename Cx<Rl>::T* Vg, Rl* __restrict__ sig, int w_sm, int v_sm, int max_sweeps, Rl tol,
                 int* __restrict__ sweeps_out) {
  using C = typename Cx<Rl>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const bool tr = m < n;
  const int R = tr ? n : m;
  const int Cn = tr ? m : n;
  C* W = w_sm ? (C*)smem_raw : Wg;
  C* V = v_sm ? (C*)smem_raw + (w_sm ? R * Cn : 0) : Vg;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __shared__ Rl s_red[kSvdWarps];

  Rl f2 = 0;
  for (int i = threadIdx.x; i < R * Cn; i += blockDim.x) {
    const int r = i % R, j = i / R;
    const C a = tr ? cconj(A[j + (int64_t)m * r]) : A[i];
    W[i] = a;
    f2 += a.x * a.x + a.y * a.y;
  }
  for (int i = threadIdx.x; i < Cn * Cn; i += blockDim.x) V[i] = mk<C>((i % Cn) == (i / Cn) ? Rl(1) : Rl(0), Rl(0));
  // ||W||_F^2: pairs whose inner product is at most tol^2 of it are left as
  // they are; together they move no singular value by more than
  // sqrt(Cn) tol ||W||_F (Weyl's bound on the Gram matrix W^H W)
  f2 = wsum(f2);
  if (lane == 0) s_red[warp] = f2;
  __syncthreads();
  f2 = 0;
  for (int w = 0; w < kSvdWarps; ++w) f2 += s_red[w];
  const Rl floor2 = (tol * tol * f2) * (tol * tol * f2), tol2 = tol * tol;
  __syncthreads();

  const int N = Cn + (Cn & 1);
  const int L = N / 2 <= kSvdWarps ? 32 : (N / 2 <= 2 * kSvdWarps ? 16 : 8);
  const int sub = lane % L;
  const int slot = warp * (32 / L) + lane / L;  // the pair index k of every round
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    int rotated = 0;
    for (int r = 0; r < N - 1; ++r) {
      int a = 0, b = 0;
      bool live = slot < N / 2;
      if (live) {
        pair_of(r, slot, N, a, b);
        live = a < Cn && b < Cn;  // not the padding column
      }
      C* x = W + a * R;
      C* y = W + b * R;
      Rl al = 0, be = 0, gr = 0, gi = 0;
      if (live)
        for (int i = sub; i < R; i += L) {
          const C u = x[i], v = y[i];
          al += u.x * u.x + u.y * u.y;
          be += v.x * v.x + v.y * v.y;
          gr += u.x * v.x + u.y * v.y;  // conj(u) v
          gi += u.x * v.y - u.y * v.x;
        }
      for (int o = L / 2; o > 0; o >>= 1) {
        al += __shfl_xor_sync(0xffffffffu, al, o);
        be += __shfl_xor_sync(0xffffffffu, be, o);
        gr += __shfl_xor_sync(0xffffffffu, gr, o);
        gi += __shfl_xor_sync(0xffffffffu, gi, o);
      }
      Rl c, s;
      C e;
      if (live && rot_params<Rl>(al, be, gr, gi, floor2, tol2, c, s, e)) {
        rotated = 1;
        for (int i = sub; i < R; i += L) {
          const C u = x[i], yt = cmul(y[i], cconj(e));
          x[i] = mk<C>(c * u.x - s * yt.x, c * u.y - s * yt.y);
          y[i] = cmul(mk<C>(s * u.x + c * yt.x, s * u.y + c * yt.y), e);
        }
        C* va = V + a * Cn;
        C* vb = V + b * Cn;
        for (int i = sub; i < Cn; i += L) {
          const C u = va[i], yt = cmul(vb[i], cconj(e));
          va[i] = mk<C>(c * u.x - s * yt.x, c * u.y - s * yt.y);
          vb[i] = cmul(mk<C>(s * u.x + c * yt.x, s * u.y + c * yt.y), e);
        }
      }
      __syncthreads();
    }
    // converged when a whole sweep found every pair orthogonal to tol
    if (!__syncthreads_or(rotated)) {
      ++sweep;
      break;
    }
  }
  for (int j = warp; j < Cn; j += kSvdWarps) {
    const C* x = W + j * R;
    Rl n2 = 0;
    for (int i = lane; i < R; i += 32) n2 += x[i].x * x[i].x + x[i].y * x[i].y;
    n2 = wsum(n2);
    if (lane == 0) sig[j] = sqrt(n2);
  }
  if (w_sm)
    for (int i = threadIdx.x; i < R * Cn; i += blockDim.x) Wg[i] = W[i];
  if (v_sm)
    for (int i = threadIdx.x; i < Cn * Cn; i += blockDim.x) Vg[i] = V[i];
  if (threadIdx.x == 0) *sweeps_out = sweep;
}

template <typename TO, typename C>
__device__ __forceinline__ TO to_out(C v) {
  TO r;
  r.x = v.x;
  r.y = v.y;
  return r;
}

// B (m x chi) = U_chi sqrt(S), C (chi x n) = sqrt(S) V_chi^H for A (m x n)
// from the Jacobi result of W = A (m >= n: U_j = W_j / s_j) or of W = A^H
// (m < n: A = V S U^H with U_j = W_j / s_j).  order[j] is the column of the
// j-th largest singular value; every selected s_j is positive.
template <typename Rl, typename TB, typename TC>
__global__ void k_svd_factors(const typename Cx<Rl>::T* __restrict__ W, const typename Cx<Rl>::T* __restrict__ V,
                              const Rl* __restrict__ sig, const int* __restrict__ order, int chi, int64_t m,
                              int64_t n, TB* __restrict__ B, TC* __restrict__ Cm) {
  using C = typename Cx<Rl>::T;
  const bool tr = m < n;
  const int64_t R = tr ? n : m;
  const int64_t Cn = tr ? m : n;
  const int64_t nb = m * chi, total = nb + (int64_t)chi * n;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    if (i < nb) {
      const int64_t r = i % m;
      const int o = order[i / m];
      const Rl q = sqrt(sig[o]);
      C v;
      if (!tr) {
        const C w = W[r + R * o];
        v = mk<C>(w.x / q, w.y / q);
      } else {
        const C w = V[r + Cn * o];
        v = mk<C>(w.x * q, w.y * q);
      }
      B[i] = to_out<TB>(v);
    } else {
      const int64_t t = i - nb;
      const int64_t k = t / chi;
      const int o = order[t % chi];
      const Rl q = sqrt(sig[o]);
      C v;
      if (!tr) {
        const C w = cconj(V[k + Cn * o]);
        v = mk<C>(w.x * q, w.y * q);
      } else {
        const C w = cconj(W[k + R * o]);
        v = mk<C>(w.x / q, w.y / q);
      }
      Cm[t] = to_out<TC>(v);
    }
  }
}

template <typename Rl>
cudaError_t jacobi_t(const void* A, int64_t m, int64_t n, void* W, void* V, void* sig, int max_sweeps, double tol,
                     int* sweeps, cudaStream_t s) {
  using C = typename Cx<Rl>::T;
  const int64_t R = m < n ? n : m, Cn = m < n ? m : n;
  const size_t wb = (size_t)(R * Cn) * sizeof(C), vb = (size_t)(Cn * Cn) * sizeof(C);
  const size_t cap = kSvdSmemCap;
  const int w_sm = wb <= cap, v_sm = w_sm && wb + vb <= cap;
  const size_t smem = (w_sm ? wb : 0) + (v_sm ? vb : 0);
  cudaError_t e = cudaSuccess;
  // the opt-in counts dynamic shared memory only, but the 48 KB default
  // limit also covers the kernel's static reduction array: always set it
  if (smem > 0)
    e = cudaFuncSetAttribute(k_jacobi_svd<Rl>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_jacobi_svd<Rl><<<1, kSvdThreads, smem, s>>>((const C*)A, (int)m, (int)n, (C*)W, (C*)V, (Rl*)sig, w_sm, v_sm,
                                                 max_sweeps, (Rl)tol, sweeps);
  return cudaGetLastError();
}

template <typename Rl>
cudaError_t factors_t(const void* W, const void* V, const void* sig, const int* order, int chi, int64_t m, int64_t n,
                      int tb, void* B, int tc, void* Cm, cudaStream_t s) {
  using C = typename Cx<Rl>::T;
  const int64_t total = (m + n) * (int64_t)chi;
  if (total == 0) return cudaSuccess;
  const int grid = grid_for(total, 256);
  const C* w = (const C*)W;
  const C* v = (const C*)V;
  const Rl* sg = (const Rl*)sig;
  if (tb == PQ_C128 && tc == PQ_C128)
    k_svd_factors<Rl, double2, double2><<<grid, 256, 0, s>>>(w, v, sg, order, chi, m, n, (double2*)B, (double2*)Cm);
  else if (tb == PQ_C128)
    k_svd_factors<Rl, double2, float2><<<grid, 256, 0, s>>>(w, v, sg, order, chi, m, n, (double2*)B, (float2*)Cm);
  else if (tc == PQ_C128)
    k_svd_factors<Rl, float2, double2><<<grid, 256, 0, s>>>(w, v, sg, order, chi, m, n, (float2*)B, (double2*)Cm);
  else
    k_svd_factors<Rl, float2, float2><<<grid, 256, 0, s>>>(w, v, sg, order, chi, m, n, (float2*)B, (float2*)Cm);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_jacobi_svd(int wt, const void* A, int64_t m, int64_t n, void* W, void* V, void* sig,
                              int max_sweeps, double tol, int* sweeps, cudaStream_t s) {
  return wt == PQ_C128 ? jacobi_t<double>(A, m, n, W, V, sig, max_sweeps, tol, sweeps, s)
                       : jacobi_t<float>(A, m, n, W, V, sig, max_sweeps, tol, sweeps, s);
}

cudaError_t launch_svd_factors(int wt, const void* W, const void* V, const void* sig, const int* order, int chi,
                               int64_t m, int64_t n, int tb, void* B, int tc, void* Cm, cudaStream_t s) {
  return wt == PQ_C128 ? factors_t<double>(W, V, sig, order, chi, m, n, tb, B, tc, Cm, s)
                       : factors_t<float>(W, V, sig, order, chi, m, n, tb, B, tc, Cm, s);
}

}  // namespace pq
