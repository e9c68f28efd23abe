// Internal declarations shared by the pqgb300 translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/pqgb300.h"

namespace pq {

constexpr int kMaxModes = 32;   // modes of one side of a pair after merging
constexpr int kGenericKTab = 2048;  // K <= this runs in the table-driven SIMT kernel

// One operand / result mode after analysis: its extent and its strides (in
// elements) in A, B and C.  A stride of 0 means the mode is absent there.
struct Mode {
  int64_t dim;
  int64_t sa, sb, sc;
};

// Kernel-facing description of one pairwise contraction
//   C[c] = sum_k A[oa(c) + ka(k)] * B[ob(c) + kb(k)]
// where c runs over the C modes in C storage order (column-major).
struct GenericDesc {
  int nc;            // number of (merged) C modes
  int nk;            // number of (merged) contracted modes
  int pow2;          // 1 if every C and K dim is a power of two
  int pad_;
  int64_t csize, ksize;
  int64_t cdim[kMaxModes], csa[kMaxModes], csb[kMaxModes];
  int32_t clog[kMaxModes];
  int64_t kdim[kMaxModes], ksa[kMaxModes], ksb[kMaxModes];
  int32_t klog[kMaxModes];
};

// Description for the tiled GEMM-class kernel:
//   C[cm(m)+cn(n)+cb(z)] = sum_k A[am(m)+ak(k)+ab(z)] * B[bk(k)+bn(n)+bb(z)]
struct GemmDesc {
  int64_t M, N, K, Z;
  int nm, nn, nk, nz;
  int64_t mdim[kMaxModes], msa[kMaxModes], msc[kMaxModes];
  int64_t ndim[kMaxModes], nsb[kMaxModes], nsc[kMaxModes];
  int64_t kdim[kMaxModes], ksa[kMaxModes], ksb[kMaxModes];
  int64_t zdim[kMaxModes], zsa[kMaxModes], zsb[kMaxModes], zsc[kMaxModes];
  // Autotuned launch shape of the exact-accumulation tensor-core class:
  // tile_n = columns per tile (16/32/64/128; 0 = the default rule), orient =
  // 1 to run as given, 2 to run as C = B x A (0 = the default rule).
  int tile_n, orient;
};

enum KernelClass : int { KC_GENERIC = 0, KC_GEMM = 1, KC_TC = 2, KC_COPY = 3, KC_SKINNY = 4 };
// Skinny pairs (pq_skinny.cu): a large operand (>= kSkinnyMinRows rows over
// its free modes) against a small one, K <= kSkinnyK, the small side's free
// extent <= kSkinnyN, no batch modes.
constexpr int kSkinnyK = 16, kSkinnyN = 16;
constexpr int64_t kSkinnyMinRows = 4096;
// SIMT GEMM tile shapes: 64x64, 256x16 (narrow N), 16x256 (narrow M).
enum GemmShape : int { GEMM_SQUARE = 0, GEMM_TALL = 1, GEMM_WIDE = 2 };
struct GemmDesc;
int gemm_tile_shape(const GemmDesc& d);

// Host-side analysis of one contraction.
struct PairPlan {
  std::vector<int> c_labels;   // result labels in storage order
  std::vector<int64_t> c_dims;
  int64_t csize = 1, ksize = 1, asize = 1, bsize = 1;
  int64_t M = 1, N = 1, Z = 1;
  KernelClass kclass = KC_GENERIC;
  GenericDesc g;
  GemmDesc m;
  int64_t run_a = 1, run_b = 1;   // extent of the unit-stride run of A / B that
                                   // is read contiguously (coalescing feature)
  bool k_both = false;      // every contracted mode is in both operands
  bool gemm_shape = false;  // large enough for the tiled GEMM classes
  bool tuned = false;       // the class came from the tuning table
};

// Autotuning (pq_tune.cpp).  A tuning class is the pair's precision mode, the
// ceil-log2 of its M, N, K and batch extents and whether the unit-stride mode
// of A / of B is contracted; a choice is a kernel class plus, for the
// exact-accumulation tensor-core class, a tile width and an orientation.
struct TuneChoice {
  int kclass;
  int tile_n;
  int orient;
};
using TuningTable = std::unordered_map<uint64_t, TuneChoice>;
uint64_t tuning_key(int precision, const GemmDesc& d);
// Every choice the kernels can run for this analysed pair (the default first).
std::vector<TuneChoice> tuning_candidates(int precision, const PairPlan& p);
bool choice_eligible(int precision, const PairPlan& p, const TuneChoice& c);

// Analyse C = A x B given labels (A/B storage order) and the result labels
// (storage order).  Labels of A or B absent from C are summed.  Returns
// false with `err` set on inconsistent input.  With a tuning table, a pair
// whose class is in the table runs the table's choice when eligible.
bool analyse_pair(const std::vector<int>& la, const std::vector<int64_t>& da,
                  const std::vector<int>& lb, const std::vector<int64_t>& db,
                  const std::vector<int>& lc, int precision, PairPlan& out, std::string& err,
                  const TuningTable* tune = nullptr);

// Result labels in the reference's order: A's labels not in B (A order),
// then B's labels not in A (B order).
std::vector<int> symdiff_labels(const std::vector<int>& la, const std::vector<int>& lb);

struct Tensor {
  void* ptr = nullptr;
  int dtype = PQ_C128;  // storage element type
  std::vector<int64_t> dims;
  int64_t size = 1;
  size_t bytes = 0;
};

struct Ctx {
  int device = 0;
  int precision = PQ_PREC_C128;
  size_t elem = 16;   // bytes per stored element
  cudaStream_t stream = nullptr;
  cudaMemPool_t pool = nullptr;
  int* d_status = nullptr;          // device status word (0 = ok)
  std::unordered_map<int64_t, Tensor> tensors;
  std::string last_error;
  int64_t mem_cap = 0;
  int64_t mem_in_use = 0;
  int64_t launches = 0;
  // batched uploads (pq_save_tensors): pinned host and device staging,
  // reused across calls; the host side is rewritten only after the event of
  // the previous batch's copy has completed
  void* h_stage = nullptr;
  size_t h_stage_cap = 0;
  void* d_stage = nullptr;
  size_t d_stage_cap = 0;
  cudaEvent_t stage_done = nullptr;
  // Mixed-precision contexts store tensors of at most this many elements as
  // complex128 (gates, per-qubit tensors: cheap, and their rounding would
  // dominate the error) and larger ones as complex64.
  int64_t small_elems = int64_t(1) << 16;
  // Autotuned choices per tuning class (pq_ctx_set_tuning), consulted when
  // pairs are analysed (contractions, plans, measurements).
  TuningTable tuning;
};

inline size_t elem_bytes(int dt) { return dt == PQ_C128 ? 16 : 8; }
// Storage type of a tensor of `n` elements in this context.
inline int storage_dtype(const Ctx* ctx, int64_t n) {
  if (ctx->precision == PQ_PREC_C128) return PQ_C128;
  return n <= ctx->small_elems ? PQ_C128 : PQ_C64;
}

// Status helpers: set the context error and return the code.
int fail(Ctx* ctx, int code, const std::string& msg);
int cuda_fail(Ctx* ctx, cudaError_t e, const char* what);

// Stream-ordered device allocation accounted against the context cap.
int dev_alloc(Ctx* ctx, size_t bytes, void** p);
void dev_free(Ctx* ctx, void* p, size_t bytes);

// ---- kernel launchers (pq_kernels.cu, pq_gemm.cu, pq_skinny.cu) -----------
// Element types are PQ_C64 / PQ_C128 per operand.  All launches are
// asynchronous on `stream` and return the launch error.
cudaError_t launch_generic(int ta, int tb, int tc, const void* A, const void* B, void* C,
                           const GenericDesc& d, cudaStream_t stream);
cudaError_t launch_gemm(int ta, int tb, int tc, const void* A, const void* B, void* C,
                        const GemmDesc& d, cudaStream_t stream);
// Up to kGroupMax independent small generic steps (complex128 operands and
// result, K <= kGroupK) in one launch; member m runs on blocks
// [blk[m], blk[m+1]) with descriptor descs[desc[m]] (device table).
constexpr int kGroupMax = 64, kGroupK = 256;
struct GenericGroup {
  int n;
  int blk[kGroupMax + 1];
  int desc[kGroupMax];
  const void* A[kGroupMax];
  const void* B[kGroupMax];
  void* C[kGroupMax];
};
cudaError_t launch_generic_group(const GenericGroup& g, const GenericDesc* d_descs, cudaStream_t stream);
bool skinny_eligible(const GemmDesc& d);
cudaError_t launch_skinny(int ta, int tb, int tc, const void* A, const void* B, void* C,
                          const GemmDesc& d, cudaStream_t stream);
// out[c] = in[base + sum_i idx_i * stride_i] over `d` (uses csa as input
// strides, C storage column-major), converting tin -> tout.
cudaError_t launch_permute(int tin, int tout, const void* in, int64_t base, void* out,
                           const GenericDesc& d, cudaStream_t stream);
cudaError_t launch_gather(int dt, const void* in, const int64_t* d_idx, int64_t n,
                          void* out, cudaStream_t stream);
// One launch copying n byte ranges from a device staging buffer to their
// destinations (src offsets 16-byte aligned).
struct CopyJob {
  int64_t src_off;
  void* dst;
  int64_t bytes;
};
cudaError_t launch_scatter(const void* src, const CopyJob* d_jobs, int n, cudaStream_t stream);
// Batched leaf gather for slicing: out[x + xs*b] = in[x_off(x) + slice_off(s0+b)]
// for b < nb, where x runs over `d` (csa = input strides of the kept modes)
// and the slice offset is the mixed-radix digits of (s0+b) over the sliced
// dims times their strides in `in`.  Entries with s0+b >= s_end are zero.
cudaError_t launch_slice_gather(int dt, const void* in, void* out, const GenericDesc& d,
                                int nsl, const int64_t* sl_dim, const int64_t* sl_stride,
                                int64_t s0, int64_t nb, int64_t s_end, cudaStream_t stream);
// Neumaier FP64 sum over the batch axis: acc[e] += sum_b X[e + n*b].
// FP64 squared 2-norm of n complex elements into *out (device); `part`
// holds 2 * norm2_blocks(n) doubles of scratch.
int norm2_blocks(int64_t n);
cudaError_t launch_norm2(int dt, const void* X, int64_t n, double* part, double* out, cudaStream_t stream);
cudaError_t launch_slice_sum(int dt, const void* X, int64_t n, int64_t nb,
                             double* acc, double* comp, cudaStream_t stream);
// Split-precision tensor-core GEMM-class contraction (pq_tc.cu).  Returns
// cudaErrorNotSupported when the shape is not eligible.
cudaError_t launch_tc(int precision, int ta, int tb, int tc, const void* A, const void* B, void* C,
                      const GemmDesc& d, void* scratch, size_t scratch_bytes, int* status, cudaStream_t stream);
size_t tc_scratch_bytes(int precision, const GemmDesc& d);
bool tc_eligible(int precision, const GemmDesc& d);
int tc_launch_count(int precision, const GemmDesc& d);  // kernels one launch_tc issues
// Exact-accumulation (Ozaki scheme, bf16 slices) tensor-core contraction
// (pq_oz.cu), used by launch_tc when K <= 512: 5 slices for PQ_PREC_OZAKI,
// 4 for PQ_PREC_OZAKI4, 3 for PQ_PREC_3XBF16.
bool oz_eligible(const GemmDesc& d);
size_t oz_scratch_bytes(int slices, const GemmDesc& d);
cudaError_t launch_oz(int slices, int ta, int tb, int tc, const void* A, const void* B, void* C, const GemmDesc& d,
                      void* scratch, size_t scratch_bytes, int* status, cudaStream_t stream);

// Device SVD for bond splits (pq_svd.cu): one-sided Jacobi on A (m x n,
// column-major, element type wt: PQ_C64 -> complex FP32 arithmetic, PQ_C128
// -> complex FP64), through W = A (m >= n) or W = A^H (m < n), R x Cn with
// R = max(m, n), Cn = min(m, n).  Writes W (R x Cn) and V (Cn x Cn) of type
// wt and sig[Cn] (float or double, unsorted column norms).
cudaError_t launch_jacobi_svd(int wt, const void* A, int64_t m, int64_t n, void* W, void* V, void* sig,
                              int max_sweeps, double tol, int* sweeps, cudaStream_t s);
// B (m x chi) = U sqrt(S) and C (chi x n) = sqrt(S) V^H of the chi singular
// values order[0..chi) (columns of W), stored as tb / tc.
cudaError_t launch_svd_factors(int wt, const void* W, const void* V, const void* sig, const int* order, int chi,
                               int64_t m, int64_t n, int tb, void* B, int tc, void* Cm, cudaStream_t s);

}  // namespace pq

struct pq_ctx {
  pq::Ctx impl;
};
