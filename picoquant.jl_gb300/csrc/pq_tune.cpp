// Autotuning support: tuning classes of analysed pairs, the kernel choices
// each can run, and the C ABI that installs a tuned table in a context.
//
// The reference leaves every kernel decision to its array library
// (TensorOperations -> BLAS / cuTENSOR, src/layer1.jl:85-92).  Here the
// library's own rules (analyse_pair, the tile width and orientation rules of
// the exact-accumulation class) are the defaults; the autotuner in the
// Python package times every eligible choice of a tuning class with
// pq_measure_pairs and installs the fastest per class.
#include <algorithm>
#include <cstring>

#include "pq_internal.h"

namespace pq {

namespace {

int ceil_log2(int64_t x) {
  int r = 0;
  while (r < 62 && (int64_t(1) << r) < x) ++r;
  return r;
}

bool tc_precision(int precision) {
  return precision == PQ_PREC_3XTF32 || precision == PQ_PREC_6XTF32 || precision == PQ_PREC_OZAKI ||
         precision == PQ_PREC_OZAKI4 || precision == PQ_PREC_3XBF16;
}

bool sliced_precision(int precision) {
  return precision == PQ_PREC_OZAKI || precision == PQ_PREC_OZAKI4 || precision == PQ_PREC_3XBF16;
}

bool same(const TuneChoice& a, const TuneChoice& b) {
  return a.kclass == b.kclass && a.tile_n == b.tile_n && a.orient == b.orient;
}

}  // namespace

uint64_t tuning_key(int precision, const GemmDesc& d) {
  bool a_unit_k = false, b_unit_k = false;
  for (int i = 0; i < d.nk; ++i) {
    if (d.ksa[i] == 1) a_unit_k = true;
    if (d.ksb[i] == 1) b_unit_k = true;
  }
  return (uint64_t)(precision & 15) | (uint64_t)ceil_log2(d.M) << 4 | (uint64_t)ceil_log2(d.N) << 12 |
         (uint64_t)ceil_log2(d.K) << 20 | (uint64_t)ceil_log2(d.Z) << 28 | (uint64_t)a_unit_k << 36 |
         (uint64_t)b_unit_k << 37;
}

bool choice_eligible(int precision, const PairPlan& p, const TuneChoice& c) {
  if (!p.k_both) return c.kclass == p.kclass && c.tile_n == 0 && c.orient == 0;
  if (c.kclass != KC_TC && (c.tile_n || c.orient)) return false;
  switch (c.kclass) {
    case KC_TC: {
      if (!p.gemm_shape || !tc_precision(precision)) return false;
      GemmDesc g = p.m;
      g.tile_n = c.tile_n;
      g.orient = c.orient;
      if (c.tile_n || c.orient) return sliced_precision(precision) && g.K <= 512 && oz_eligible(g);
      return tc_eligible(precision, g);
    }
    case KC_SKINNY:
      return skinny_eligible(p.m);
    case KC_GEMM:
      return p.gemm_shape || (p.ksize > kGenericKTab && p.M >= 8 && p.N >= 8);
    case KC_GENERIC:
      return true;
    default:
      return false;
  }
}

std::vector<TuneChoice> tuning_candidates(int precision, const PairPlan& p) {
  std::vector<TuneChoice> v;
  v.push_back({(int)p.kclass, p.kclass == KC_TC ? p.m.tile_n : 0, p.kclass == KC_TC ? p.m.orient : 0});
  if (!p.k_both) return v;
  auto add = [&](TuneChoice c) {
    for (const auto& x : v)
      if (same(x, c)) return;
    if (choice_eligible(precision, p, c)) v.push_back(c);
  };
  if (p.gemm_shape && tc_precision(precision)) {
    add({KC_TC, 0, 0});
    if (sliced_precision(precision))
      for (int orient = 1; orient <= 2; ++orient) {
        // tiles no wider than the oriented N needs (a wider tile only adds idle columns)
        const int64_t n = orient == 2 ? p.m.M : p.m.N;
        for (int tn : {16, 32, 64, 128})
          if (tn == 16 || tn / 2 < n) add({KC_TC, tn, orient});
      }
  }
  add({KC_SKINNY, 0, 0});
  add({KC_GEMM, 0, 0});
  add({KC_GENERIC, 0, 0});
  return v;
}

int check_status(Ctx* ctx);

}  // namespace pq

using namespace pq;

extern "C" {

int pq_ctx_set_tuning(pq_ctx* c, int n, const uint64_t* keys, const int32_t* choices) {
  if (!c) return PQ_ERR_INVALID;
  Ctx* ctx = &c->impl;
  if (n < 0 || (n && (!keys || !choices))) return fail(ctx, PQ_ERR_INVALID, "set_tuning: bad arguments");
  TuningTable t;
  for (int i = 0; i < n; ++i) {
    TuneChoice ch{choices[3 * i], choices[3 * i + 1], choices[3 * i + 2]};
    const bool ok_class = ch.kclass == KC_GENERIC || ch.kclass == KC_GEMM || ch.kclass == KC_TC ||
                          ch.kclass == KC_SKINNY;
    const bool ok_tile = ch.tile_n == 0 || ch.tile_n == 16 || ch.tile_n == 32 || ch.tile_n == 64 || ch.tile_n == 128;
    if (!ok_class || !ok_tile || ch.orient < 0 || ch.orient > 2)
      return fail(ctx, PQ_ERR_INVALID, "set_tuning: entry " + std::to_string(i) + " is not a kernel choice");
    t[keys[i]] = ch;
  }
  ctx->tuning.swap(t);
  return PQ_OK;
}

int pq_device_name(int device, char* out, int cap) {
  if (!out || cap < 1) return PQ_ERR_INVALID;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return PQ_ERR_CUDA;
  std::strncpy(out, prop.name, (size_t)cap - 1);
  out[cap - 1] = 0;
  return PQ_OK;
}

int pq_ctx_tuning_size(pq_ctx* c, int* n) {
  if (!c || !n) return PQ_ERR_INVALID;
  *n = (int)c->impl.tuning.size();
  return PQ_OK;
}

int pq_pair_tuning(pq_ctx* c, int a_rank, int b_rank, const int32_t* labels, const int64_t* dims, uint64_t* key,
                   int max_choices, int32_t* choices, int* n_choices) {
  if (!c) return PQ_ERR_INVALID;
  Ctx* ctx = &c->impl;
  if (a_rank < 0 || b_rank < 0 || a_rank > PQ_MAX_RANK || b_rank > PQ_MAX_RANK || !key || !n_choices ||
      ((a_rank + b_rank) && (!labels || !dims)) || max_choices < 0 || (max_choices && !choices))
    return fail(ctx, PQ_ERR_INVALID, "pair_tuning: bad arguments");
  std::vector<int> la(labels, labels + a_rank), lb(labels + a_rank, labels + a_rank + b_rank);
  std::vector<int64_t> da(dims, dims + a_rank), db(dims + a_rank, dims + a_rank + b_rank);
  PairPlan pp;
  std::string err;
  if (!analyse_pair(la, da, lb, db, symdiff_labels(la, lb), ctx->precision, pp, err))
    return fail(ctx, PQ_ERR_INVALID, "pair_tuning: " + err);
  *key = tuning_key(ctx->precision, pp.m);
  std::vector<TuneChoice> v = tuning_candidates(ctx->precision, pp);
  *n_choices = (int)v.size();
  for (int i = 0; i < (int)v.size() && i < max_choices; ++i) {
    choices[3 * i] = v[i].kclass;
    choices[3 * i + 1] = v[i].tile_n;
    choices[3 * i + 2] = v[i].orient;
  }
  return PQ_OK;
}

}  // extern "C"
