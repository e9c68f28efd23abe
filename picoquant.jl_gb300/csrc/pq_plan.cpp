// Plan executor: compile a whole pairwise contraction of a network once, then
// execute it many times (directly, from a captured CUDA graph, or sliced in
// batches with an FP64 compensated sum over slices).
//
// Follows the plan-execution semantics of src/layer2.jl:294-321
// (contract_network! with a pair plan) and the slicing of
// src/layer2/slicing.jl:37-110, with the GB300-specific changes:
//   * all intermediate buffers live in one arena whose offsets come from a
//     liveness analysis at compile time (no allocation while executing);
//   * the final permutation to the requested output order is folded into the
//     last contraction's index map;
//   * slices are not materialised as separate networks: sliced leaves are
//     gathered for a batch of slices at once (the batch becomes a shared mode
//     of every intermediate that depends on a sliced leaf) and sub-trees that
//     touch no sliced leaf are computed once per run.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <set>

#include "pq_internal.h"

namespace pq {
int alloc_tensor(Ctx* ctx, const std::vector<int64_t>& dims, int dtype, Tensor& t);
int check_status(Ctx* ctx);
}  // namespace pq

using namespace pq;

namespace {

struct Step {
  int x = -1, y = -1;  // SSA operands
  PairPlan pp;
  size_t off = 0;      // arena offset of the result
  size_t bytes = 0;
  bool batched = false;
  bool is_copy = false;  // single-leaf network: result = permuted copy of x
  int ta = PQ_C128, tb = PQ_C128, tc = PQ_C128;  // storage types of A, B, C
  int group = -1;        // launch group of small steps (consecutive steps share it)
};

struct Compiled {
  int nleaves = 0;
  std::vector<std::vector<int>> labels;    // per SSA value
  std::vector<std::vector<int64_t>> dims;  // per SSA value
  std::vector<int> dt;                     // storage type per SSA value
  std::vector<Step> steps;                 // in execution order
  std::vector<int> order;                  // steps' original indices
  size_t arena_bytes = 0;
  size_t scratch_bytes = 0;
  int result_ssa = -1;
  double cmacs = 0;
  int64_t max_elems = 0;
  int64_t launches = 0;
  std::vector<GenericDesc> gdesc;  // descriptors of grouped steps (uploaded per plan)
  std::vector<int> gdesc_of;       // per step: index into gdesc, or -1
};

// Small steps: complex128 generic or skinny contractions of at most
// kGroupSmall result elements and K <= kGroupK.  They are launch-bound one by
// one; in a group they run as generic contractions side by side.
constexpr int64_t kGroupSmall = 1 << 16;

bool groupable(const Step& s) {
  return !s.is_copy && s.y >= 0 && (s.pp.kclass == KC_GENERIC || s.pp.kclass == KC_SKINNY) &&
         s.ta == PQ_C128 && s.tb == PQ_C128 && s.tc == PQ_C128 && s.pp.csize >= 1 && s.pp.csize <= kGroupSmall &&
         s.pp.g.ksize <= kGroupK;
}

// Launch groups of small steps, in two parts.
//  1. Hoisted: every small step whose producers are leaves or hoisted small
//     steps (the per-qubit chains of small gate tensors that do not wait for
//     any large intermediate).  These run first, by dependency level -- one
//     more than the highest level of a hoisted producer -- and each (level,
//     batched flag) becomes launches of up to kGroupMax steps, so the chains
//     of the whole plan advance together.
//  2. The rest keep their order; within every maximal run of consecutive small
//     steps (same batched flag) the steps are reordered by dependency level
//     inside the run and each level becomes one launch of up to kGroupMax.
// Every step still follows its producers, and the batched (per slice batch)
// and unbatched (once per call) steps keep their relative orders, so both the
// plain and the sliced executors stay valid.
void form_groups(Compiled& cp) {
  const int n = (int)cp.steps.size();
  std::vector<int> prod(cp.labels.size(), -1);
  for (int i = 0; i < n; ++i) prod[cp.nleaves + cp.order[i]] = i;
  std::vector<Step> steps;
  std::vector<int> order;
  steps.reserve(n);
  order.reserve(n);
  int gid = 0;
  // emit the steps idx[a..b) (original positions) as one launch group when
  // there are at least two of them
  auto emit = [&](const std::vector<int>& idx, size_t a, size_t b) {
    const bool grp = b - a >= 2;
    for (size_t c = a; c < b; ++c) {
      Step st = cp.steps[idx[c]];
      st.group = grp ? gid : -1;
      steps.push_back(st);
      order.push_back(cp.order[idx[c]]);
    }
    if (grp) ++gid;
  };
  // 1. hoisted small steps
  std::vector<char> hoisted(n, 0);
  std::vector<int> hlevel(n, 0);
  for (int i = 0; i < n; ++i) {
    if (!groupable(cp.steps[i])) continue;
    bool ok = true;
    int L = 0;
    for (int v : {cp.steps[i].x, cp.steps[i].y}) {
      if (v < 0 || v < cp.nleaves) continue;
      const int pi = prod[v];
      if (pi < 0 || !hoisted[pi]) {
        ok = false;
        break;
      }
      L = std::max(L, hlevel[pi] + 1);
    }
    hoisted[i] = ok;
    hlevel[i] = L;
  }
  std::vector<int> hidx;
  for (int i = 0; i < n; ++i)
    if (hoisted[i]) hidx.push_back(i);
  std::stable_sort(hidx.begin(), hidx.end(), [&](int a, int b) {
    if (hlevel[a] != hlevel[b]) return hlevel[a] < hlevel[b];
    return (int)cp.steps[a].batched < (int)cp.steps[b].batched;
  });
  for (size_t a = 0; a < hidx.size();) {
    size_t b = a;
    while (b < hidx.size() && hlevel[hidx[b]] == hlevel[hidx[a]] &&
           cp.steps[hidx[b]].batched == cp.steps[hidx[a]].batched && b - a < (size_t)kGroupMax)
      ++b;
    emit(hidx, a, b);
    a = b;
  }
  // 2. the rest, runs of consecutive small steps grouped by level
  std::vector<int> rest;
  for (int i = 0; i < n; ++i)
    if (!hoisted[i]) rest.push_back(i);
  const int nr = (int)rest.size();
  std::vector<int> rpos(n, -1);
  for (int q = 0; q < nr; ++q) rpos[rest[q]] = q;
  for (int i = 0; i < nr;) {
    const Step& si = cp.steps[rest[i]];
    if (!groupable(si)) {
      emit(rest, i, i + 1);
      ++i;
      continue;
    }
    int j = i;
    while (j < nr && groupable(cp.steps[rest[j]]) && cp.steps[rest[j]].batched == si.batched) ++j;
    std::vector<int> lvl(j - i, 0);
    for (int t = i; t < j; ++t) {
      int L = 0;
      for (int v : {cp.steps[rest[t]].x, cp.steps[rest[t]].y}) {
        if (v < 0 || v < cp.nleaves) continue;
        const int pi = prod[v];
        const int q = pi >= 0 ? rpos[pi] : -1;
        if (q >= i && q < t) L = std::max(L, lvl[q - i] + 1);
      }
      lvl[t - i] = L;
    }
    std::vector<int> idx(j - i);
    for (int t = 0; t < j - i; ++t) idx[t] = t;
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return lvl[a] < lvl[b]; });
    std::vector<int> run(j - i);
    for (int t = 0; t < j - i; ++t) run[t] = rest[i + idx[t]];
    for (size_t a = 0; a < run.size();) {
      size_t b = a;
      while (b < run.size() && lvl[idx[b]] == lvl[idx[a]] && b - a < (size_t)kGroupMax) ++b;
      emit(run, a, b);
      a = b;
    }
    i = j;
  }
  cp.steps.swap(steps);
  cp.order.swap(order);
  cp.gdesc.clear();
  cp.gdesc_of.assign(cp.steps.size(), -1);
  for (size_t k = 0; k < cp.steps.size(); ++k)
    if (cp.steps[k].group >= 0) {
      cp.gdesc_of[k] = (int)cp.gdesc.size();
      cp.gdesc.push_back(cp.steps[k].pp.g);
    }
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Liveness-driven first-fit arena assignment.  `pinned[v]` values are never
// released once computed (used for sliced execution: values computed once and
// read by the batched steps).  They are also never placed in released space:
// the sliced executor runs every unbatched step before the batched ones, so a
// block that a batched value used earlier in the step order is written again
// by the batched pass after the pinned value was stored there.
void assign_arena(Compiled& cp, const std::vector<char>& pinned) {
  const int nv = (int)cp.labels.size();
  std::vector<int> last_use(nv, -1);
  for (int i = 0; i < (int)cp.steps.size(); ++i) {
    last_use[cp.steps[i].x] = i;
    if (cp.steps[i].y >= 0) last_use[cp.steps[i].y] = i;
  }
  std::map<size_t, size_t> free_blocks;  // offset -> size
  size_t top = 0;
  auto take = [&](size_t sz) -> size_t {
    for (auto it = free_blocks.begin(); it != free_blocks.end(); ++it) {
      if (it->second >= sz) {
        size_t off = it->first, rem = it->second - sz;
        free_blocks.erase(it);
        if (rem) free_blocks[off + sz] = rem;
        return off;
      }
    }
    size_t off = top;
    top += sz;
    return off;
  };
  auto give = [&](size_t off, size_t sz) {
    auto it = free_blocks.emplace(off, sz).first;
    auto nx = std::next(it);
    if (nx != free_blocks.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_blocks.erase(nx);
    }
    if (it != free_blocks.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_blocks.erase(it);
      }
    }
  };
  std::vector<size_t> voff(nv, 0), vsz(nv, 0);
  // a launch group runs concurrently: all its results are placed before any
  // of its inputs is released
  const int n = (int)cp.steps.size();
  for (int i = 0; i < n;) {
    int j = i + 1;
    if (cp.steps[i].group >= 0)
      while (j < n && cp.steps[j].group == cp.steps[i].group) ++j;
    for (int t = i; t < j; ++t) {
      Step& s = cp.steps[t];
      const int r = cp.nleaves + cp.order[t];
      const size_t sz = align_up(std::max<size_t>(s.bytes, 16), 256);
      if (pinned[r]) {
        s.off = top;
        top += sz;
      } else {
        s.off = take(sz);
      }
      voff[r] = s.off;
      vsz[r] = sz;
    }
    for (int t = i; t < j; ++t)
      for (int v : {cp.steps[t].x, cp.steps[t].y}) {
        if (v < cp.nleaves || v < 0) continue;
        if (last_use[v] == t && !pinned[v] && v != cp.result_ssa) give(voff[v], vsz[v]);
      }
    i = j;
  }
  cp.arena_bytes = top;
}

}  // namespace

struct pq_plan {
  Ctx* ctx = nullptr;
  int nleaves = 0;
  int nlabels = 0;
  std::vector<std::vector<int>> leaf_labels;
  std::vector<std::vector<int64_t>> leaf_dims;
  std::vector<int64_t> label_dims;
  std::vector<int> steps_in;  // 2*n_steps SSA operands as given
  std::vector<int> out_labels;
  Compiled cp;
  void* arena = nullptr;
  size_t arena_cap = 0;
  void* scratch = nullptr;
  size_t scratch_cap = 0;
  // device tables of the grouped steps' descriptors (cp, scp)
  void* d_gdesc = nullptr;
  size_t d_gdesc_bytes = 0;
  void* d_sgdesc = nullptr;
  size_t d_sgdesc_bytes = 0;
  // graph
  cudaGraphExec_t gexec = nullptr;
  std::vector<const void*> graph_ptrs;
  // sliced execution state
  std::vector<int> sl_labels;
  int sl_batch = 0;
  Compiled scp;
  std::vector<int> sl_leaf_of;             // SSA leaf -> index into sl_leafbuf (or -1)
  std::vector<size_t> sl_leaf_off;         // offsets of gathered leaves in arena (after scp arena)
  std::vector<GenericDesc> sl_leaf_desc;
  std::vector<std::vector<int64_t>> sl_leaf_sdim, sl_leaf_sstride;
  std::vector<int> sl_leaf_dt;             // storage type of each gathered leaf
  size_t sl_total_bytes = 0;
  double* d_acc = nullptr;  // 2*n complex sum + 2*n compensation
  int64_t out_elems = 0;
  // the sliced run as a CUDA graph: captured on the second consecutive call
  // with the same device pointers and arguments, replayed after that
  cudaGraphExec_t sgexec = nullptr;
  std::vector<const void*> sg_key;
  std::vector<int64_t> sg_args;
  int64_t sg_launches = 0;
  int sg_seen = 0;
};

namespace {

// Compile `steps` (SSA pairs in execution order) for the given leaf labels.
bool compile(const Ctx* ctx, const std::vector<std::vector<int>>& leaf_labels,
             const std::vector<int64_t>& label_dims, const std::vector<int>& steps,
             const std::vector<int>& out_labels, const std::vector<int>& exec_order,
             const std::vector<char>* batched_leaf, Compiled& cp, std::string& err,
             const std::vector<int>* leaf_dt = nullptr) {
  cp = Compiled();
  const int precision = ctx->precision;
  const int nl = (int)leaf_labels.size();
  const int ns = (int)steps.size() / 2;
  cp.nleaves = nl;
  cp.labels.assign(nl + std::max(ns, 1), {});
  cp.dims.assign(nl + std::max(ns, 1), {});
  cp.dt.assign(nl + std::max(ns, 1), PQ_C128);
  for (int i = 0; i < nl; ++i) {
    cp.labels[i] = leaf_labels[i];
    for (int l : leaf_labels[i]) {
      if (l < 0 || l >= (int)label_dims.size()) {
        err = "leaf label out of range";
        return false;
      }
      cp.dims[i].push_back(label_dims[l]);
    }
    int64_t sz = 1;
    for (auto d : cp.dims[i]) sz *= d;
    cp.dt[i] = leaf_dt ? (*leaf_dt)[i] : storage_dtype(ctx, sz);
  }
  for (int l : out_labels)
    if (l < 0 || l >= (int)label_dims.size()) {
      err = "output label out of range";
      return false;
    }
  // label multiplicities among live values (+ output)
  std::vector<int> cnt(label_dims.size(), 0);
  for (int i = 0; i < nl; ++i)
    for (int l : leaf_labels[i]) cnt[l]++;
  std::set<int> outset(out_labels.begin(), out_labels.end());
  for (int l : out_labels) cnt[l]++;
  std::vector<char> live(nl + ns, 0), defined(nl + ns, 0), batched(nl + ns, 0);
  for (int i = 0; i < nl; ++i) {
    live[i] = defined[i] = 1;
    if (batched_leaf) batched[i] = (*batched_leaf)[i];
  }
  if (ns == 0) {
    if (nl != 1) {
      err = "a plan without steps needs exactly one leaf";
      return false;
    }
    // single leaf: result is the leaf permuted into output order
    Step s;
    s.x = 0;
    s.is_copy = true;
    std::vector<int> la = leaf_labels[0];
    std::set<int> ls(la.begin(), la.end());
    if (ls != outset || out_labels.size() != la.size()) {
      err = "output labels do not match the single leaf";
      return false;
    }
    if (!analyse_pair(la, cp.dims[0], {}, {}, out_labels, precision, s.pp, err)) return false;
    s.ta = s.tb = cp.dt[0];
    s.tc = cp.dt[0];
    s.bytes = (size_t)s.pp.csize * elem_bytes(s.tc);
    cp.dt[nl] = s.tc;
    cp.steps.push_back(s);
    cp.order.push_back(0);
    cp.labels[nl] = out_labels;
    cp.dims[nl] = s.pp.c_dims;
    cp.result_ssa = nl;
    cp.max_elems = s.pp.csize;
    cp.launches = 1;
    std::vector<char> pinned(nl + 1, 0);
    assign_arena(cp, pinned);
    return true;
  }
  // first pass in given order to define labels (must be a valid SSA program)
  std::vector<Step> tmp(ns);
  for (int i = 0; i < ns; ++i) {
    int x = steps[2 * i], y = steps[2 * i + 1];
    if (x < 0 || y < 0 || x >= nl + i || y >= nl + i || x == y) {
      err = "step " + std::to_string(i) + " has an invalid operand";
      return false;
    }
    if (!live[x] || !live[y]) {
      err = "step " + std::to_string(i) + " uses a consumed operand";
      return false;
    }
    live[x] = live[y] = 0;
    for (int l : cp.labels[x]) cnt[l]--;
    for (int l : cp.labels[y]) cnt[l]--;
    const bool last = (i == ns - 1);
    std::vector<int> lr;
    if (last) {
      lr = out_labels;
    } else {
      for (int l : cp.labels[x])
        if (cnt[l] > 0) lr.push_back(l);
      for (int l : cp.labels[y])
        if (cnt[l] > 0 && std::find(lr.begin(), lr.end(), l) == lr.end()) lr.push_back(l);
    }
    if (last) {
      // everything not in the output must be summed now
      std::set<int> have(cp.labels[x].begin(), cp.labels[x].end());
      have.insert(cp.labels[y].begin(), cp.labels[y].end());
      for (int l : out_labels)
        if (!have.count(l)) {
          err = "output label " + std::to_string(l) + " does not reach the last step";
          return false;
        }
    }
    int r = nl + i;
    Step& s = tmp[i];
    s.x = x;
    s.y = y;
    s.batched = batched[x] || batched[y];
    batched[r] = s.batched;
    if (!analyse_pair(cp.labels[x], cp.dims[x], cp.labels[y], cp.dims[y], lr, precision, s.pp, err, &ctx->tuning)) {
      err = "step " + std::to_string(i) + ": " + err;
      return false;
    }
    s.ta = cp.dt[x];
    s.tb = cp.dt[y];
    s.tc = storage_dtype(ctx, s.pp.csize);
    cp.dt[r] = s.tc;
    s.bytes = (size_t)s.pp.csize * elem_bytes(s.tc);
    cp.labels[r] = lr;
    cp.dims[r] = s.pp.c_dims;
    for (int l : lr) cnt[l]++;
    live[r] = 1;
  }
  int nlive = 0;
  for (int v = 0; v < nl + ns; ++v) nlive += live[v];
  if (nlive != 1 || !live[nl + ns - 1]) {
    err = "plan does not contract the network to a single tensor (" + std::to_string(nlive) + " left)";
    return false;
  }
  cp.result_ssa = nl + ns - 1;
  for (int i = 0; i < ns; ++i) {
    int idx = exec_order.empty() ? i : exec_order[i];
    cp.steps.push_back(tmp[idx]);
    cp.order.push_back(idx);
    const PairPlan& p = tmp[idx].pp;
    cp.cmacs += (double)p.csize * (double)p.ksize;
    cp.max_elems = std::max(cp.max_elems, p.csize);
    cp.launches += (p.kclass == KC_TC) ? tc_launch_count(ctx->precision, p.m) : 1;
  }
  form_groups(cp);
  cp.launches = 0;
  for (size_t i = 0; i < cp.steps.size(); ++i) {
    const Step& s = cp.steps[i];
    if (s.group >= 0 && i > 0 && cp.steps[i - 1].group == s.group) continue;  // one launch per group
    cp.launches += (s.pp.kclass == KC_TC) ? tc_launch_count(ctx->precision, s.pp.m) : 1;
  }
  size_t sb = 0;
  for (auto& s : cp.steps)
    if (s.pp.kclass == KC_TC) sb = std::max(sb, tc_scratch_bytes(precision, s.pp.m));
  cp.scratch_bytes = sb;
  std::vector<char> pinned(nl + ns, 0);
  if (batched_leaf) {
    // values computed once (not batched) but read by batched steps stay put
    for (auto& s : cp.steps)
      if (s.batched)
        for (int v : {s.x, s.y})
          if (v >= nl && !batched[v]) pinned[v] = 1;
  }
  assign_arena(cp, pinned);
  return true;
}

cudaError_t run_step(pq_plan* p, const Step& s, const void* A, const void* B, void* C) {
  Ctx* ctx = p->ctx;
  ctx->launches += (s.pp.kclass == KC_TC) ? tc_launch_count(ctx->precision, s.pp.m) : 1;
  if (s.is_copy) return launch_permute(s.ta, s.tc, A, 0, C, s.pp.g, ctx->stream);
  switch (s.pp.kclass) {
    case KC_TC:
      return launch_tc(ctx->precision, s.ta, s.tb, s.tc, A, B, C, s.pp.m, p->scratch, p->scratch_cap,
                       ctx->d_status, ctx->stream);
    case KC_GEMM:
      return launch_gemm(s.ta, s.tb, s.tc, A, B, C, s.pp.m, ctx->stream);
    case KC_SKINNY:
      return launch_skinny(s.ta, s.tb, s.tc, A, B, C, s.pp.m, ctx->stream);
    default:
      return launch_generic(s.ta, s.tb, s.tc, A, B, C, s.pp.g, ctx->stream);
  }
}

// Pointers of every SSA value for one execution.
void resolve(pq_plan* p, const Compiled& cp, const std::vector<const void*>& leaf_ptrs,
             std::vector<const void*>& vptr) {
  vptr.assign(cp.labels.size(), nullptr);
  for (int i = 0; i < cp.nleaves; ++i) vptr[i] = leaf_ptrs[i];
  for (size_t i = 0; i < cp.steps.size(); ++i)
    vptr[cp.nleaves + cp.order[i]] = (const char*)p->arena + cp.steps[i].off;
}

int ensure_buffers(pq_plan* p, size_t arena, size_t scratch) {
  Ctx* ctx = p->ctx;
  if (arena > p->arena_cap) {
    if (p->arena) dev_free(ctx, p->arena, p->arena_cap);
    p->arena = nullptr;
    p->arena_cap = 0;
    int st = dev_alloc(ctx, arena, &p->arena);
    if (st) return st;
    p->arena_cap = arena;
    if (p->gexec) {
      cudaGraphExecDestroy(p->gexec);
      p->gexec = nullptr;
    }
  }
  if (scratch > p->scratch_cap) {
    if (p->scratch) dev_free(ctx, p->scratch, p->scratch_cap);
    p->scratch = nullptr;
    p->scratch_cap = 0;
    int st = dev_alloc(ctx, scratch, &p->scratch);
    if (st) return st;
    p->scratch_cap = scratch;
  }
  return PQ_OK;
}

int leaf_pointers(pq_plan* p, const int64_t* leaf_ids, std::vector<const void*>& ptrs) {
  Ctx* ctx = p->ctx;
  ptrs.resize(p->nleaves);
  for (int i = 0; i < p->nleaves; ++i) {
    auto it = ctx->tensors.find(leaf_ids[i]);
    if (it == ctx->tensors.end())
      return fail(ctx, PQ_ERR_NOT_FOUND, "plan: no tensor " + std::to_string(leaf_ids[i]) + " for leaf " +
                                             std::to_string(i));
    const Tensor& t = it->second;
    // a leaf may be stored with any shape whose size matches (e.g. a reshaped
    // gate); its labels' extents define the interpretation
    int64_t want = 1;
    for (auto d : p->leaf_dims[i]) want *= d;
    if (t.size != want)
      return fail(ctx, PQ_ERR_INVALID, "plan: tensor " + std::to_string(leaf_ids[i]) + " has " +
                                           std::to_string(t.size) + " elements, leaf " + std::to_string(i) +
                                           " needs " + std::to_string(want));
    if (t.dtype != p->cp.dt[i])
      return fail(ctx, PQ_ERR_INVALID, "plan: tensor " + std::to_string(leaf_ids[i]) +
                                           " has a different storage type than the plan expects");
    ptrs[i] = t.ptr;
  }
  return PQ_OK;
}

int launch_all(pq_plan* p, const Compiled& cp, const std::vector<const void*>& leaf_ptrs, bool only_batched,
               bool only_unbatched) {
  Ctx* ctx = p->ctx;
  std::vector<const void*> vptr;
  resolve(p, cp, leaf_ptrs, vptr);
  const GenericDesc* dd = (const GenericDesc*)(&cp == &p->scp ? p->d_sgdesc : p->d_gdesc);
  const size_t n = cp.steps.size();
  for (size_t i = 0; i < n; ++i) {
    const Step& s = cp.steps[i];
    if (only_batched && !s.batched) continue;
    if (only_unbatched && s.batched) continue;
    if (s.group >= 0 && dd) {
      GenericGroup g;
      g.n = 0;
      int blocks = 0;
      size_t j = i;
      for (; j < n && cp.steps[j].group == s.group; ++j) {
        const Step& t = cp.steps[j];
        g.blk[g.n] = blocks;
        g.desc[g.n] = cp.gdesc_of[j];
        g.A[g.n] = vptr[t.x];
        g.B[g.n] = vptr[t.y];
        g.C[g.n] = (char*)p->arena + t.off;
        blocks += (int)std::min<int64_t>((t.pp.csize + 255) / 256, 64);
        g.n++;
      }
      g.blk[g.n] = blocks;
      ctx->launches += 1;
      cudaError_t e = launch_generic_group(g, dd, ctx->stream);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "plan group launch");
      i = j - 1;
      continue;
    }
    const void* A = vptr[s.x];
    const void* B = s.y >= 0 ? vptr[s.y] : nullptr;
    void* C = (char*)p->arena + s.off;
    cudaError_t e = run_step(p, s, A, B, C);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "plan step launch");
  }
  return PQ_OK;
}

// Copy a compiled plan's grouped-step descriptors to the device (once per
// compile, outside any stream capture).
int upload_groups(pq_plan* p, const Compiled& c, void** buf, size_t* bytes) {
  Ctx* ctx = p->ctx;
  if (*buf) dev_free(ctx, *buf, *bytes);
  *buf = nullptr;
  *bytes = 0;
  if (c.gdesc.empty()) return PQ_OK;
  const size_t b = c.gdesc.size() * sizeof(GenericDesc);
  int st = dev_alloc(ctx, b, buf);
  if (st) return st;
  *bytes = b;
  cudaError_t e = cudaMemcpyAsync(*buf, c.gdesc.data(), b, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "plan descriptor upload");
  return PQ_OK;
}

size_t result_off(const Compiled& cp) {
  for (size_t i = 0; i < cp.steps.size(); ++i)
    if (cp.nleaves + cp.order[i] == cp.result_ssa || (cp.steps[i].is_copy)) return cp.steps[i].off;
  return 0;
}

int store_result(pq_plan* p, int64_t out_id) {
  Ctx* ctx = p->ctx;
  const auto& dims = p->cp.dims[p->cp.result_ssa];
  Tensor t;
  int st = alloc_tensor(ctx, dims, p->cp.dt[p->cp.result_ssa], t);
  if (st) return st;
  cudaError_t e = cudaMemcpyAsync(t.ptr, (const char*)p->arena + result_off(p->cp), t.bytes,
                                  cudaMemcpyDeviceToDevice, ctx->stream);
  if (e != cudaSuccess) {
    dev_free(ctx, t.ptr, t.bytes);
    return cuda_fail(ctx, e, "plan result copy");
  }
  auto it = ctx->tensors.find(out_id);
  if (it != ctx->tensors.end()) {
    dev_free(ctx, it->second.ptr, it->second.bytes);
    it->second = std::move(t);
  } else {
    ctx->tensors.emplace(out_id, std::move(t));
  }
  return PQ_OK;
}

}  // namespace

extern "C" {

int pq_plan_create(pq_ctx* c, int n_leaves, const int32_t* leaf_ranks, const int32_t* leaf_labels, int n_labels,
                   const int64_t* label_dims, int n_steps, const int32_t* steps, int n_out,
                   const int32_t* out_labels, pq_plan** out) {
  if (!c || !out) return PQ_ERR_INVALID;
  Ctx* ctx = &c->impl;
  *out = nullptr;
  if (n_leaves < 1 || n_labels < 0 || n_steps < 0 || n_out < 0 || !leaf_ranks || (n_labels && !label_dims) ||
      (n_steps && !steps) || (n_out && !out_labels))
    return fail(ctx, PQ_ERR_INVALID, "plan_create: bad arguments");
  if (n_steps != n_leaves - 1) return fail(ctx, PQ_ERR_INVALID, "plan_create: a plan needs n_leaves-1 steps");
  pq_plan* p = new pq_plan();
  p->ctx = ctx;
  p->nleaves = n_leaves;
  p->nlabels = n_labels;
  p->label_dims.assign(label_dims, label_dims + n_labels);
  for (auto d : p->label_dims)
    if (d < 1) {
      delete p;
      return fail(ctx, PQ_ERR_INVALID, "plan_create: label extents must be >= 1");
    }
  int pos = 0;
  for (int i = 0; i < n_leaves; ++i) {
    if (leaf_ranks[i] < 0 || leaf_ranks[i] > PQ_MAX_RANK) {
      delete p;
      return fail(ctx, PQ_ERR_INVALID, "plan_create: bad leaf rank");
    }
    std::vector<int> l(leaf_labels + pos, leaf_labels + pos + leaf_ranks[i]);
    pos += leaf_ranks[i];
    std::vector<int64_t> d;
    for (int x : l) d.push_back((x >= 0 && x < n_labels) ? p->label_dims[x] : 0);
    p->leaf_labels.push_back(l);
    p->leaf_dims.push_back(d);
  }
  p->steps_in.assign(steps, steps + 2 * n_steps);
  p->out_labels.assign(out_labels, out_labels + n_out);
  std::string err;
  if (!compile(ctx, p->leaf_labels, p->label_dims, p->steps_in, p->out_labels, {}, nullptr,
               p->cp, err)) {
    delete p;
    return fail(ctx, PQ_ERR_INVALID, "plan_create: " + err);
  }
  const int st = upload_groups(p, p->cp, &p->d_gdesc, &p->d_gdesc_bytes);
  if (st) {
    delete p;
    return st;
  }
  *out = p;
  return PQ_OK;
}

int pq_plan_destroy(pq_plan* p) {
  if (!p) return PQ_ERR_INVALID;
  Ctx* ctx = p->ctx;
  if (p->gexec) cudaGraphExecDestroy(p->gexec);
  if (p->sgexec) cudaGraphExecDestroy(p->sgexec);
  if (p->arena) dev_free(ctx, p->arena, p->arena_cap);
  if (p->scratch) dev_free(ctx, p->scratch, p->scratch_cap);
  if (p->d_acc) dev_free(ctx, p->d_acc, (size_t)p->out_elems * 32);
  if (p->d_gdesc) dev_free(ctx, p->d_gdesc, p->d_gdesc_bytes);
  if (p->d_sgdesc) dev_free(ctx, p->d_sgdesc, p->d_sgdesc_bytes);
  delete p;
  return PQ_OK;
}

int pq_plan_info(pq_plan* p, double* cmacs, int64_t* max_elems, int64_t* arena_bytes, int64_t* launches) {
  if (!p) return PQ_ERR_INVALID;
  if (cmacs) *cmacs = p->cp.cmacs;
  if (max_elems) *max_elems = p->cp.max_elems;
  if (arena_bytes) *arena_bytes = (int64_t)p->cp.arena_bytes;
  if (launches) *launches = p->cp.launches;
  return PQ_OK;
}

int pq_plan_execute(pq_plan* p, const int64_t* leaf_ids, int64_t out_id) {
  if (!p || !leaf_ids) return PQ_ERR_INVALID;
  Ctx* ctx = p->ctx;
  std::vector<const void*> ptrs;
  int st = leaf_pointers(p, leaf_ids, ptrs);
  if (st) return st;
  st = ensure_buffers(p, p->cp.arena_bytes, p->cp.scratch_bytes);
  if (st) return st;
  bool replay = p->gexec && p->graph_ptrs.size() == ptrs.size();
  if (replay)
    for (size_t i = 0; i < ptrs.size(); ++i)
      if (p->graph_ptrs[i] != ptrs[i]) replay = false;
  if (replay) {
    cudaError_t e = cudaGraphLaunch(p->gexec, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "graph launch");
    ctx->launches += p->cp.launches;
  } else {
    st = launch_all(p, p->cp, ptrs, false, false);
    if (st) return st;
  }
  return store_result(p, out_id);
}

int pq_plan_capture(pq_plan* p, const int64_t* leaf_ids, int64_t out_id) {
  if (!p || !leaf_ids) return PQ_ERR_INVALID;
  Ctx* ctx = p->ctx;
  std::vector<const void*> ptrs;
  int st = leaf_pointers(p, leaf_ids, ptrs);
  if (st) return st;
  st = ensure_buffers(p, p->cp.arena_bytes, p->cp.scratch_bytes);
  if (st) return st;
  if (p->gexec) {
    cudaGraphExecDestroy(p->gexec);
    p->gexec = nullptr;
  }
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "capture sync");
  e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "begin capture");
  int64_t before = ctx->launches;
  st = launch_all(p, p->cp, ptrs, false, false);
  cudaGraph_t g = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &g);
  ctx->launches = before;
  if (st) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e2 != cudaSuccess) return cuda_fail(ctx, e2, "end capture");
  e = cudaGraphInstantiate(&p->gexec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    p->gexec = nullptr;
    return cuda_fail(ctx, e, "graph instantiate");
  }
  p->graph_ptrs.assign(ptrs.begin(), ptrs.end());
  return pq_plan_execute(p, leaf_ids, out_id);
}

int pq_plan_profile(pq_plan* p, const int64_t* leaf_ids, int64_t out_id, float* ms) {
  if (!p || !leaf_ids || !ms) return PQ_ERR_INVALID;
  Ctx* ctx = p->ctx;
  std::vector<const void*> ptrs;
  int st = leaf_pointers(p, leaf_ids, ptrs);
  if (st) return st;
  st = ensure_buffers(p, p->cp.arena_bytes, p->cp.scratch_bytes);
  if (st) return st;
  std::vector<const void*> vptr;
  resolve(p, p->cp, ptrs, vptr);
  const size_t n = p->cp.steps.size();
  std::vector<cudaEvent_t> ev(n + 1);
  for (auto& x : ev) cudaEventCreate(&x);
  cudaEventRecord(ev[0], ctx->stream);
  cudaError_t e = cudaSuccess;
  for (size_t i = 0; i < n && e == cudaSuccess; ++i) {
    const Step& s = p->cp.steps[i];
    e = run_step(p, s, vptr[s.x], s.y >= 0 ? vptr[s.y] : nullptr, (char*)p->arena + s.off);
    cudaEventRecord(ev[i + 1], ctx->stream);
  }
  if (e == cudaSuccess) e = cudaEventSynchronize(ev[n]);
  for (size_t i = 0; i < n; ++i) {
    float t = 0;
    if (e == cudaSuccess) cudaEventElapsedTime(&t, ev[i], ev[i + 1]);
    ms[p->cp.order[i]] = t;
  }
  for (auto& x : ev) cudaEventDestroy(x);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "plan profile");
  return store_result(p, out_id);
}

int pq_plan_step_features(pq_plan* p, double* feats) {
  if (!p || !feats) return PQ_ERR_INVALID;
  for (size_t i = 0; i < p->cp.steps.size(); ++i) {
    const PairPlan& q = p->cp.steps[i].pp;
    const Step& s = p->cp.steps[i];
    double* f = feats + 8 * p->cp.order[i];
    f[0] = std::log2((double)q.asize);
    f[1] = std::log2((double)q.bsize);
    f[2] = std::log2((double)q.csize);
    f[3] = std::log2((double)q.ksize);
    f[4] = std::log2((double)q.run_a);
    f[5] = std::log2((double)q.run_b);
    f[6] = (double)q.kclass;
    f[7] = (double)elem_bytes(s.ta) * q.asize + (s.is_copy ? 0.0 : (double)elem_bytes(s.tb) * q.bsize) +
           (double)elem_bytes(s.tc) * q.csize;
  }
  return PQ_OK;
}

}  // extern "C"

namespace {

// Validate the slicing request, (re)compile the batched network and resolve
// the leaf pointers of the original (ptrs) and batched (lp) networks.
int prepare_sliced(pq_plan* p, const int64_t* leaf_ids, int n_sliced, const int32_t* sliced_labels, int batch,
                   std::vector<const void*>& ptrs, std::vector<const void*>& lp, int64_t& total) {
  if (!p || !leaf_ids || n_sliced < 0 || (n_sliced && !sliced_labels) || batch < 1) return PQ_ERR_INVALID;
  Ctx* ctx = p->ctx;
  if (n_sliced > kMaxModes) return fail(ctx, PQ_ERR_UNSUPPORTED, "run_sliced: too many sliced labels");
  std::vector<int> S(sliced_labels, sliced_labels + n_sliced);
  total = 1;
  for (int l : S) {
    if (l < 0 || l >= p->nlabels) return fail(ctx, PQ_ERR_INVALID, "run_sliced: sliced label out of range");
    if (std::find(p->out_labels.begin(), p->out_labels.end(), l) != p->out_labels.end())
      return fail(ctx, PQ_ERR_INVALID, "run_sliced: an output label cannot be sliced");
    total *= p->label_dims[l];
  }
  int st = leaf_pointers(p, leaf_ids, ptrs);
  if (st) return st;
  // (re)compile the batched network when the slicing or batch changes
  if (S != p->sl_labels || batch != p->sl_batch || p->scp.steps.empty()) {
    const int beta = p->nlabels;  // the batch label
    std::vector<int64_t> ldims = p->label_dims;
    ldims.push_back(batch);
    std::vector<std::vector<int>> ll(p->nleaves);
    std::vector<char> bl(p->nleaves, 0);
    p->sl_leaf_of.assign(p->nleaves, -1);
    p->sl_leaf_off.clear();
    p->sl_leaf_desc.clear();
    p->sl_leaf_sdim.clear();
    p->sl_leaf_sstride.clear();
    p->sl_leaf_dt.clear();
    for (int i = 0; i < p->nleaves; ++i) {
      const auto& lab = p->leaf_labels[i];
      bool hit = false;
      for (int l : lab)
        if (std::find(S.begin(), S.end(), l) != S.end()) hit = true;
      if (!hit) {
        ll[i] = lab;
        continue;
      }
      bl[i] = 1;
      std::vector<int64_t> strides(lab.size());
      int64_t acc = 1;
      for (size_t j = 0; j < lab.size(); ++j) {
        strides[j] = acc;
        acc *= p->leaf_dims[i][j];
      }
      GenericDesc g;
      std::memset(&g, 0, sizeof(g));
      int64_t ksz = 1;
      for (size_t j = 0; j < lab.size(); ++j) {
        if (std::find(S.begin(), S.end(), lab[j]) != S.end()) continue;
        ll[i].push_back(lab[j]);
        g.cdim[g.nc] = p->leaf_dims[i][j];
        g.csa[g.nc] = strides[j];
        g.clog[g.nc] = -1;
        g.nc++;
        ksz *= p->leaf_dims[i][j];
      }
      g.csize = ksz;
      g.ksize = 1;
      ll[i].push_back(beta);
      std::vector<int64_t> sd, ss;
      for (int l : S) {
        sd.push_back(p->label_dims[l]);
        auto it = std::find(lab.begin(), lab.end(), l);
        ss.push_back(it == lab.end() ? 0 : strides[it - lab.begin()]);
      }
      p->sl_leaf_of[i] = (int)p->sl_leaf_desc.size();
      p->sl_leaf_desc.push_back(g);
      p->sl_leaf_sdim.push_back(sd);
      p->sl_leaf_sstride.push_back(ss);
      p->sl_leaf_dt.push_back(p->cp.dt[i]);
    }
    std::vector<int> outl = p->out_labels;
    outl.push_back(beta);
    // execution order: steps that touch no sliced leaf first
    const int ns = (int)p->steps_in.size() / 2;
    std::vector<char> b(p->nleaves + ns, 0);
    for (int i = 0; i < p->nleaves; ++i) b[i] = bl[i];
    std::vector<int> first, second;
    for (int i = 0; i < ns; ++i) {
      b[p->nleaves + i] = b[p->steps_in[2 * i]] || b[p->steps_in[2 * i + 1]];
      (b[p->nleaves + i] ? second : first).push_back(i);
    }
    std::vector<int> order = first;
    order.insert(order.end(), second.begin(), second.end());
    std::string err;
    if (!compile(ctx, ll, ldims, p->steps_in, outl, order, &bl, p->scp, err, &p->cp.dt))
      return fail(ctx, PQ_ERR_INVALID, "run_sliced: " + err);
    const int su = upload_groups(p, p->scp, &p->d_sgdesc, &p->d_sgdesc_bytes);
    if (su) return su;
    // gathered leaf buffers after the arena
    size_t off = align_up(p->scp.arena_bytes, 256);
    for (size_t j = 0; j < p->sl_leaf_desc.size(); ++j) {
      p->sl_leaf_off.push_back(off);
      off += align_up((size_t)p->sl_leaf_desc[j].csize * batch * elem_bytes(p->sl_leaf_dt[j]), 256);
    }
    p->sl_total_bytes = off;
    p->sl_labels = S;
    p->sl_batch = batch;
  }
  st = ensure_buffers(p, std::max(p->sl_total_bytes, p->cp.arena_bytes), p->scp.scratch_bytes);
  if (st) return st;
  lp.resize(p->nleaves);
  for (int i = 0; i < p->nleaves; ++i)
    lp[i] = p->sl_leaf_of[i] >= 0 ? (const void*)((char*)p->arena + p->sl_leaf_off[p->sl_leaf_of[i]]) : ptrs[i];
  return PQ_OK;
}

cudaError_t gather_batch(pq_plan* p, const std::vector<const void*>& ptrs, int64_t s0, int64_t nb) {
  Ctx* ctx = p->ctx;
  for (int i = 0; i < p->nleaves; ++i) {
    int j = p->sl_leaf_of[i];
    if (j < 0) continue;
    cudaError_t e = launch_slice_gather(p->sl_leaf_dt[j], ptrs[i], (char*)p->arena + p->sl_leaf_off[j],
                                        p->sl_leaf_desc[j], (int)p->sl_labels.size(), p->sl_leaf_sdim[j].data(),
                                        p->sl_leaf_sstride[j].data(), s0, p->sl_batch, s0 + nb, ctx->stream);
    ctx->launches++;
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

extern "C" {

int pq_plan_run_sliced(pq_plan* p, const int64_t* leaf_ids, int n_sliced, const int32_t* sliced_labels,
                       int64_t slice_begin, int64_t slice_end, int batch, int reset_sum) {
  if (!p) return PQ_ERR_INVALID;
  Ctx* ctx = p->ctx;
  std::vector<const void*> ptrs, lp;
  int64_t total = 0;
  int st = prepare_sliced(p, leaf_ids, n_sliced, sliced_labels, batch, ptrs, lp, total);
  if (st) return st;
  if (slice_begin < 0 || slice_end > total || slice_begin > slice_end)
    return fail(ctx, PQ_ERR_INVALID, "run_sliced: slice range outside [0, " + std::to_string(total) + ")");
  // output accumulators
  int64_t oe = 1;
  for (auto d : p->scp.dims[p->scp.result_ssa]) oe *= d;
  oe /= batch;
  if (oe != p->out_elems || !p->d_acc) {
    if (p->d_acc) dev_free(ctx, p->d_acc, (size_t)p->out_elems * 32);
    p->d_acc = nullptr;
    p->out_elems = oe;
    st = dev_alloc(ctx, (size_t)oe * 32, (void**)&p->d_acc);
    if (st) return st;
    reset_sum = 1;
  }
  // replay the captured run when nothing it depends on has changed
  std::vector<const void*> key = ptrs;
  key.push_back(p->arena);
  key.push_back(p->scratch);
  key.push_back(p->d_acc);
  std::vector<int64_t> args(sliced_labels, sliced_labels + n_sliced);
  args.insert(args.end(), {slice_begin, slice_end, (int64_t)batch, (int64_t)(reset_sum ? 1 : 0)});
  if (key == p->sg_key && args == p->sg_args && p->sgexec) {
    cudaError_t e = cudaGraphLaunch(p->sgexec, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "run_sliced graph launch");
    ctx->launches += p->sg_launches;
    return PQ_OK;
  }
  if (key != p->sg_key || args != p->sg_args) {
    if (p->sgexec) cudaGraphExecDestroy(p->sgexec);
    p->sgexec = nullptr;
    p->sg_key = key;
    p->sg_args = args;
    p->sg_seen = 0;
  }
  // the first call runs directly (it also sets kernel attributes, allocates
  // nothing later); the second identical call is captured and launched
  const bool capture = ++p->sg_seen >= 2;
  if (capture) {
    cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "run_sliced capture");
  }
  const int64_t l0 = ctx->launches;
  st = PQ_OK;
  if (reset_sum) {
    cudaError_t e = cudaMemsetAsync(p->d_acc, 0, (size_t)oe * 32, ctx->stream);
    if (e != cudaSuccess) st = cuda_fail(ctx, e, "run_sliced reset");
  }
  // unbatched part once
  if (!st) st = launch_all(p, p->scp, lp, false, true);
  const size_t res_off = result_off(p->scp);
  for (int64_t s0 = slice_begin; s0 < slice_end && !st; s0 += batch) {
    int64_t nb = std::min<int64_t>(batch, slice_end - s0);
    cudaError_t eg = gather_batch(p, ptrs, s0, nb);
    if (eg != cudaSuccess) {
      st = cuda_fail(ctx, eg, "slice gather");
      break;
    }
    st = launch_all(p, p->scp, lp, true, false);
    if (st) break;
    cudaError_t e = launch_slice_sum(p->scp.dt[p->scp.result_ssa], (const char*)p->arena + res_off, oe, nb, p->d_acc,
                                     p->d_acc + 2 * oe, ctx->stream);
    ctx->launches++;
    if (e != cudaSuccess) st = cuda_fail(ctx, e, "slice sum");
  }
  if (capture) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (!st && e == cudaSuccess) e = cudaGraphInstantiate(&p->sgexec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (st || e != cudaSuccess) {
      if (p->sgexec) cudaGraphExecDestroy(p->sgexec);
      p->sgexec = nullptr;
      p->sg_key.clear();
      return st ? st : cuda_fail(ctx, e, "run_sliced capture");
    }
    p->sg_launches = ctx->launches - l0;  // counted once, when captured
    e = cudaGraphLaunch(p->sgexec, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "run_sliced graph launch");
  }
  return st;
}

int pq_plan_profile_sliced(pq_plan* p, const int64_t* leaf_ids, int n_sliced, const int32_t* sliced_labels,
                           int batch, float* ms, int32_t* batched, double* feats) {
  if (!p || !ms || !batched || !feats) return PQ_ERR_INVALID;
  Ctx* ctx = p->ctx;
  std::vector<const void*> ptrs, lp;
  int64_t total = 0;
  int st = prepare_sliced(p, leaf_ids, n_sliced, sliced_labels, batch, ptrs, lp, total);
  if (st) return st;
  cudaError_t e = gather_batch(p, ptrs, 0, std::min<int64_t>(batch, total));
  if (e != cudaSuccess) return cuda_fail(ctx, e, "profile gather");
  const Compiled& cp = p->scp;
  std::vector<const void*> vptr;
  resolve(p, cp, lp, vptr);
  const size_t n = cp.steps.size();
  std::vector<cudaEvent_t> ev(n + 1);
  for (auto& x : ev) cudaEventCreate(&x);
  cudaEventRecord(ev[0], ctx->stream);
  for (size_t i = 0; i < n && e == cudaSuccess; ++i) {
    const Step& s = cp.steps[i];
    e = run_step(p, s, vptr[s.x], s.y >= 0 ? vptr[s.y] : nullptr, (char*)p->arena + s.off);
    cudaEventRecord(ev[i + 1], ctx->stream);
  }
  if (e == cudaSuccess) e = cudaEventSynchronize(ev[n]);
  for (size_t i = 0; i < n; ++i) {
    float t = 0;
    if (e == cudaSuccess) cudaEventElapsedTime(&t, ev[i], ev[i + 1]);
    const int o = cp.order[i];
    ms[o] = t;
    batched[o] = cp.steps[i].batched ? 1 : 0;
    const PairPlan& q = cp.steps[i].pp;
    double* f = feats + 8 * o;
    f[0] = std::log2((double)q.asize);
    f[1] = std::log2((double)q.bsize);
    f[2] = std::log2((double)q.csize);
    f[3] = std::log2((double)q.ksize);
    f[4] = std::log2((double)q.run_a);
    f[5] = std::log2((double)q.run_b);
    f[6] = (double)q.kclass;
    const Step& s = cp.steps[i];
    f[7] = (double)elem_bytes(s.ta) * q.asize + (s.is_copy ? 0.0 : (double)elem_bytes(s.tb) * q.bsize) +
           (double)elem_bytes(s.tc) * q.csize;
  }
  for (auto& x : ev) cudaEventDestroy(x);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "profile sliced");
  return PQ_OK;
}

int pq_sliced_result(pq_plan* p, double* out, int64_t n) {
  if (!p || !out) return PQ_ERR_INVALID;
  Ctx* ctx = p->ctx;
  if (!p->d_acc || n < p->out_elems) return fail(ctx, PQ_ERR_INVALID, "sliced_result: no result or buffer too small");
  std::vector<double> h((size_t)p->out_elems * 4);
  cudaError_t e = cudaMemcpyAsync(h.data(), p->d_acc, h.size() * 8, cudaMemcpyDeviceToHost, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "sliced_result copy");
  int st = check_status(ctx);
  if (st) return st;
  for (int64_t i = 0; i < 2 * p->out_elems; ++i) out[i] = h[i] + h[2 * p->out_elems + i];
  return PQ_OK;
}

}  // extern "C"
