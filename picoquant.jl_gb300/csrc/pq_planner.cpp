// Host planners: Boltzmann-greedy pair selection (the flop-count planner) and
// the choice of labels to slice.
//
// The pair heuristic is the Gray & Kourtis cost used by the reference's
// bgreedy (src/layer2/bgreedy_contraction.jl:76-94):
//     energy(A, B) = |C| - alpha * (|A| + |B|)
// sampled with weight exp(-(energy - min_energy) / (tau * max(1, |min_energy|)))
// (the temperature is relative to the scale of the energies so the sampler
// stays meaningful when tensor sizes span many orders of magnitude).  Only
// pairs that share a label are candidates (pairs without a shared label are
// outer products; they are taken last, smallest first, as
// src/layer2.jl:260-264 does for disjoint pieces).  The plan with the fewest
// complex multiply-adds (src/backends.jl:30-41) over `n_trials` draws wins.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <random>
#include <set>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/pqgb300.h"

namespace {

struct Net {
  std::vector<std::vector<int>> labels;  // per SSA value
  std::vector<double> l2size;            // log2 of the element count
};

struct Trial {
  std::vector<int32_t> steps;
  double cmacs = 0;
  double max_l2 = 0;
};

double l2size_of(const std::vector<int>& l, const std::vector<double>& l2dim) {
  double s = 0;
  for (int x : l) s += l2dim[x];
  return s;
}

// Candidate pairs with their energies: a dense array (uniform sampling and
// swap-removal), a key -> slot index, and the same pairs ordered by energy
// (minimum, ties, and the exact sampling window).
struct CandSet {
  std::vector<uint64_t> keys;
  std::vector<double> en;
  std::unordered_map<uint64_t, int> slot;
  std::set<std::pair<double, uint64_t>> order;
  static uint64_t key(int u, int v) {
    const int a = std::min(u, v), b = std::max(u, v);
    return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b;
  }
  void set(uint64_t k, double e) {
    auto it = slot.find(k);
    if (it != slot.end()) {
      order.erase({en[it->second], k});
      en[it->second] = e;
    } else {
      slot.emplace(k, (int)keys.size());
      keys.push_back(k);
      en.push_back(e);
    }
    order.insert({e, k});
  }
  void erase(uint64_t k) {
    auto it = slot.find(k);
    if (it == slot.end()) return;
    const int i = it->second, last = (int)keys.size() - 1;
    order.erase({en[i], k});
    if (i != last) {
      keys[i] = keys[last];
      en[i] = en[last];
      slot[keys[i]] = i;
    }
    keys.pop_back();
    en.pop_back();
    slot.erase(it);
  }
};

Trial greedy_once(int n_leaves, const std::vector<std::vector<int>>& leaves, const std::vector<double>& l2dim,
                  const std::vector<int>& out_labels, double alpha, double tau, std::mt19937_64& rng) {
  const int nl = n_leaves;
  const int nv = 2 * nl - 1;
  const int nlab = (int)l2dim.size();
  std::vector<std::vector<int>> lab(nv);
  std::vector<double> l2(nv, 0);
  std::vector<char> live(nv, 0);
  std::vector<int> cnt(nlab, 0);
  std::vector<std::vector<int>> holders(nlab);  // live values per label (lazy)
  std::vector<uint32_t> stamp(nlab, 0);         // label marks for set intersections
  uint32_t cur_stamp = 0;
  for (int i = 0; i < nl; ++i) {
    lab[i] = leaves[i];
    l2[i] = l2size_of(lab[i], l2dim);
    live[i] = 1;
    for (int x : lab[i]) {
      cnt[x]++;
      holders[x].push_back(i);
    }
  }
  for (int x : out_labels) cnt[x]++;
  Trial t;
  CandSet cs;
  // labels of the result of (a, b) -- a's kept labels in a's order, then b's
  // labels not in a -- with log2 of its size and of the size of every label
  // involved; O(|a| + |b|) with the label stamps
  auto result_labels = [&](int a, int b, std::vector<int>* r, double& l2c, double& l2all) {
    if (r) r->clear();
    l2c = 0;
    l2all = 0;
    ++cur_stamp;
    for (int x : lab[b]) stamp[x] = cur_stamp;
    for (int x : lab[a]) {
      l2all += l2dim[x];
      const bool in_b = stamp[x] == cur_stamp;
      if (cnt[x] - 1 - (in_b ? 1 : 0) > 0) {
        l2c += l2dim[x];
        if (r) r->push_back(x);
      }
      if (in_b) stamp[x] = cur_stamp - 1;  // seen: skipped in b's pass
    }
    for (int x : lab[b]) {
      if (stamp[x] != cur_stamp) continue;  // also in a
      l2all += l2dim[x];
      if (cnt[x] - 1 > 0) {
        l2c += l2dim[x];
        if (r) r->push_back(x);
      }
    }
    ++cur_stamp;  // a's marks (cur_stamp - 2 after this) never match again
  };
  auto score = [&](int a, int b) {
    double l2c, l2all;
    result_labels(a, b, nullptr, l2c, l2all);
    return std::exp2(l2c) - alpha * (std::exp2(l2[a]) + std::exp2(l2[b]));
  };
  auto set_score = [&](int u, int v) { cs.set(CandSet::key(u, v), score(u, v)); };
  // live values sharing a label with v
  auto partners = [&](int v, std::vector<int>& nb) {
    nb.clear();
    for (int x : lab[v])
      for (int u : holders[x])
        if (u != v && live[u]) nb.push_back(u);
    std::sort(nb.begin(), nb.end());
    nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
  };
  std::vector<int> nb, nb2, hyper;
  for (int i = 0; i < nl; ++i) {
    partners(i, nb);
    for (int u : nb)
      if (u > i) set_score(i, u);
  }
  int next = nl;
  int nlive = nl;
  std::uniform_real_distribution<double> U(0.0, 1.0);
  std::vector<uint64_t> keys;
  std::vector<double> w;
  auto split = [](uint64_t k, int& a, int& b) {
    a = (int)(k >> 32);
    b = (int)(k & 0xffffffffu);
  };
  std::vector<int> r;
  while (nlive > 1) {
    int a = -1, b = -1;
    if (!cs.order.empty()) {
      const double emin = cs.order.begin()->first;
      keys.clear();
      if (tau <= 0) {
        // deterministic greedy with random tie-break
        for (auto it = cs.order.begin(); it != cs.order.end() && it->first <= emin; ++it) keys.push_back(it->second);
        split(keys[std::uniform_int_distribution<size_t>(0, keys.size() - 1)(rng)], a, b);
      } else {
        // weights exp(-(e - emin) / T): a uniform pick accepted with its
        // weight (at most 64 tries), else the exact draw over the pairs
        // within 50 T of the minimum (beyond it weights are below e^-50)
        const double T = tau * std::max(1.0, std::fabs(emin));
        std::uniform_int_distribution<size_t> pick(0, cs.keys.size() - 1);
        for (int tries = 0; tries < 64 && a < 0; ++tries) {
          const size_t i = pick(rng);
          if (U(rng) < std::exp(-(cs.en[i] - emin) / T)) split(cs.keys[i], a, b);
        }
        if (a < 0) {
          w.clear();
          double tot = 0;
          for (auto it = cs.order.begin(); it != cs.order.end() && it->first - emin <= 50.0 * T; ++it) {
            const double x = std::exp(-(it->first - emin) / T);
            keys.push_back(it->second);
            w.push_back(x);
            tot += x;
          }
          double u = U(rng) * tot;
          size_t k = 0;
          for (; k + 1 < w.size(); ++k) {
            u -= w[k];
            if (u <= 0) break;
          }
          split(keys[k], a, b);
        }
      }
    } else {
      // disjoint pieces: outer product of the two smallest
      int s1 = -1, s2 = -1;
      for (int v = 0; v < next; ++v) {
        if (!live[v]) continue;
        if (s1 < 0 || l2[v] < l2[s1]) {
          s2 = s1;
          s1 = v;
        } else if (s2 < 0 || l2[v] < l2[s2]) {
          s2 = v;
        }
      }
      a = std::min(s1, s2);
      b = std::max(s1, s2);
    }
    double l2c, l2all;
    result_labels(a, b, &r, l2c, l2all);
    t.cmacs += std::exp2(l2all);
    t.max_l2 = std::max(t.max_l2, l2c);
    t.steps.push_back(a);
    t.steps.push_back(b);
    // labels held by both and kept (hyper-indices): their counts drop, so
    // the pairs of their other holders are rescored below; no other pair's
    // energy changes
    hyper.clear();
    ++cur_stamp;
    for (int x : lab[b]) stamp[x] = cur_stamp;
    for (int x : lab[a])
      if (stamp[x] == cur_stamp && cnt[x] - 2 > 0) hyper.push_back(x);
    ++cur_stamp;
    // retire a, b and every candidate pair that holds one of them
    partners(a, nb);
    for (int u : nb) cs.erase(CandSet::key(a, u));
    partners(b, nb);
    for (int u : nb) cs.erase(CandSet::key(b, u));
    live[a] = live[b] = 0;
    for (int x : lab[a]) cnt[x]--;
    for (int x : lab[b]) cnt[x]--;
    const int v = next++;
    lab[v] = r;
    l2[v] = l2c;
    live[v] = 1;
    for (int x : r) {
      cnt[x]++;
      auto& h = holders[x];
      h.erase(std::remove_if(h.begin(), h.end(), [&](int u) { return !live[u]; }), h.end());
      h.push_back(v);
    }
    nlive--;
    for (int x : hyper)
      for (int u : holders[x]) {
        if (u == v || !live[u]) continue;
        partners(u, nb2);
        for (int y : nb2)
          if (y != v) set_score(u, y);
      }
    partners(v, nb);
    for (int u : nb) set_score(v, u);
  }
  return t;
}

}  // namespace

extern "C" {

int pq_plan_greedy(int n_leaves, const int32_t* leaf_ranks, const int32_t* leaf_labels, int n_labels,
                   const int64_t* label_dims, int n_out, const int32_t* out_labels, double alpha, double tau,
                   int n_trials, uint64_t seed, int32_t* steps, double* cmacs, int64_t* max_elems) {
  if (n_leaves < 1 || !leaf_ranks || (n_labels && !label_dims) || (n_out && !out_labels) || n_trials < 1 ||
      (n_leaves > 1 && !steps))
    return PQ_ERR_INVALID;
  std::vector<double> l2dim(n_labels);
  for (int i = 0; i < n_labels; ++i) {
    if (label_dims[i] < 1) return PQ_ERR_INVALID;
    l2dim[i] = std::log2((double)label_dims[i]);
  }
  std::vector<std::vector<int>> leaves(n_leaves);
  int pos = 0;
  for (int i = 0; i < n_leaves; ++i) {
    if (leaf_ranks[i] < 0) return PQ_ERR_INVALID;
    for (int j = 0; j < leaf_ranks[i]; ++j) {
      int x = leaf_labels[pos++];
      if (x < 0 || x >= n_labels) return PQ_ERR_INVALID;
      leaves[i].push_back(x);
    }
  }
  std::vector<int> outl(out_labels, out_labels + n_out);
  for (int x : outl)
    if (x < 0 || x >= n_labels) return PQ_ERR_INVALID;
  std::mt19937_64 rng(seed);
  Trial best;
  best.cmacs = INFINITY;
  for (int t = 0; t < n_trials; ++t) {
    // the first draw is the plain greedy order (tau = 0)
    Trial tr = greedy_once(n_leaves, leaves, l2dim, outl, alpha, t == 0 ? 0.0 : tau, rng);
    if (tr.cmacs < best.cmacs || (tr.cmacs == best.cmacs && tr.max_l2 < best.max_l2)) best = tr;
  }
  if (n_leaves > 1) std::memcpy(steps, best.steps.data(), best.steps.size() * sizeof(int32_t));
  if (cmacs) *cmacs = n_leaves > 1 ? best.cmacs : 0.0;
  if (max_elems) *max_elems = (int64_t)std::llround(std::exp2(best.max_l2));
  return PQ_OK;
}

int pq_plan_greedy_many(int n_leaves, const int32_t* leaf_ranks, const int32_t* leaf_labels, int n_labels,
                        const int64_t* label_dims, int n_out, const int32_t* out_labels, double alpha, double tau,
                        int n_draws, uint64_t seed, int n_threads, int32_t* steps, double* cmacs,
                        int64_t* max_elems) {
  if (n_leaves < 1 || !leaf_ranks || (n_labels && !label_dims) || (n_out && !out_labels) || n_draws < 1 ||
      (n_leaves > 1 && !steps) || !cmacs || !max_elems)
    return PQ_ERR_INVALID;
  std::vector<double> l2dim(n_labels);
  for (int i = 0; i < n_labels; ++i) {
    if (label_dims[i] < 1) return PQ_ERR_INVALID;
    l2dim[i] = std::log2((double)label_dims[i]);
  }
  std::vector<std::vector<int>> leaves(n_leaves);
  int pos = 0;
  for (int i = 0; i < n_leaves; ++i) {
    if (leaf_ranks[i] < 0) return PQ_ERR_INVALID;
    for (int j = 0; j < leaf_ranks[i]; ++j) {
      int x = leaf_labels[pos++];
      if (x < 0 || x >= n_labels) return PQ_ERR_INVALID;
      leaves[i].push_back(x);
    }
  }
  std::vector<int> outl(out_labels, out_labels + n_out);
  for (int x : outl)
    if (x < 0 || x >= n_labels) return PQ_ERR_INVALID;
  const size_t per = n_leaves > 1 ? (size_t)(2 * (n_leaves - 1)) : 0;
  // draw d: its own generator seeded with seed + d, so results do not depend
  // on the thread count; draw 0 is the plain greedy order (tau = 0)
  auto run = [&](int d) {
    std::mt19937_64 rng(seed + (uint64_t)d);
    Trial tr = greedy_once(n_leaves, leaves, l2dim, outl, alpha, d == 0 ? 0.0 : tau, rng);
    if (per) std::memcpy(steps + per * (size_t)d, tr.steps.data(), per * sizeof(int32_t));
    cmacs[d] = per ? tr.cmacs : 0.0;
    max_elems[d] = (int64_t)std::llround(std::exp2(tr.max_l2));
  };
  int nt = n_threads > 0 ? n_threads : (int)std::max(1u, std::thread::hardware_concurrency());
  nt = std::min(nt, n_draws);
  if (nt <= 1) {
    for (int d = 0; d < n_draws; ++d) run(d);
    return PQ_OK;
  }
  std::vector<std::thread> pool;
  for (int t = 0; t < nt; ++t)
    pool.emplace_back([&, t] {
      for (int d = t; d < n_draws; d += nt) run(d);
    });
  for (auto& th : pool) th.join();
  return PQ_OK;
}

int pq_plan_cost(int n_leaves, const int32_t* leaf_ranks, const int32_t* leaf_labels, int n_labels,
                 const int64_t* label_dims, int n_steps, const int32_t* steps, int n_out,
                 const int32_t* out_labels, double* cmacs, double* max_elems) {
  if (n_leaves < 1 || !leaf_ranks || n_steps < 0 || (n_steps && !steps) || (n_out && !out_labels) || !cmacs ||
      !max_elems || n_labels < 0 || (n_labels && !label_dims))
    return PQ_ERR_INVALID;
  std::vector<double> l2dim(n_labels);
  for (int i = 0; i < n_labels; ++i) {
    if (label_dims[i] < 1) return PQ_ERR_INVALID;
    l2dim[i] = std::log2((double)label_dims[i]);
  }
  std::vector<std::vector<int>> lab(n_leaves + n_steps);
  std::vector<int> cnt(n_labels, 0);
  int pos = 0;
  for (int i = 0; i < n_leaves; ++i) {
    if (leaf_ranks[i] < 0) return PQ_ERR_INVALID;
    for (int j = 0; j < leaf_ranks[i]; ++j) {
      const int x = leaf_labels[pos++];
      if (x < 0 || x >= n_labels) return PQ_ERR_INVALID;
      lab[i].push_back(x);
      cnt[x]++;
    }
  }
  for (int i = 0; i < n_out; ++i) {
    if (out_labels[i] < 0 || out_labels[i] >= n_labels) return PQ_ERR_INVALID;
    cnt[out_labels[i]]++;
  }
  std::vector<uint32_t> seen(n_labels, 0);
  uint32_t stamp = 0;
  double cost = 0, mx = 0;
  std::vector<int> uni;
  for (int s = 0; s < n_steps; ++s) {
    const int x = steps[2 * s], y = steps[2 * s + 1];
    if (x < 0 || y < 0 || x >= n_leaves + s || y >= n_leaves + s) return PQ_ERR_INVALID;
    for (int l : lab[x]) cnt[l]--;
    for (int l : lab[y]) cnt[l]--;
    // the union of both label lists, first occurrences in order
    ++stamp;
    uni.clear();
    for (const auto* side : {&lab[x], &lab[y]})
      for (int l : *side)
        if (seen[l] != stamp) {
          seen[l] = stamp;
          uni.push_back(l);
        }
    double l2u = 0, l2k = 0;
    std::vector<int>& keep = lab[n_leaves + s];
    for (int l : uni) {
      l2u += l2dim[l];
      if (cnt[l] > 0) keep.push_back(l);
    }
    for (int l : keep) {
      cnt[l]++;
      l2k += l2dim[l];
    }
    cost += std::exp2(l2u);
    mx = std::max(mx, l2k);
  }
  *cmacs = cost;
  *max_elems = std::exp2(mx);
  return PQ_OK;
}

int pq_plan_choose_slices(int n_leaves, const int32_t* leaf_ranks, const int32_t* leaf_labels, int n_labels,
                          const int64_t* label_dims, int n_steps, const int32_t* steps, int n_out,
                          const int32_t* out_labels, int max_sliced, double log2_target, int32_t* sliced,
                          int* n_sliced) {
  if (n_leaves < 1 || !leaf_ranks || n_steps != n_leaves - 1 || (n_steps && !steps) || !sliced || !n_sliced ||
      max_sliced < 0)
    return PQ_ERR_INVALID;
  std::vector<double> l2dim(n_labels);
  for (int i = 0; i < n_labels; ++i) {
    if (label_dims[i] < 1) return PQ_ERR_INVALID;
    l2dim[i] = std::log2((double)label_dims[i]);
  }
  const int nv = n_leaves + n_steps;
  std::vector<std::vector<int>> lab(nv);
  std::vector<std::vector<int>> all(nv);      // labels involved in the step producing v
  std::vector<std::vector<char>> dep(nv);     // labels of leaves in v's subtree
  int pos = 0;
  std::vector<int> cnt(n_labels, 0);
  for (int i = 0; i < n_leaves; ++i) {
    for (int j = 0; j < leaf_ranks[i]; ++j) {
      int x = leaf_labels[pos++];
      if (x < 0 || x >= n_labels) return PQ_ERR_INVALID;
      lab[i].push_back(x);
      cnt[x]++;
    }
    dep[i].assign(n_labels, 0);
    for (int x : lab[i]) dep[i][x] = 1;
  }
  std::vector<char> is_out(n_labels, 0);
  for (int i = 0; i < n_out; ++i) {
    is_out[out_labels[i]] = 1;
    cnt[out_labels[i]]++;
  }
  for (int s = 0; s < n_steps; ++s) {
    int a = steps[2 * s], b = steps[2 * s + 1];
    if (a < 0 || b < 0 || a >= n_leaves + s || b >= n_leaves + s) return PQ_ERR_INVALID;
    int v = n_leaves + s;
    for (int x : lab[a]) cnt[x]--;
    for (int x : lab[b]) cnt[x]--;
    std::vector<int> r, u;
    for (int x : lab[a]) {
      u.push_back(x);
      if (cnt[x] > 0) r.push_back(x);
    }
    for (int x : lab[b]) {
      if (std::find(lab[a].begin(), lab[a].end(), x) != lab[a].end()) continue;
      u.push_back(x);
      if (cnt[x] > 0) r.push_back(x);
    }
    for (int x : r) cnt[x]++;
    lab[v] = r;
    all[v] = u;
    dep[v].assign(n_labels, 0);
    for (int x = 0; x < n_labels; ++x) dep[v][x] = dep[a][x] | dep[b][x];
  }
  // Membership tables: inlab[v][x] (x is a mode of value v) and inall[v][x]
  // (x takes part in the step producing v).
  std::vector<std::vector<char>> inlab(nv, std::vector<char>(n_labels, 0)), inall(nv);
  for (int v = 0; v < nv; ++v) {
    for (int x : lab[v]) inlab[v][x] = 1;
    inall[v].assign(n_labels, 0);
    for (int x : all[v]) inall[v][x] = 1;
  }
  // Current (sliced) log2 size of every value, log2 cost of every step, and
  // whether the step varies with the slice (depends on a sliced leaf).
  std::vector<char> chosen(n_labels, 0);
  std::vector<int> S;
  std::vector<double> sz(nv, 0), cc(nv, 0);
  std::vector<char> varies(nv, 0);
  for (int v = 0; v < nv; ++v) {
    for (int x : lab[v]) sz[v] += l2dim[x];
    for (int x : all[v]) cc[v] += l2dim[x];
  }
  double nsl = 0;
  auto cur_max = [&]() {
    double m = 0;
    for (int v = 0; v < nv; ++v) m = std::max(m, sz[v]);
    return m;
  };
  // Objective of slicing label x next: (largest intermediate clipped at the
  // target, number of values at that size, total cost over all slices), in
  // lexicographic order.  Once the largest intermediate is within the target
  // only the total cost (the redundant work slicing causes) matters.
  while ((int)S.size() < max_sliced) {
    const double cmax = cur_max();
    int best = -1;
    double bkey = INFINITY, bcost = INFINITY;
    int bcnt = 1 << 30;
    for (int x = 0; x < n_labels; ++x) {
      if (chosen[x] || is_out[x]) continue;
      bool used = false;
      for (int v = n_leaves; v < nv && !used; ++v) used = inall[v][x];
      if (!used) continue;
      double m = 0, cost = 0;
      for (int v = 0; v < nv; ++v) m = std::max(m, sz[v] - (inlab[v][x] ? l2dim[x] : 0));
      int cntm = 0;
      for (int v = 0; v < nv; ++v)
        if (sz[v] - (inlab[v][x] ? l2dim[x] : 0) >= m - 1e-9) ++cntm;
      for (int v = n_leaves; v < nv; ++v) {
        const bool var = varies[v] || dep[v][x];
        cost += std::exp2(cc[v] - (inall[v][x] ? l2dim[x] : 0) + (var ? nsl + l2dim[x] : 0));
      }
      const double key = std::max(m, log2_target);
      const bool over = key > log2_target + 1e-9;
      bool better;
      if (key < bkey - 1e-9)
        better = true;
      else if (key > bkey + 1e-9)
        better = false;
      else if (over)
        better = cntm < bcnt || (cntm == bcnt && cost < bcost);
      else
        better = cost < bcost;
      if (better) {
        best = x;
        bkey = key;
        bcnt = cntm;
        bcost = cost;
      }
    }
    if (best < 0) break;
    (void)cmax;
    chosen[best] = 1;
    S.push_back(best);
    nsl += l2dim[best];
    for (int v = 0; v < nv; ++v) {
      if (inlab[v][best]) sz[v] -= l2dim[best];
      if (inall[v][best]) cc[v] -= l2dim[best];
      if (dep[v][best]) varies[v] = 1;
    }
  }
  for (size_t i = 0; i < S.size(); ++i) sliced[i] = S[i];
  *n_sliced = (int)S.size();
  return PQ_OK;
}

}  // extern "C"
