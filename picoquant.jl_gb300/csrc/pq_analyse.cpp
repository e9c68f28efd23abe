// Mode analysis of one pairwise contraction: which labels are kept, which are
// summed, their strides in A/B/C, mode merging, and the choice of kernel class.
//
// Semantics follow src/layer1.jl:85-92 (tensorcontract with output labels
// symdiff(ia, ib)) for the interactive path; the plan executor passes its own
// result label order (which may keep labels shared by both operands, i.e.
// batch/hyper indices, and may put the result in any mode order).
#include <algorithm>
#include <cstring>

#include "pq_internal.h"

namespace pq {

std::vector<int> symdiff_labels(const std::vector<int>& la, const std::vector<int>& lb) {
  std::vector<int> out;
  for (int x : la)
    if (std::find(lb.begin(), lb.end(), x) == lb.end()) out.push_back(x);
  for (int x : lb)
    if (std::find(la.begin(), la.end(), x) == la.end() &&
        std::find(out.begin(), out.end(), x) == out.end())
      out.push_back(x);
  return out;
}

static int ilog2_exact(int64_t d) {
  if (d <= 0 || (d & (d - 1))) return -1;
  int l = 0;
  while ((int64_t(1) << l) < d) ++l;
  return l;
}

static std::vector<int64_t> colmajor_strides(const std::vector<int64_t>& dims) {
  std::vector<int64_t> s(dims.size());
  int64_t acc = 1;
  for (size_t i = 0; i < dims.size(); ++i) {
    s[i] = acc;
    acc *= dims[i];
  }
  return s;
}

// Merge consecutive modes whose strides chain in every operand.
static void merge_modes(std::vector<Mode>& v) {
  std::vector<Mode> out;
  for (const Mode& m : v) {
    if (m.dim == 1) continue;
    if (!out.empty()) {
      Mode& p = out.back();
      if (m.sa == p.sa * p.dim && m.sb == p.sb * p.dim && m.sc == p.sc * p.dim) {
        p.dim *= m.dim;
        continue;
      }
    }
    out.push_back(m);
  }
  v.swap(out);
}

bool analyse_pair(const std::vector<int>& la, const std::vector<int64_t>& da,
                  const std::vector<int>& lb, const std::vector<int64_t>& db,
                  const std::vector<int>& lc, int precision, PairPlan& out, std::string& err,
                  const TuningTable* tune) {
  if (la.size() != da.size() || lb.size() != db.size()) {
    err = "label/dim count mismatch";
    return false;
  }
  auto has_dup = [](const std::vector<int>& l) {
    for (size_t i = 0; i < l.size(); ++i)
      for (size_t j = i + 1; j < l.size(); ++j)
        if (l[i] == l[j]) return true;
    return false;
  };
  if (has_dup(la) || has_dup(lb)) {
    err = "repeated label within one operand (traces are not supported)";
    return false;
  }
  if (has_dup(lc)) {
    err = "repeated label in the result";
    return false;
  }
  auto sa = colmajor_strides(da), sb = colmajor_strides(db);
  auto find = [](const std::vector<int>& l, int x) {
    for (size_t i = 0; i < l.size(); ++i)
      if (l[i] == x) return int(i);
    return -1;
  };
  out = PairPlan();
  out.asize = 1;
  for (auto d : da) out.asize *= d;
  out.bsize = 1;
  for (auto d : db) out.bsize *= d;
  // shared labels must agree in extent
  for (size_t i = 0; i < la.size(); ++i) {
    int j = find(lb, la[i]);
    if (j >= 0 && da[i] != db[j]) {
      err = "extent mismatch on label " + std::to_string(la[i]) + ": " + std::to_string(da[i]) +
            " vs " + std::to_string(db[j]);
      return false;
    }
  }
  // result modes
  std::vector<Mode> cm;
  int64_t csz = 1;
  for (int x : lc) {
    int ia = find(la, x), ib = find(lb, x);
    if (ia < 0 && ib < 0) {
      err = "result label " + std::to_string(x) + " is in neither operand";
      return false;
    }
    Mode m;
    m.dim = ia >= 0 ? da[ia] : db[ib];
    m.sa = ia >= 0 ? sa[ia] : 0;
    m.sb = ib >= 0 ? sb[ib] : 0;
    m.sc = csz;
    csz *= m.dim;
    cm.push_back(m);
    out.c_labels.push_back(x);
    out.c_dims.push_back(m.dim);
  }
  out.csize = csz;
  // summed modes (in A or B, not in C)
  std::vector<Mode> km;
  int64_t ksz = 1;
  for (size_t i = 0; i < la.size(); ++i) {
    if (find(lc, la[i]) >= 0) continue;
    int ib = find(lb, la[i]);
    km.push_back(Mode{da[i], sa[i], ib >= 0 ? sb[ib] : 0, 0});
    ksz *= da[i];
  }
  for (size_t i = 0; i < lb.size(); ++i) {
    if (find(lc, lb[i]) >= 0 || find(la, lb[i]) >= 0) continue;
    km.push_back(Mode{db[i], 0, sb[i], 0});
    ksz *= db[i];
  }
  out.ksize = ksz;
  // K modes ordered for locality in the larger operand, then merged.
  bool a_big = out.asize >= out.bsize;
  std::stable_sort(km.begin(), km.end(), [a_big](const Mode& x, const Mode& y) {
    int64_t xa = a_big ? x.sa : x.sb, ya = a_big ? y.sa : y.sb;
    if (xa == 0) xa = INT64_MAX;
    if (ya == 0) ya = INT64_MAX;
    return xa < ya;
  });

  // ---- generic descriptor
  std::vector<Mode> gc = cm, gk = km;
  merge_modes(gc);
  merge_modes(gk);
  if ((int)gc.size() > kMaxModes || (int)gk.size() > kMaxModes) {
    err = "too many modes after merging";
    return false;
  }
  GenericDesc& g = out.g;
  std::memset(&g, 0, sizeof(g));
  g.nc = (int)gc.size();
  g.nk = (int)gk.size();
  g.csize = out.csize;
  g.ksize = out.ksize;
  g.pow2 = 1;
  for (int i = 0; i < g.nc; ++i) {
    g.cdim[i] = gc[i].dim;
    g.csa[i] = gc[i].sa;
    g.csb[i] = gc[i].sb;
    g.clog[i] = ilog2_exact(gc[i].dim);
    if (g.clog[i] < 0) g.pow2 = 0;
  }
  for (int i = 0; i < g.nk; ++i) {
    g.kdim[i] = gk[i].dim;
    g.ksa[i] = gk[i].sa;
    g.ksb[i] = gk[i].sb;
    g.klog[i] = ilog2_exact(gk[i].dim);
    if (g.klog[i] < 0) g.pow2 = 0;
  }
  // coalescing features: contiguous run along the first result mode
  out.run_a = (g.nc > 0 && g.csa[0] == 1) ? g.cdim[0] : ((g.nk > 0 && g.ksa[0] == 1) ? g.kdim[0] : 1);
  out.run_b = (g.nc > 0 && g.csb[0] == 1) ? g.cdim[0] : ((g.nk > 0 && g.ksb[0] == 1) ? g.kdim[0] : 1);

  // ---- GEMM descriptor: split result modes into A-only (m), B-only (n)
  // and shared (z, batch) groups, each kept in result order.
  std::vector<Mode> mm, nn, zz;
  for (const Mode& m : cm) {
    if (m.sa && !m.sb)
      mm.push_back(m);
    else if (m.sb && !m.sa)
      nn.push_back(m);
    else
      zz.push_back(m);
  }
  merge_modes(mm);
  merge_modes(nn);
  merge_modes(zz);
  if ((int)mm.size() > kMaxModes || (int)nn.size() > kMaxModes || (int)zz.size() > kMaxModes) {
    err = "too many modes after merging";
    return false;
  }
  GemmDesc& G = out.m;
  std::memset(&G, 0, sizeof(G));
  G.nm = (int)mm.size();
  G.nn = (int)nn.size();
  G.nk = (int)gk.size();
  G.nz = (int)zz.size();
  G.M = G.N = G.K = G.Z = 1;
  for (int i = 0; i < G.nm; ++i) {
    G.mdim[i] = mm[i].dim;
    G.msa[i] = mm[i].sa;
    G.msc[i] = mm[i].sc;
    G.M *= mm[i].dim;
  }
  for (int i = 0; i < G.nn; ++i) {
    G.ndim[i] = nn[i].dim;
    G.nsb[i] = nn[i].sb;
    G.nsc[i] = nn[i].sc;
    G.N *= nn[i].dim;
  }
  for (int i = 0; i < G.nk; ++i) {
    G.kdim[i] = gk[i].dim;
    G.ksa[i] = gk[i].sa;
    G.ksb[i] = gk[i].sb;
    G.K *= gk[i].dim;
  }
  for (int i = 0; i < G.nz; ++i) {
    G.zdim[i] = zz[i].dim;
    G.zsa[i] = zz[i].sa;
    G.zsb[i] = zz[i].sb;
    G.zsc[i] = zz[i].sc;
    G.Z *= zz[i].dim;
  }
  out.M = G.M;
  out.N = G.N;
  out.Z = G.Z;

  // ---- kernel class
  // A K mode present in only one operand is a plain sum; the GEMM kernels
  // need every K mode in both operands.
  bool k_both = true;
  for (const Mode& m : gk)
    if (!m.sa || !m.sb) k_both = false;
  // square tiles for M, N >= 32; the narrow tiles take one side down to 8
  const bool narrow = std::min(G.M, G.N) >= 8 && std::max(G.M, G.N) >= 256;
  bool gemm_shape = k_both && G.K >= 16 && ((G.M >= 32 && G.N >= 32) || narrow) &&
                    (double)G.M * (double)G.N * (double)G.K * (double)G.Z >= double(1 << 20);
  if (gemm_shape &&
      (precision == PQ_PREC_3XTF32 || precision == PQ_PREC_6XTF32 || precision == PQ_PREC_OZAKI ||
       precision == PQ_PREC_OZAKI4 || precision == PQ_PREC_3XBF16) &&
      tc_eligible(precision, G))
    out.kclass = KC_TC;
  else if (k_both && skinny_eligible(G))
    out.kclass = KC_SKINNY;
  else if (gemm_shape || (k_both && out.ksize > kGenericKTab && G.M >= 8 && G.N >= 8))
    out.kclass = KC_GEMM;
  else
    out.kclass = KC_GENERIC;
  out.k_both = k_both;
  out.gemm_shape = gemm_shape;
  if (tune && !tune->empty() && k_both) {
    auto it = tune->find(tuning_key(precision, G));
    if (it != tune->end() && choice_eligible(precision, out, it->second)) {
      out.kclass = (KernelClass)it->second.kclass;
      G.tile_n = it->second.kclass == KC_TC ? it->second.tile_n : 0;
      G.orient = it->second.kclass == KC_TC ? it->second.orient : 0;
      out.tuned = true;
    }
  }
  return true;
}

}  // namespace pq
