// plan.cpp -- compiles a factor graph + binary contraction tree into the
// runtime program executed by the contraction kernels (see plan.h).
//
// The network and tree are the ones TensorQEC builds in
// compile(::TNMMAP, ...) (src/decoding/tndecoder.jl:97-146, :186-219) and
// optimises with OMEinsum (tndecoder.jl:140-144).  The reference evaluates
// the tree afresh for every syndrome after writing one-hot syndrome leaves
// (tndecoder.jl:148-158); here everything that does not depend on the
// syndrome is evaluated once, on the host, in float64.
#include "plan.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <set>
#include <sstream>
#include <unordered_map>

namespace tqec {
namespace {

enum NodeKind { NK_TABLE = 0, NK_PARITY = 1, NK_RUNTIME = 2 };

struct PNode {
  int kind = NK_TABLE;
  std::vector<int> vars;      // TABLE: bit j of a data index <-> vars[j]
  std::vector<double> data;   // TABLE: 2^|sel| variants of 2^|vars| entries
  std::vector<int> sel;       // TABLE: syndrome bits choosing the variant
  int par_bit = -1;           // PARITY
  int left = -1, right = -1;  // RUNTIME children (node ids)
  int rstep = -1;             // RUNTIME: index in execution order
  bool live = true;
};

// out[c] = sum over the union of x and y of x * y, keeping `keep` (ordered).
// x/y data use "bit j <-> vars[j]".
void fold_pair(const std::vector<int>& xv, const double* xd, const std::vector<int>& yv,
               const double* yd, const std::vector<int>& keep, double* out) {
  std::vector<int> uni = xv;
  for (int v : yv)
    if (std::find(uni.begin(), uni.end(), v) == uni.end()) uni.push_back(v);
  const int nu = (int)uni.size();
  std::vector<int64_t> dx(nu, 0), dy(nu, 0), dc(nu, 0);
  for (int p = 0; p < nu; ++p) {
    auto fx = std::find(xv.begin(), xv.end(), uni[p]);
    if (fx != xv.end()) dx[p] = int64_t(1) << (fx - xv.begin());
    auto fy = std::find(yv.begin(), yv.end(), uni[p]);
    if (fy != yv.end()) dy[p] = int64_t(1) << (fy - yv.begin());
    auto fc = std::find(keep.begin(), keep.end(), uni[p]);
    if (fc != keep.end()) dc[p] = int64_t(1) << (fc - keep.begin());
  }
  const int64_t nc = int64_t(1) << keep.size();
  std::fill(out, out + nc, 0.0);
  const int64_t n = int64_t(1) << nu;
  for (int64_t u = 0; u < n; ++u) {
    int64_t ix = 0, iy = 0, ic = 0;
    for (int p = 0; p < nu; ++p)
      if ((u >> p) & 1) { ix += dx[p]; iy += dy[p]; ic += dc[p]; }
    out[ic] += xd[ix] * yd[iy];
  }
}

bool is_even_parity(const PNode& n) {
  if (n.kind != NK_TABLE || !n.sel.empty()) return false;
  const int64_t sz = int64_t(1) << n.vars.size();
  for (int64_t i = 0; i < sz; ++i) {
    double want = (__builtin_popcountll(i) & 1) ? 0.0 : 1.0;
    if (n.data[i] != want) return false;
  }
  return true;
}

// Materialises a PARITY node as a TABLE with one select bit.
PNode parity_as_table(const PNode& p) {
  PNode t;
  t.kind = NK_TABLE;
  t.vars = p.vars;
  t.sel = {p.par_bit};
  const int64_t sz = int64_t(1) << p.vars.size();
  t.data.resize(2 * sz);
  for (int s = 0; s < 2; ++s)
    for (int64_t i = 0; i < sz; ++i)
      t.data[s * sz + i] = (((__builtin_popcountll(i) & 1) ^ s) == 0) ? 1.0 : 0.0;
  return t;
}

// Sum a table over the labels not in `keep_set`.
void reduce_table(PNode& n, const std::set<int>& keep_set) {
  std::vector<int> keep;
  for (int v : n.vars)
    if (keep_set.count(v)) keep.push_back(v);
  if (keep.size() == n.vars.size()) return;
  const int64_t nvar = int64_t(1) << n.sel.size();
  const int64_t in_sz = int64_t(1) << n.vars.size();
  const int64_t out_sz = int64_t(1) << keep.size();
  std::vector<double> nd(nvar * out_sz, 0.0);
  std::vector<int64_t> dc(n.vars.size(), 0);
  for (size_t p = 0; p < n.vars.size(); ++p) {
    auto f = std::find(keep.begin(), keep.end(), n.vars[p]);
    if (f != keep.end()) dc[p] = int64_t(1) << (f - keep.begin());
  }
  for (int64_t v = 0; v < nvar; ++v)
    for (int64_t i = 0; i < in_sz; ++i) {
      int64_t ic = 0;
      for (size_t p = 0; p < n.vars.size(); ++p)
        if ((i >> p) & 1) ic += dc[p];
      nd[v * out_sz + ic] += n.data[v * in_sz + i];
    }
  n.vars = keep;
  n.data.swap(nd);
}

// Fold two TABLE nodes into one (variants over the union of select bits).
PNode fold_tables(const PNode& x, const PNode& y, const std::vector<int>& keep) {
  PNode c;
  c.kind = NK_TABLE;
  c.vars = keep;
  c.sel = x.sel;
  for (int b : y.sel)
    if (std::find(c.sel.begin(), c.sel.end(), b) == c.sel.end()) c.sel.push_back(b);
  const int m = (int)c.sel.size();
  const int64_t csz = int64_t(1) << keep.size();
  const int64_t xsz = int64_t(1) << x.vars.size();
  const int64_t ysz = int64_t(1) << y.vars.size();
  c.data.assign((int64_t(1) << m) * csz, 0.0);
  for (int64_t v = 0; v < (int64_t(1) << m); ++v) {
    int64_t vx = 0, vy = 0;
    for (int i = 0; i < m; ++i) {
      if (!((v >> i) & 1)) continue;
      auto fx = std::find(x.sel.begin(), x.sel.end(), c.sel[i]);
      if (fx != x.sel.end()) vx |= int64_t(1) << (fx - x.sel.begin());
      auto fy = std::find(y.sel.begin(), y.sel.end(), c.sel[i]);
      if (fy != y.sel.end()) vy |= int64_t(1) << (fy - y.sel.begin());
    }
    fold_pair(x.vars, x.data.data() + vx * xsz, y.vars, y.data.data() + vy * ysz, keep,
              c.data.data() + v * csz);
  }
  return c;
}

// Reorders a TABLE's data so that bit j of the index <-> layout[j].
std::vector<double> permute_table(const PNode& n, const std::vector<int>& layout) {
  const int r = (int)n.vars.size();
  std::vector<int64_t> d(r, 0);
  for (int p = 0; p < r; ++p) {
    auto f = std::find(layout.begin(), layout.end(), n.vars[p]);
    d[p] = int64_t(1) << (f - layout.begin());
  }
  const int64_t sz = int64_t(1) << r;
  const int64_t nv = int64_t(1) << n.sel.size();
  std::vector<double> out(nv * sz);
  for (int64_t v = 0; v < nv; ++v)
    for (int64_t i = 0; i < sz; ++i) {
      int64_t j = 0;
      for (int p = 0; p < r; ++p)
        if ((i >> p) & 1) j += d[p];
      out[v * sz + j] = n.data[v * sz + i];
    }
  return out;
}

}  // namespace

// Shared-memory store wavefronts of one warp's permuted output stores
// (items of `vw` consecutive outputs, lane l owning item l), with or without
// the kernel's lane rotation; rotation pays when it saves more wavefronts
// than its register selects cost.
static int store_wavefronts(const std::vector<int32_t>& perm, int32_t off, int lw, int vw, bool rotate) {
  const int lv = vw == 8 ? 3 : 2;
  if (lw < lv) return 0;
  auto addr = [&](int e) {
    int a = 0, tab = off;
    for (int sh = 0; sh < lw; sh += 8) {
      const int cb = std::min(8, lw - sh);
      a |= perm[tab + ((e >> sh) & ((1 << cb) - 1))];
      tab += 1 << cb;
    }
    return a;
  };
  const int lanes = std::min(32, 1 << (lw - lv));
  int total = 0;
  for (int s = 0; s < vw; ++s) {
    int count[32] = {0};
    for (int l = 0; l < lanes; ++l) {
      const int j = rotate ? (s + l) & (vw - 1) : s;
      count[addr((l << lv) + j) & 31]++;
    }
    total += *std::max_element(count, count + 32);
  }
  return total;
}

static bool rotation_pays(const std::vector<int32_t>& perm, int32_t off, int lw, int vw) {
  const int plain = store_wavefronts(perm, off, lw, vw, false);
  const int rot = store_wavefronts(perm, off, lw, vw, true);
  return plain - rot > (vw == 8 ? 24 : 8);
}

static std::string build_plan_once(const NetworkView& net, int32_t n_steps, const int32_t* steps,
                                   const PlanLimits& lim, Plan* out, bool* unsupported) {
  *unsupported = false;
  const int T = net.n_tensors;
  if (T < 1) return "network has no tensors";
  if (!net.ix_offsets || !net.ix_labels || !net.data_offsets || !net.data)
    return "network arrays must not be NULL";
  if (net.n_out < 0 || (!lim.map_mode && net.n_out > 16)) {
    *unsupported = net.n_out > 16;
    return "n_out must be in [0, 16]";
  }
  if (net.n_out > 0 && !net.out_labels) return "output labels must not be NULL";
  if (net.n_syndrome < 0 || (net.n_syndrome > 0 && !net.syndrome_tensors))
    return "bad syndrome leaf list";
  if (n_steps != T - 1) return "tree must have n_tensors - 1 steps";
  if (n_steps > 0 && !steps) return "tree steps must not be NULL";

  // ---- labels -> dense variable ids --------------------------------------
  std::unordered_map<int32_t, int> var_of;
  auto vid = [&](int32_t lab) {
    auto it = var_of.find(lab);
    if (it != var_of.end()) return it->second;
    int id = (int)var_of.size();
    var_of.emplace(lab, id);
    return id;
  };
  std::vector<PNode> nodes(T + n_steps);
  std::vector<int> syn_bit_of(T, -1);
  for (int j = 0; j < net.n_syndrome; ++j) {
    int p = net.syndrome_tensors[j];
    if (p < 0 || p >= T) return "syndrome leaf position out of range";
    if (syn_bit_of[p] != -1) return "syndrome leaf listed twice";
    syn_bit_of[p] = j;
  }
  for (int i = 0; i < T; ++i) {
    int32_t a = net.ix_offsets[i], b = net.ix_offsets[i + 1];
    if (a < 0 || b < a) return "ix_offsets must be non-decreasing";
    int rank = b - a;
    if (rank > 26) {
      *unsupported = true;
      return "tensor rank above 26";
    }
    PNode& n = nodes[i];
    for (int32_t q = a; q < b; ++q) {
      if (net.ix_labels[q] <= 0) return "labels must be positive";
      int v = vid(net.ix_labels[q]);
      if (std::find(n.vars.begin(), n.vars.end(), v) != n.vars.end()) {
        *unsupported = true;
        return "repeated label inside one tensor";
      }
      n.vars.push_back(v);
    }
    int64_t da = net.data_offsets[i], db = net.data_offsets[i + 1];
    if (syn_bit_of[i] >= 0) {
      if (rank != 1) return "syndrome leaves must have rank 1";
      n.kind = NK_PARITY;  // (x == s) is the parity of a one-label index
      n.par_bit = syn_bit_of[i];
      continue;
    }
    if (db - da != (int64_t(1) << rank)) {
      *unsupported = true;
      return "tensor size is not 2^rank (all dimensions must be 2)";
    }
    n.kind = NK_TABLE;
    n.data.assign(net.data + da, net.data + db);
  }
  const bool map_mode = lim.map_mode;
  std::vector<int> out_vars, report_vars;
  for (int i = 0; i < net.n_out; ++i) {
    auto it = var_of.find(net.out_labels[i]);
    if (it == var_of.end()) {
      *unsupported = true;
      return "output label does not appear in any tensor";
    }
    std::vector<int>& dst = map_mode ? report_vars : out_vars;
    if (std::find(dst.begin(), dst.end(), it->second) != dst.end()) return "repeated output label";
    dst.push_back(it->second);
  }
  const int V = (int)var_of.size();
  std::vector<int> cnt(V, 0);
  for (int i = 0; i < T; ++i)
    for (int v : nodes[i].vars) cnt[v]++;
  for (int v : out_vars) cnt[v]++;
  // labels of the syndrome leaves: evidence, never reported
  std::vector<char> is_syn_var(V, 0);
  for (int i = 0; i < T; ++i)
    if (syn_bit_of[i] >= 0) is_syn_var[nodes[i].vars[0]] = 1;
  std::vector<int8_t> fixed(V, -1);

  // ---- dead labels inside a single leaf are summed right away -------------
  for (int i = 0; i < T; ++i) {
    PNode& n = nodes[i];
    std::set<int> keep;
    bool dead = false;
    for (int v : n.vars) {
      if (cnt[v] > 1) keep.insert(v);
      else dead = true;
    }
    if (!dead) continue;
    if (map_mode) {
      // maximising over a label only this leaf carries: a one-label prior
      // decides its value on the host; anything else needs the search
      if (n.kind == NK_PARITY && n.vars.size() == 1 && is_syn_var[n.vars[0]]) {
        cnt[n.vars[0]]--;
        n.kind = NK_TABLE;
        n.vars.clear();
        n.data.assign(1, 1.0);
        n.par_bit = -1;
        continue;
      }
      if (n.kind == NK_TABLE && n.vars.size() == 1) {
        const int v = n.vars[0];
        fixed[v] = n.data[1] > n.data[0] ? 1 : 0;
        const double m = std::max(n.data[0], n.data[1]);
        cnt[v]--;
        n.vars.clear();
        n.data.assign(1, m);
        continue;
      }
      *unsupported = true;
      return "MAP mode: a label occurs in a single multi-label tensor";
    }
    if (n.kind == NK_PARITY) {
      // summing a parity indicator over one of its labels gives all ones
      for (int v : n.vars)
        if (!keep.count(v)) cnt[v]--;
      n.kind = NK_TABLE;
      n.vars.assign(keep.begin(), keep.end());
      n.data.assign(int64_t(1) << n.vars.size(), 1.0);
      n.par_bit = -1;
      continue;
    }
    for (int v : n.vars)
      if (!keep.count(v)) cnt[v]--;
    reduce_table(n, keep);
  }

  // ---- walk the tree, folding what does not need the runtime --------------
  double macs_tree = 0.0;
  std::vector<char> used(T + n_steps, 0);
  for (int s = 0; s < n_steps; ++s) {
    int x = steps[2 * s], y = steps[2 * s + 1];
    int me = T + s;
    if (x < 0 || y < 0 || x >= me || y >= me || x == y) return "tree step references an invalid node";
    if (used[x] || used[y]) return "tree uses a node twice";
    used[x] = used[y] = 1;
    PNode& nx = nodes[x];
    PNode& ny = nodes[y];
    std::vector<int> uni = nx.vars;
    for (int v : ny.vars)
      if (std::find(uni.begin(), uni.end(), v) == uni.end()) uni.push_back(v);
    macs_tree += std::ldexp(1.0, (int)uni.size());
    std::vector<int> keep;
    for (int v : uni) {
      int inx = std::count(nx.vars.begin(), nx.vars.end(), v);
      int iny = std::count(ny.vars.begin(), ny.vars.end(), v);
      if (cnt[v] - inx - iny > 0) keep.push_back(v);
    }
    for (int v : nx.vars) cnt[v]--;
    for (int v : ny.vars) cnt[v]--;
    for (int v : keep) cnt[v]++;
    if ((int)keep.size() > lim.max_width) {
      *unsupported = true;
      std::ostringstream os;
      os << "intermediate of width " << keep.size() << " exceeds the limit " << lim.max_width;
      return os.str();
    }
    PNode c;
    bool folded = false;
    // one-hot syndrome leaf meeting an even parity tensor -> parity operand
    for (int pass = 0; pass < 2 && !folded; ++pass) {
      PNode& a = pass ? ny : nx;
      PNode& b = pass ? nx : ny;
      if (a.kind == NK_PARITY && a.vars.size() == 1 && b.kind == NK_TABLE && b.sel.empty()) {
        int v = a.vars[0];
        bool in_b = std::find(b.vars.begin(), b.vars.end(), v) != b.vars.end();
        bool v_kept = std::find(keep.begin(), keep.end(), v) != keep.end();
        if (in_b && !v_kept && is_even_parity(b) && keep.size() + 1 == b.vars.size()) {
          c.kind = NK_PARITY;
          c.par_bit = a.par_bit;
          c.vars = keep;
          folded = true;
        }
      }
    }
    // MAP mode folds only products that eliminate nothing but evidence
    bool fold_ok = true;
    if (map_mode)
      for (int v : uni)
        if (std::find(keep.begin(), keep.end(), v) == keep.end() && !is_syn_var[v]) fold_ok = false;
    if (!folded && fold_ok && nx.kind != NK_RUNTIME && ny.kind != NK_RUNTIME) {
      PNode tx = nx.kind == NK_PARITY ? parity_as_table(nx) : nx;
      PNode ty = ny.kind == NK_PARITY ? parity_as_table(ny) : ny;
      std::set<int> sb(tx.sel.begin(), tx.sel.end());
      sb.insert(ty.sel.begin(), ty.sel.end());
      int nsel = (int)sb.size();
      bool ok = false;
      if (nsel == 0) ok = keep.size() <= 22 && uni.size() <= 24;
      else ok = nsel <= lim.max_sel_bits && (int)keep.size() <= lim.max_sel_rank &&
                uni.size() <= 24;
      if (ok) {
        c = fold_tables(tx, ty, keep);
        folded = true;
      }
      // too wide to fold on the host: contracted at run time like any other
      // step (its operands are constant tables)
    }
    if (!folded) {
      c.kind = NK_RUNTIME;
      c.vars = keep;
      c.left = x;
      c.right = y;
    }
    nodes[me] = std::move(c);
  }
  const int root_id = T + n_steps - 1;
  {
    std::vector<int> rv = nodes[root_id].vars, ov = out_vars;
    std::sort(rv.begin(), rv.end());
    std::sort(ov.begin(), ov.end());
    if (rv != ov) return "the tree's root does not carry exactly the output labels";
  }
  // A root that is not a runtime node is materialised by multiplying it with
  // a scalar one.
  int root = root_id;
  if (nodes[root].kind != NK_RUNTIME) {
    PNode one;
    one.kind = NK_TABLE;
    one.data = {1.0};
    nodes.push_back(one);
    PNode r;
    r.kind = NK_RUNTIME;
    r.vars = nodes[root].vars;
    r.left = root;
    r.right = (int)nodes.size() - 1;
    nodes.push_back(r);
    root = (int)nodes.size() - 1;
  }

  // ---- execution order: children with the larger peak first ---------------
  std::vector<double> peak(nodes.size(), 0.0);
  std::vector<char> first_right(nodes.size(), 0);
  std::vector<int> order;
  std::function<void(int)> peak_of = [&](int id) {
    PNode& n = nodes[id];
    if (n.kind != NK_RUNTIME) return;
    peak_of(n.left);
    peak_of(n.right);
    double me = std::ldexp(1.0, (int)n.vars.size());
    auto sz = [&](int c) { return nodes[c].kind == NK_RUNTIME ? std::ldexp(1.0, (int)nodes[c].vars.size()) : 0.0; };
    double pl = peak[n.left], pr = peak[n.right], sl = sz(n.left), sr = sz(n.right);
    double lf = std::max({pl, sl + pr, sl + sr + me});
    double rf = std::max({pr, sr + pl, sl + sr + me});
    first_right[id] = rf < lf;
    peak[id] = std::min(lf, rf);
  };
  peak_of(root);
  std::function<void(int)> post = [&](int id) {
    PNode& n = nodes[id];
    if (n.kind != NK_RUNTIME) return;
    if (first_right[id]) { post(n.right); post(n.left); }
    else { post(n.left); post(n.right); }
    n.rstep = (int)order.size();
    order.push_back(id);
  };
  post(root);
  if (lim.level_order) {
    // level of a runtime step: one more than the deepest runtime step it reads
    std::vector<int> level(nodes.size(), 0);
    for (int id : order) {  // children come first in the post-order
      const PNode& n = nodes[id];
      int l = 0;
      for (int c : {n.left, n.right})
        if (nodes[c].kind == NK_RUNTIME) l = std::max(l, level[c]);
      level[id] = l + 1;
    }
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return level[x] < level[y]; });
    for (int r = 0; r < (int)order.size(); ++r) nodes[order[r]].rstep = r;
  }
  const int R = (int)order.size();
  // A parity operand of a runtime step becomes a two-variant table selected
  // by its syndrome bit: the kernel then reads only arena and constant
  // operands (one code path per step shape, a smaller kernel).
  for (int id : order)
    for (int op : {nodes[id].left, nodes[id].right})
      if (nodes[op].kind == NK_PARITY) nodes[op] = parity_as_table(nodes[op]);

  // ---- layouts --------------------------------------------------------------
  struct StepLayout {
    std::vector<int> H, Fa, Fb, K;  // ordered groups
    int a = -1, b = -1;             // operand node ids
    std::vector<int> out_layout;    // required layout of the output
    bool tensor = false;            // GEMM-shaped (B read K-major)
  };
  std::vector<StepLayout> lay(R);
  // Group orders are assigned bottom-up: a step orders each of its index
  // groups by the position its labels hold in the producing step's natural
  // output order ([fb][fa][h], fb lowest), so an intermediate's lowest
  // natural bits (the ones adjacent threads differ in when they write it)
  // stay among the lowest address bits of the layout its consumer reads.
  // Stores then spread over the shared-memory banks.  The root's natural
  // order is permuted into the output order at the last step.
  std::map<int, std::vector<int>> nat;  // runtime node id -> natural order (bit 0 first)
  for (int r = 0; r < R; ++r) {
    const int id = order[r];
    PNode& n = nodes[id];
    StepLayout& L = lay[r];
    const std::vector<int>& lv = nodes[n.left].vars;
    const std::vector<int>& rv = nodes[n.right].vars;
    auto in = [](const std::vector<int>& s, int v) { return std::find(s.begin(), s.end(), v) != s.end(); };
    std::vector<int> fl, fr;
    for (int v : lv)
      if (!in(rv, v)) fl.push_back(v);
    for (int v : rv)
      if (!in(lv, v)) fr.push_back(v);
    // the operand with more free labels goes innermost (B), so that adjacent
    // threads read adjacent B elements -- except for a GEMM-shaped step,
    // whose A side (the 128-row tiles) is the operand with more free labels
    bool swap = fl.size() > fr.size();
    {
      int nk = 0;
      for (int v : lv)
        if (in(rv, v) && !in(n.vars, v)) ++nk;
      const int big = (int)std::max(fl.size(), fr.size()), small = (int)std::min(fl.size(), fr.size());
      auto sel_free = [&](int node) { return nodes[node].kind != NK_TABLE || nodes[node].sel.empty(); };
      L.tensor = lim.tensor_steps && !map_mode && big >= kTensorMinFa && small >= kTensorMinFb &&
                 nk >= kTensorMinK && sel_free(n.left) && sel_free(n.right) &&
                 nodes[n.left].kind != NK_PARITY && nodes[n.right].kind != NK_PARITY;
      if (L.tensor) swap = fr.size() > fl.size();
    }
    L.a = swap ? n.right : n.left;
    L.b = swap ? n.left : n.right;
    const std::vector<int>& av = nodes[L.a].vars;
    const std::vector<int>& bv = nodes[L.b].vars;
    for (int v : av) {
      if (in(bv, v)) (in(n.vars, v) ? L.H : L.K).push_back(v);
      else L.Fa.push_back(v);
    }
    for (int v : bv)
      if (!in(av, v)) L.Fb.push_back(v);
    // position of a label in an operand's natural order (leaves: label id)
    auto natpos = [&](int node, int v) {
      auto it = nat.find(node);
      if (it == nat.end()) return 1000000 + v;
      const std::vector<int>& o = it->second;
      return int(std::find(o.begin(), o.end(), v) - o.begin());
    };
    auto order_by = [&](std::vector<int>& g, int node) {
      std::sort(g.begin(), g.end(), [&](int p, int q) { return natpos(node, p) < natpos(node, q); });
    };
    order_by(L.Fb, L.b);
    order_by(L.Fa, L.a);
    order_by(L.H, L.b);
    // contracted labels follow the larger intermediate operand's natural order
    {
      const bool ra = nat.count(L.a) > 0, rb = nat.count(L.b) > 0;
      int pick = L.b;
      if (ra && (!rb || nodes[L.a].vars.size() > nodes[L.b].vars.size())) pick = L.a;
      order_by(L.K, pick);
    }
    std::vector<int> nn;
    nn.insert(nn.end(), L.Fb.begin(), L.Fb.end());
    nn.insert(nn.end(), L.Fa.begin(), L.Fa.end());
    nn.insert(nn.end(), L.H.begin(), L.H.end());
    nat[id] = nn;
  }
  Plan& P = *out;
  P = Plan();
  P.n_syndrome = net.n_syndrome;
  P.syndrome_bytes = (net.n_syndrome + 7) / 8;
  P.n_out = map_mode ? 0 : net.n_out;
  P.n_classes = map_mode ? 1 : 1 << net.n_out;
  P.n_tree_steps = n_steps;
  P.macs_tree = macs_tree;
  std::map<int, std::pair<int64_t, std::vector<int8_t>>> const_ref;  // node -> (offset, sel)
  std::map<int, std::vector<int>> req;  // node id -> required (read) layout
  double err_terms = 0.0;
  for (int r = 0; r < R; ++r) {
    const int id = order[r];
    StepLayout& L = lay[r];
    std::vector<int> la, lb;
    la.insert(la.end(), L.K.begin(), L.K.end());
    la.insert(la.end(), L.Fa.begin(), L.Fa.end());
    la.insert(la.end(), L.H.begin(), L.H.end());
    if (L.tensor) {  // [h][fb][k]: K-major like A
      lb.insert(lb.end(), L.K.begin(), L.K.end());
      lb.insert(lb.end(), L.Fb.begin(), L.Fb.end());
    } else {
      lb.insert(lb.end(), L.Fb.begin(), L.Fb.end());
      lb.insert(lb.end(), L.K.begin(), L.K.end());
    }
    lb.insert(lb.end(), L.H.begin(), L.H.end());
    req[L.a] = la;
    req[L.b] = lb;
    // float32 rounding of the K products and sums; a tensor-core step splits
    // each operand into two tf32 halves (three products, the dropped and
    // truncated parts below 3 x 2^-20 of each product, i.e. 48u) and may
    // accumulate with twice the rounding of round-to-nearest
    const double kk = std::ldexp(1.0, (int)L.K.size());
    err_terms += L.tensor ? 2.0 * (kk + 1.0) + 48.0 : kk + 1.0;
    for (int op : {L.a, L.b}) {
      PNode& o = nodes[op];
      if (o.kind != NK_TABLE) continue;
      std::vector<double> d = permute_table(o, req[op]);
      int64_t off = (int64_t)P.consts.size();
      // keep every constant operand 16-byte aligned for float and double
      P.consts.insert(P.consts.end(), d.begin(), d.end());
      while (P.consts.size() % 4) P.consts.push_back(0.0);
      std::vector<int8_t> sel(kMaxSel, -1);
      if ((int)o.sel.size() > kMaxSel) return "internal: too many select bits";
      for (size_t i = 0; i < o.sel.size(); ++i) sel[i] = (int8_t)o.sel[i];
      const_ref[op] = {off, sel};
      err_terms += 1.0;
    }
    (void)id;
  }
  req[root] = out_vars;
  for (int r = 0; r < R; ++r) lay[r].out_layout = req.at(order[r]);
  if (P.consts.size() > (size_t)INT32_MAX) {
    *unsupported = true;
    return "constant data above 2^31 entries";
  }

  // ---- arena: first fit in execution order, in two pools ------------------
  // Intermediates of more than kBigElems elements go to the big pool, the
  // rest to the small pool; a launch may keep the small pool in shared memory
  // and the big pool in global memory.  Offsets: small pool [0, S), big pool
  // [S, S + B) once S is known (patched after allocation).
  const int64_t kBigElems = lim.big_elems > 0 ? lim.big_elems : 1024;
  struct Block { int64_t off, size; };
  struct Pool {
    std::vector<Block> free_list = {{0, int64_t(1) << 40}};
    int64_t top = 0;
    int64_t alloc(int64_t sz) {
      sz = (sz + 7) & ~int64_t(7);
      for (size_t i = 0; i < free_list.size(); ++i) {
        if (free_list[i].size >= sz) {
          int64_t off = free_list[i].off;
          free_list[i].off += sz;
          free_list[i].size -= sz;
          if (free_list[i].size == 0) free_list.erase(free_list.begin() + i);
          top = std::max(top, off + sz);
          return off;
        }
      }
      return int64_t(-1);
    }
    void release(int64_t off, int64_t sz) {
      sz = (sz + 7) & ~int64_t(7);
      free_list.push_back({off, sz});
      std::sort(free_list.begin(), free_list.end(), [](const Block& a, const Block& b) { return a.off < b.off; });
      std::vector<Block> merged;
      for (const Block& b : free_list) {
        if (!merged.empty() && merged.back().off + merged.back().size == b.off) merged.back().size += b.size;
        else merged.push_back(b);
      }
      free_list.swap(merged);
    }
  };
  Pool small_pool, big_pool;
  std::vector<int64_t> arena_off(nodes.size(), -1);
  std::vector<char> in_big(nodes.size(), 0);
  auto alloc_node = [&](int id, int64_t sz) {
    in_big[id] = sz > kBigElems;
    arena_off[id] = (in_big[id] ? big_pool : small_pool).alloc(sz);
    return arena_off[id];
  };
  auto release_node = [&](int id, int64_t sz) { (in_big[id] ? big_pool : small_pool).release(arena_off[id], sz); };
  // ---- barrier groups: consecutive steps that do not read each other's
  // outputs run between the same pair of block barriers.  Wide steps stay
  // alone (they fill the block by themselves and dominate the arena).
  std::vector<char> group_end(R, 0);
  {
    const int kMaxGroup = lim.level_order ? 16 : 8;
    const int kMaxGroupedWidth = lim.level_order ? 64 : 12;
    std::vector<char> in_group(nodes.size(), 0);
    std::vector<int> members;
    for (int r = 0; r < R; ++r) {
      const int id = order[r];
      const StepLayout& L = lay[r];
      const bool wide = (int)nodes[id].vars.size() > kMaxGroupedWidth;
      bool dep = false;
      for (int op : {L.a, L.b})
        if (nodes[op].kind == NK_RUNTIME && in_group[op]) dep = true;
      if (r > 0 && (dep || wide || (int)members.size() >= kMaxGroup ||
                    (int)nodes[order[r - 1]].vars.size() > kMaxGroupedWidth)) {
        group_end[r - 1] = 1;
        for (int m : members) in_group[m] = 0;
        members.clear();
      }
      in_group[id] = 1;
      members.push_back(id);
    }
    group_end[R - 1] = 1;
  }
  int width = 0;
  double macs_rt = 0.0;
  P.steps.resize(R);
  std::vector<int> pending_release;
  int32_t d_var_off = 0;
  for (int r = 0; r < R; ++r) {
    const int id = order[r];
    PNode& n = nodes[id];
    StepLayout& L = lay[r];
    const int64_t osz = int64_t(1) << n.vars.size();
    width = std::max(width, (int)n.vars.size());
    int64_t off = alloc_node(id, osz);
    // operands are freed when the whole barrier group has run
    for (int op : {L.a, L.b})
      if (nodes[op].kind == NK_RUNTIME) pending_release.push_back(op);
    if (group_end[r]) {
      if (!map_mode)  // MAP back-tracking reads every intermediate again
        for (int op : pending_release) release_node(op, int64_t(1) << nodes[op].vars.size());
      pending_release.clear();
    }
    if (map_mode) {
      d_var_off = (int32_t)P.vartab.size();
      for (const std::vector<int>* g : {&L.Fb, &L.Fa, &L.H, &L.K}) P.vartab.insert(P.vartab.end(), g->begin(), g->end());
    }
    macs_rt += std::ldexp(1.0, (int)(L.H.size() + L.Fa.size() + L.Fb.size() + L.K.size()));
    StepDesc d;
    std::memset(&d, 0, sizeof(d));
    d.lh = (int)L.H.size();
    d.lfa = (int)L.Fa.size();
    d.lfb = (int)L.Fb.size();
    d.lk = (int)L.K.size();
    d.out_off = (int32_t)off;
    d.flags = (group_end[r] ? kStepSync : 0) | (L.tensor ? kStepTensor : 0);
    if (L.tensor) P.tensor_steps++;
    d.var_off = map_mode ? d_var_off : 0;
    for (int side = 0; side < 2; ++side) {
      int op = side ? L.b : L.a;
      PNode& o = nodes[op];
      int32_t kind, ref, prod = -1;
      int8_t sel[kMaxSel] = {-1, -1, -1, -1};
      if (o.kind == NK_RUNTIME) {
        kind = OP_ARENA;
        ref = (int32_t)arena_off[op];
        prod = o.rstep;
      } else if (o.kind == NK_PARITY) {
        kind = OP_PARITY;
        ref = o.par_bit;
      } else {
        kind = OP_CONST;
        auto& cr = const_ref.at(op);
        ref = (int32_t)cr.first;
        for (int i = 0; i < kMaxSel; ++i) sel[i] = cr.second[i];
      }
      if (side == 0) { d.a_kind = kind; d.a_ref = ref; d.a_prod = prod; std::memcpy(d.a_sel, sel, kMaxSel); }
      else { d.b_kind = kind; d.b_ref = ref; d.b_prod = prod; std::memcpy(d.b_sel, sel, kMaxSel); }
    }
    // natural output order: Fb (low bits), Fa, H (high bits)
    std::vector<int> nat;
    nat.insert(nat.end(), L.Fb.begin(), L.Fb.end());
    nat.insert(nat.end(), L.Fa.begin(), L.Fa.end());
    nat.insert(nat.end(), L.H.begin(), L.H.end());
    const std::vector<int>& want = L.out_layout;
    bool ident = nat == want;
    if (ident) {
      d.perm_off = -1;
    } else {
      // tables start on a multiple of 8 entries (16-byte vector loads of the
      // low table, as int32 or as uint16)
      while (P.perm.size() % 8) P.perm.push_back(0);
      d.perm_off = (int32_t)P.perm.size();
      const int nb = (int)nat.size();
      for (int c0 = 0; c0 < nb; c0 += 8) {
        int cb = std::min(8, nb - c0);
        for (int v = 0; v < (1 << cb); ++v) {
          int32_t a = 0;
          for (int q = 0; q < cb; ++q)
            if ((v >> q) & 1) {
              int var = nat[c0 + q];
              int dst = int(std::find(want.begin(), want.end(), var) - want.begin());
              a |= int32_t(1) << dst;
            }
          P.perm.push_back(a);
        }
      }
      for (int vw : {4, 8})
        if (rotation_pays(P.perm, d.perm_off, nb, vw)) d.flags |= vw == 4 ? kStepRotate4 : kStepRotate8;
    }
    P.steps[r] = d;
  }
  P.width = width;
  if (map_mode) {
    P.map_mode = true;
    P.n_vars = V;
    P.fixed = fixed;
    P.report.assign(report_vars.begin(), report_vars.end());
    // every reported label is decided by some step's k group or on the host
    std::vector<char> decided(V, 0);
    for (int r = 0; r < R; ++r)
      for (int v : lay[r].K) decided[v] = 1;
    for (int v = 0; v < V; ++v)
      if (fixed[v] >= 0) decided[v] = 1;
    for (int v : report_vars)
      if (!decided[v]) {
        *unsupported = true;
        return "MAP mode: a reported label is never maximised over (is it an output of the tree?)";
      }
  }
  // the big pool follows the small one: patch its tensors' offsets
  const int64_t S = (small_pool.top + 31) & ~int64_t(31);
  const int64_t Bg = (big_pool.top + 31) & ~int64_t(31);
  for (int r = 0; r < R; ++r) {
    StepDesc& d = P.steps[r];
    if (in_big[order[r]]) d.out_off += (int32_t)S;
    if (d.a_kind == OP_ARENA && in_big[order[d.a_prod]]) d.a_ref += (int32_t)S;
    if (d.b_kind == OP_ARENA && in_big[order[d.b_prod]]) d.b_ref += (int32_t)S;
  }
  P.arena_small = Bg > 0 ? S : 0;
  P.arena_elems = std::max<int64_t>(S + Bg, 32);
  P.root_step = R - 1;
  P.macs_runtime = macs_rt;
  P.err_terms = err_terms;
  if (P.arena_elems > (int64_t(1) << 31)) {
    *unsupported = true;
    return "per-syndrome working set above 2^31 elements";
  }
  return "";
}

// Tensor-core steps pay only when they carry a good share of the work: the
// kernel instantiation that runs them has fewer threads and registers per
// block and holds the staging buffers in shared memory, which slows every
// other step.  Below lim.tensor_min_share of the multiply-adds the program is
// planned again without them.
std::string build_plan(const NetworkView& net, int32_t n_steps, const int32_t* steps,
                       const PlanLimits& lim, Plan* out, bool* unsupported) {
  std::string err = build_plan_once(net, n_steps, steps, lim, out, unsupported);
  if (!err.empty() || out->tensor_steps == 0) return err;
  double all = 0.0, tc = 0.0;
  for (const StepDesc& d : out->steps) {
    const double m = std::ldexp(1.0, d.lh + d.lfa + d.lfb + d.lk);
    all += m;
    if (d.flags & kStepTensor) tc += m;
  }
  if (tc >= lim.tensor_min_share * all) return err;
  PlanLimits simt = lim;
  simt.tensor_steps = false;
  *out = Plan();
  return build_plan_once(net, n_steps, steps, simt, out, unsupported);
}

}  // namespace tqec
