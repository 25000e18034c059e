// order.cpp -- contraction-order search for binary-label factor graphs.
//
// Stands in for OMEinsum's optimize_code(code, uniformsize(code, 2),
// TreeSA()) (src/decoding/tndecoder.jl:140-144): a randomised greedy pass
// (many trials, Gumbel-perturbed pair costs) seeds a tree that simulated
// annealing then improves by local rotations ((A,(B,C)) -> ((A,B),C) or
// ((A,C),B)).  The objective is log2 of the multiply-adds of the tree plus a
// penalty per label of width above a target, because the width decides
// whether a syndrome's working set fits in shared memory.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <queue>
#include <random>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/tqec_gb300.h"

namespace tqec {
std::string& last_error_ref();
}  // namespace tqec

namespace {

struct VC {  // a label and how many leaves of the subtree carry it
  int v;
  int c;
};

struct Problem {
  int T = 0;                          // leaves
  int V = 0;                          // labels
  std::vector<std::vector<int>> leaf; // labels per leaf
  std::vector<int> total;             // leaves carrying each label
  std::vector<char> is_out;
  double tdisc = 1.0;                 // cost divisor of GEMM-shaped steps
};

// kept labels of merging x and y (each sorted by label)
void merge_sets(const Problem& P, const std::vector<VC>& x, const std::vector<VC>& y, std::vector<VC>* out,
                int* union_size) {
  out->clear();
  size_t i = 0, j = 0;
  int u = 0;
  while (i < x.size() || j < y.size()) {
    VC e;
    if (j >= y.size() || (i < x.size() && x[i].v < y[j].v)) e = x[i++];
    else if (i >= x.size() || y[j].v < x[i].v) e = y[j++];
    else { e = {x[i].v, x[i].c + y[j].c}; ++i; ++j; }
    ++u;
    if (e.c < P.total[e.v] || P.is_out[e.v]) out->push_back(e);
  }
  *union_size = u;
}

struct Tree {
  // nodes 0..T-1 leaves, T..2T-2 internal
  std::vector<int> l, r, parent;
  std::vector<std::vector<VC>> sets;
  std::vector<int> uni;  // union size of an internal node
  int root = -1;
};

// The cost of internal node n: its multiply-adds, divided by P.tdisc when
// the step is GEMM-shaped -- labels kept from one child only (fa, fb), labels
// summed (k): |k| >= 5 and one of fa, fb >= 7 with the other >= 5.
double node_cost(const Problem& P, const Tree& t, int n) {
  const double m = std::ldexp(1.0, t.uni[n]);
  if (P.tdisc <= 1.0) return m;
  const std::vector<VC>& X = t.sets[t.l[n]];
  const std::vector<VC>& Y = t.sets[t.r[n]];
  const std::vector<VC>& O = t.sets[n];
  size_t i = 0, j = 0, o = 0;
  int fx = 0, fy = 0, kk = 0;
  while (i < X.size() || j < Y.size()) {
    int v;
    bool inx = false, iny = false;
    if (j >= Y.size() || (i < X.size() && X[i].v < Y[j].v)) { v = X[i++].v; inx = true; }
    else if (i >= X.size() || Y[j].v < X[i].v) { v = Y[j++].v; iny = true; }
    else { v = X[i].v; ++i; ++j; inx = iny = true; }
    while (o < O.size() && O[o].v < v) ++o;
    const bool kept = o < O.size() && O[o].v == v;
    if (!kept) ++kk;
    else if (inx && !iny) ++fx;
    else if (iny && !inx) ++fy;
  }
  const bool gemm = kk >= 5 && ((fx >= 7 && fy >= 5) || (fy >= 7 && fx >= 5));
  return gemm ? m / P.tdisc : m;
}

double tree_macs(const Problem& P, const Tree& t) {
  double s = 0;
  for (int i = P.T; i < (int)t.l.size(); ++i) s += node_cost(P, t, i);
  return s;
}

int tree_width(const Tree& t, int T) {
  int w = 0;
  for (int i = T; i < (int)t.l.size(); ++i) w = std::max(w, (int)t.sets[i].size());
  return w;
}

double energy(double macs, int width, int target, double wpen) {
  return std::log2(std::max(macs, 1.0)) + wpen * std::max(0, width - target);
}

// One randomised greedy pass; fills `t` (internal nodes in merge order).
void greedy(const Problem& P, std::mt19937_64& rng, double temp, Tree* t) {
  const int T = P.T;
  t->l.assign(2 * T - 1, -1);
  t->r.assign(2 * T - 1, -1);
  t->parent.assign(2 * T - 1, -1);
  t->sets.assign(2 * T - 1, {});
  t->uni.assign(2 * T - 1, 0);
  std::vector<int> cnt(P.V, 0);
  for (int i = 0; i < T; ++i) {
    std::vector<int> s = P.leaf[i];
    std::sort(s.begin(), s.end());
    for (int v : s) t->sets[i].push_back({v, 1});
  }
  for (int v = 0; v < P.V; ++v) cnt[v] = P.total[v];
  std::vector<std::vector<int>> holders(P.V);
  for (int i = 0; i < T; ++i)
    for (auto& e : t->sets[i]) holders[e.v].push_back(i);
  std::vector<char> live(2 * T - 1, 0);
  for (int i = 0; i < T; ++i) live[i] = 1;
  std::uniform_real_distribution<double> U(1e-12, 1.0);
  struct Cand {
    double cost;
    int a, b;
    bool operator<(const Cand& o) const { return cost > o.cost; }
  };
  std::priority_queue<Cand> heap;
  std::vector<VC> tmp;
  auto pair_cost = [&](int a, int b) {
    int u;
    // kept labels: those still carried by other live nodes or the output;
    // per-subtree counts against the global totals give exactly that
    merge_sets(P, t->sets[a], t->sets[b], &tmp, &u);
    double c = std::ldexp(1.0, (int)tmp.size()) - std::ldexp(1.0, (int)t->sets[a].size()) -
               std::ldexp(1.0, (int)t->sets[b].size());
    if (temp > 0) c -= temp * std::log(-std::log(U(rng)));
    return c;
  };
  auto push_neighbours = [&](int a) {
    std::vector<int> nb;
    for (auto& e : t->sets[a])
      for (int h : holders[e.v])
        if (h != a && live[h]) nb.push_back(h);
    std::sort(nb.begin(), nb.end());
    nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
    for (int b : nb) heap.push({pair_cost(a, b), std::min(a, b), std::max(a, b)});
  };
  for (int i = 0; i < T; ++i) {
    std::vector<int> nb;
    for (auto& e : t->sets[i])
      for (int h : holders[e.v])
        if (h > i) nb.push_back(h);
    std::sort(nb.begin(), nb.end());
    nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
    for (int b : nb) heap.push({pair_cost(i, b), i, b});
  }
  int next = T;
  int nlive = T;
  while (nlive > 1) {
    int a = -1, b = -1;
    while (!heap.empty()) {
      Cand c = heap.top();
      heap.pop();
      if (live[c.a] && live[c.b]) { a = c.a; b = c.b; break; }
    }
    if (a < 0) {  // disconnected: merge the two smallest live nodes
      std::vector<std::pair<int, int>> ls;
      for (int i = 0; i < next; ++i)
        if (live[i]) ls.push_back({(int)t->sets[i].size(), i});
      std::sort(ls.begin(), ls.end());
      a = ls[0].second;
      b = ls[1].second;
    }
    int u;
    merge_sets(P, t->sets[a], t->sets[b], &t->sets[next], &u);
    t->uni[next] = u;
    t->l[next] = a;
    t->r[next] = b;
    t->parent[a] = t->parent[b] = next;
    live[a] = live[b] = 0;
    live[next] = 1;
    for (auto& e : t->sets[next]) holders[e.v].push_back(next);
    push_neighbours(next);
    ++next;
    --nlive;
  }
  t->root = next - 1;
}

void recompute(const Problem& P, Tree* t, int n) {
  int u;
  merge_sets(P, t->sets[t->l[n]], t->sets[t->r[n]], &t->sets[n], &u);
  t->uni[n] = u;
}

// Simulated annealing over rotations at random internal nodes.
void anneal(const Problem& P, Tree* t, std::mt19937_64& rng, int sweeps, int target, double wpen) {
  Tree best_tree = *t;
  const int T = P.T;
  const int N = 2 * T - 1;
  if (T < 3) return;
  std::vector<int> wcount(64, 0);
  double macs = 0;
  for (int i = T; i < N; ++i) {
    macs += node_cost(P, *t, i);
    wcount[std::min<int>(63, (int)t->sets[i].size())]++;
  }
  auto width_of = [&]() {
    for (int w = 63; w >= 0; --w)
      if (wcount[w]) return w;
    return 0;
  };
  double E = energy(macs, width_of(), target, wpen);
  double best_E = E;
  std::uniform_int_distribution<int> pick(T, N - 1);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  std::vector<VC> save_set;
  const double beta0 = 4.0, beta1 = 80.0;
  const int per = std::max(1, 10 * T);
  for (int s = 0; s < sweeps; ++s) {
    const double beta = beta0 * std::pow(beta1 / beta0, double(s) / std::max(1, sweeps - 1));
    for (int it = 0; it < per; ++it) {
      const int x = pick(rng);
      int a = t->l[x], b = t->r[x];
      // choose an internal child to rotate through
      int inner, outer;
      if (b >= T && (a < T || U(rng) < 0.5)) { inner = b; outer = a; }
      else if (a >= T) { inner = a; outer = b; }
      else continue;
      const int c = t->l[inner], d = t->r[inner];
      const bool keep_c = U(rng) < 0.5;  // new inner = (outer, c) or (outer, d)
      const int join = keep_c ? c : d;
      const int other = keep_c ? d : c;
      // old local cost
      const double old_local = node_cost(P, *t, inner) + node_cost(P, *t, x);
      const int old_w_inner = (int)t->sets[inner].size();
      save_set = t->sets[inner];
      const int save_uni = t->uni[inner];
      // apply: inner = (outer, join); x = (inner, other)
      t->l[inner] = outer; t->r[inner] = join;
      t->parent[outer] = inner; t->parent[join] = inner;
      t->l[x] = inner; t->r[x] = other;
      t->parent[other] = x; t->parent[inner] = x;
      recompute(P, t, inner);
      const int old_ux = t->uni[x];
      recompute(P, t, x);  // x's set is unchanged (same leaves), union may differ
      const double new_local = node_cost(P, *t, inner) + node_cost(P, *t, x);
      const double nmacs = macs - old_local + new_local;
      wcount[std::min(63, old_w_inner)]--;
      wcount[std::min<int>(63, (int)t->sets[inner].size())]++;
      const double nE = energy(nmacs, width_of(), target, wpen);
      if (nE <= E || U(rng) < std::exp(-beta * (nE - E))) {
        macs = nmacs;
        E = nE;
        if (E < best_E - 1e-12) {
          best_E = E;
          best_tree = *t;
        }
      } else {  // undo
        wcount[std::min<int>(63, (int)t->sets[inner].size())]--;
        wcount[std::min(63, old_w_inner)]++;
        t->l[inner] = c; t->r[inner] = d;
        t->parent[c] = inner; t->parent[d] = inner;
        t->l[x] = a; t->r[x] = b;
        t->parent[a] = x; t->parent[b] = x;
        t->sets[inner] = save_set;
        t->uni[inner] = save_uni;
        t->uni[x] = old_ux;
      }
    }
  }
  *t = best_tree;
}

// Emits steps in post-order (children before parents); node ids follow the
// tqec_tree convention.  `leaf_id` maps the search's leaves to node ids of
// the caller's network and `next` is the first free step index (steps before
// it were emitted by the caller).
void emit(const Tree& t, int T, const std::vector<int>& leaf_id, int next, int n_net, int32_t* steps) {
  std::vector<int> id(t.l.size(), -1);
  for (int i = 0; i < T; ++i) id[i] = leaf_id[i];
  std::vector<std::pair<int, int>> stack = {{t.root, 0}};
  while (!stack.empty()) {
    auto [n, state] = stack.back();
    stack.pop_back();
    if (n < T) continue;
    if (state == 0) {
      stack.push_back({n, 1});
      stack.push_back({t.r[n], 0});
      stack.push_back({t.l[n], 0});
    } else {
      steps[2 * next] = id[t.l[n]];
      steps[2 * next + 1] = id[t.r[n]];
      id[n] = n_net + next;
      ++next;
    }
  }
}

}  // namespace

extern "C" int tqec_optimize_order(const tqec_network* net, const tqec_order_options* opts, int32_t* steps_out,
                                   double* log2_macs_out, int32_t* width_out) {
  auto invalid = [](const char* m) {
    tqec::last_error_ref() = m;
    return TQEC_ERR_INVALID;
  };
  if (!net || !steps_out || net->n_tensors < 1 || !net->ix_offsets || !net->ix_labels)
    return invalid("NULL argument or empty network");
  if (net->n_out < 0 || (net->n_out > 0 && !net->out_labels)) return invalid("bad output label list");
  for (int i = 0; i < net->n_tensors; ++i)
    if (net->ix_offsets[i] < 0 || net->ix_offsets[i + 1] < net->ix_offsets[i])
      return invalid("ix_offsets must be non-negative and non-decreasing");
  tqec_order_options o;
  std::memset(&o, 0, sizeof(o));
  o.trials = 32;
  o.sweeps = 60;
  o.target_width = 0;
  o.width_penalty = 1.0;
  o.seed = 1;
  if (opts) o = *opts;
  const int NT = net->n_tensors;
  std::unordered_map<int32_t, int> var_of;
  std::vector<std::vector<int>> net_leaf(NT);
  for (int i = 0; i < NT; ++i)
    for (int32_t q = net->ix_offsets[i]; q < net->ix_offsets[i + 1]; ++q) {
      auto it = var_of.find(net->ix_labels[q]);
      int v;
      if (it == var_of.end()) {
        v = (int)var_of.size();
        var_of.emplace(net->ix_labels[q], v);
      } else {
        v = it->second;
      }
      net_leaf[i].push_back(v);
    }
  const int V = (int)var_of.size();
  std::vector<int> total(V, 0);
  std::vector<char> is_out(V, 0);
  for (int i = 0; i < NT; ++i)
    for (int v : net_leaf[i]) total[v]++;
  for (int i = 0; i < net->n_out; ++i) {
    auto it = var_of.find(net->out_labels[i]);
    if (it != var_of.end()) is_out[it->second] = 1;
  }
  // A one-hot syndrome leaf whose label one other tensor carries is merged
  // with that tensor before the search: the planner folds the pair into a
  // parity or selected-table operand, so the syndrome label never becomes a
  // runtime dimension and must not count in the search's cost or width.
  std::vector<int> group(NT);
  for (int i = 0; i < NT; ++i) group[i] = i;
  std::function<int(int)> find = [&](int x) { return group[x] == x ? x : group[x] = find(group[x]); };
  std::vector<std::pair<int, int>> pre;  // (syndrome leaf, partner)
  if (net->syndrome_tensors)
    for (int j = 0; j < net->n_syndrome; ++j) {
      const int sl = net->syndrome_tensors[j];
      if (sl < 0 || sl >= NT || net_leaf[sl].size() != 1) continue;
      const int v = net_leaf[sl][0];
      if (total[v] != 2 || is_out[v]) continue;
      int partner = -1;
      for (int i = 0; i < NT; ++i)
        if (i != sl && std::find(net_leaf[i].begin(), net_leaf[i].end(), v) != net_leaf[i].end()) partner = i;
      if (partner < 0 || find(partner) == find(sl)) continue;
      pre.push_back({sl, partner});
      group[find(sl)] = find(partner);
    }
  // the search's leaves: one per group, carrying the labels that leave it
  Problem P;
  std::vector<int> rep_leaf(NT, -1);
  std::vector<std::vector<int>> members;
  for (int i = 0; i < NT; ++i) {
    const int g = find(i);
    if (rep_leaf[g] < 0) {
      rep_leaf[g] = (int)members.size();
      members.push_back({});
    }
    members[rep_leaf[g]].push_back(i);
  }
  P.T = (int)members.size();
  P.V = V;
  P.tdisc = o.tensor_discount > 1.0 ? o.tensor_discount : 1.0;
  P.total = total;
  P.is_out = is_out;
  P.leaf.resize(P.T);
  for (int k = 0; k < P.T; ++k) {
    std::unordered_map<int, int> c;
    for (int i : members[k])
      for (int v : net_leaf[i]) c[v]++;
    for (auto& [v, n] : c)
      if (n < total[v] || is_out[v]) P.leaf[k].push_back(v);
    for (auto& [v, n] : c)
      if (n == total[v] && !is_out[v]) P.total[v] = 0;  // contracted inside the group
  }
  // pre-merge steps: the members of each group, left to right
  std::vector<int> leaf_id(P.T);
  int next_step = 0;
  for (int k = 0; k < P.T; ++k) {
    int acc = members[k][0];
    for (size_t m = 1; m < members[k].size(); ++m) {
      steps_out[2 * next_step] = acc;
      steps_out[2 * next_step + 1] = members[k][m];
      acc = NT + next_step;
      ++next_step;
    }
    leaf_id[k] = acc;
  }
  if (P.T == 1) {
    if (log2_macs_out) *log2_macs_out = 0;
    if (width_out) *width_out = (int)P.leaf[0].size();
    return TQEC_OK;
  }
  std::mt19937_64 rng(o.seed ? o.seed : 1);
  Tree best;
  double bestE = 1e300;
  const int trials = std::max(1, o.trials);
  const int target = o.target_width > 0 ? o.target_width : 64;
  for (int tr = 0; tr < trials; ++tr) {
    Tree t;
    const double temp = tr == 0 ? 0.0 : std::ldexp(1.0, tr % 8);
    greedy(P, rng, temp, &t);
    double E = energy(tree_macs(P, t), tree_width(t, P.T), target, o.width_penalty);
    if (E < bestE) { bestE = E; best = t; }
  }
  if (o.sweeps > 0) {
    Tree t = best;
    anneal(P, &t, rng, o.sweeps, target, o.width_penalty);
    double E = energy(tree_macs(P, t), tree_width(t, P.T), target, o.width_penalty);
    if (E < bestE) { bestE = E; best = t; }
  }
  emit(best, P.T, leaf_id, next_step, NT, steps_out);
  if (log2_macs_out) {  // the multiply-adds themselves, whatever the discount
    double m = 0;
    for (int i = P.T; i < (int)best.l.size(); ++i) m += std::ldexp(1.0, best.uni[i]);
    *log2_macs_out = std::log2(m);
  }
  if (width_out) *width_out = tree_width(best, P.T);
  return TQEC_OK;
}
