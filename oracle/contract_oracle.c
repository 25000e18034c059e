/*
 * contract_oracle.c -- CPU oracle and CPU baseline for the TNMMAP path
 * (test infrastructure only; never linked into the product).
 *
 * Restates what TensorQEC does per syndrome in decode(ct, syndrome)
 * (src/decoding/tndecoder.jl:148-165, :240-253): write the one-hot syndrome
 * leaves, then evaluate every binary step of the contraction tree in float64
 * (OMEinsum's NestedEinsum evaluation, tndecoder.jl:162), then findmax.
 * Nothing is folded across syndromes, as in the reference.  Syndromes are
 * spread over OpenMP threads.
 *
 * Network and tree use the tqec_network / tqec_tree conventions: tensor data
 * in Julia column-major order (index bit j <-> the tensor's j-th label),
 * node n_tensors + s is the result of step s.
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  int a, b;            /* operand node ids */
  int nu;              /* union size */
  int nc;              /* kept labels */
  int64_t *sa, *sb, *sc; /* per-union-label strides into a, b, c */
  int64_t c_off;       /* offset of the output in the per-thread buffer */
} ostep;

typedef struct {
  int T, S, n_out, n_syn, syn_bytes;
  int64_t *off;        /* per node: offset into the per-thread buffer (leaves too) */
  int64_t *size;       /* per node: elements */
  int *syn_leaf;       /* per syndrome bit: leaf tensor */
  double *leaf_data;   /* template buffer holding the leaves */
  int64_t buf_elems;
  ostep *steps;
  int *root_perm;      /* root element -> Julia linear index of iy */
} oracle_prog;

static int find(const int *v, int n, int x) {
  for (int i = 0; i < n; ++i)
    if (v[i] == x) return i;
  return -1;
}

oracle_prog *oracle_create(int T, const int32_t *ix_off, const int32_t *labels, const int64_t *d_off,
                           const double *data, int n_out, const int32_t *out_labels, int n_syn,
                           const int32_t *syn_pos, int n_steps, const int32_t *steps) {
  if (n_steps != T - 1) return NULL;
  oracle_prog *p = (oracle_prog *)calloc(1, sizeof(oracle_prog));
  p->T = T;
  p->S = n_steps;
  p->n_out = n_out;
  p->n_syn = n_syn;
  p->syn_bytes = (n_syn + 7) / 8;
  int N = T + n_steps;
  int **lab = (int **)calloc(N, sizeof(int *));
  int *nl = (int *)calloc(N, sizeof(int));
  p->off = (int64_t *)calloc(N, sizeof(int64_t));
  p->size = (int64_t *)calloc(N, sizeof(int64_t));
  /* label multiplicities over the leaves + output */
  int maxlab = 0;
  for (int i = 0; i < ix_off[T]; ++i)
    if (labels[i] > maxlab) maxlab = labels[i];
  for (int i = 0; i < n_out; ++i)
    if (out_labels[i] > maxlab) maxlab = out_labels[i];
  int *cnt = (int *)calloc(maxlab + 1, sizeof(int));
  for (int i = 0; i < ix_off[T]; ++i) cnt[labels[i]]++;
  for (int i = 0; i < n_out; ++i) cnt[out_labels[i]]++;
  int64_t pos = 0;
  for (int i = 0; i < T; ++i) {
    nl[i] = ix_off[i + 1] - ix_off[i];
    lab[i] = (int *)malloc(sizeof(int) * (nl[i] + 1));
    memcpy(lab[i], labels + ix_off[i], sizeof(int) * nl[i]);
    p->size[i] = d_off[i + 1] - d_off[i];
    p->off[i] = pos;
    pos += p->size[i];
  }
  p->steps = (ostep *)calloc(n_steps, sizeof(ostep));
  for (int s = 0; s < n_steps; ++s) {
    int a = steps[2 * s], b = steps[2 * s + 1];
    ostep *st = &p->steps[s];
    st->a = a;
    st->b = b;
    int u[128], nu = 0;
    for (int i = 0; i < nl[a]; ++i) u[nu++] = lab[a][i];
    for (int i = 0; i < nl[b]; ++i)
      if (find(u, nu, lab[b][i]) < 0) u[nu++] = lab[b][i];
    int me = T + s;
    lab[me] = (int *)malloc(sizeof(int) * (nu + 1));
    nl[me] = 0;
    for (int i = 0; i < nu; ++i) {
      int in_a = find(lab[a], nl[a], u[i]) >= 0, in_b = find(lab[b], nl[b], u[i]) >= 0;
      if (cnt[u[i]] - in_a - in_b > 0) lab[me][nl[me]++] = u[i];
    }
    for (int i = 0; i < nl[a]; ++i) cnt[lab[a][i]]--;
    for (int i = 0; i < nl[b]; ++i) cnt[lab[b][i]]--;
    for (int i = 0; i < nl[me]; ++i) cnt[lab[me][i]]++;
    st->nu = nu;
    st->nc = nl[me];
    st->sa = (int64_t *)calloc((size_t)(nu > 0 ? nu : 1), sizeof(int64_t));
    st->sb = (int64_t *)calloc((size_t)(nu > 0 ? nu : 1), sizeof(int64_t));
    st->sc = (int64_t *)calloc((size_t)(nu > 0 ? nu : 1), sizeof(int64_t));
    for (int i = 0; i < nu; ++i) {
      int ja = find(lab[a], nl[a], u[i]), jb = find(lab[b], nl[b], u[i]), jc = find(lab[me], nl[me], u[i]);
      st->sa[i] = ja >= 0 ? ((int64_t)1 << ja) : 0;
      st->sb[i] = jb >= 0 ? ((int64_t)1 << jb) : 0;
      st->sc[i] = jc >= 0 ? ((int64_t)1 << jc) : 0;
    }
    p->size[me] = (int64_t)1 << nl[me];
    p->off[me] = pos;
    st->c_off = pos;
    pos += p->size[me];
  }
  p->buf_elems = pos;
  p->leaf_data = (double *)malloc(sizeof(double) * (size_t)p->off[T - 1] + sizeof(double) * p->size[T - 1]);
  for (int i = 0; i < T; ++i) memcpy(p->leaf_data + p->off[i], data + d_off[i], sizeof(double) * p->size[i]);
  p->syn_leaf = (int *)malloc(sizeof(int) * (n_syn + 1));
  for (int j = 0; j < n_syn; ++j) p->syn_leaf[j] = syn_pos[j];
  /* root labels -> position in out_labels */
  int root = T + n_steps - 1;
  if (T == 1) root = 0;
  p->root_perm = (int *)malloc(sizeof(int) * ((size_t)1 << n_out));
  for (int64_t e = 0; e < ((int64_t)1 << n_out); ++e) {
    int64_t j = 0;
    for (int q = 0; q < nl[root]; ++q)
      if ((e >> q) & 1) j |= (int64_t)1 << find(out_labels, n_out, lab[root][q]);
    p->root_perm[e] = (int)j;
  }
  for (int i = 0; i < N; ++i) free(lab[i]);
  free(lab);
  free(nl);
  free(cnt);
  return p;
}

static void contract_one(const oracle_prog *p, const uint8_t *row, double *buf, double *out) {
  int64_t leaf_elems = p->off[p->T - 1] + p->size[p->T - 1];
  memcpy(buf, p->leaf_data, sizeof(double) * leaf_elems);
  for (int j = 0; j < p->n_syn; ++j) { /* update_syndrome!, tndecoder.jl:148-158 */
    int s = (row[j >> 3] >> (j & 7)) & 1;
    double *l = buf + p->off[p->syn_leaf[j]];
    l[0] = s ? 0.0 : 1.0;
    l[1] = s ? 1.0 : 0.0;
  }
  for (int s = 0; s < p->S; ++s) {
    const ostep *st = &p->steps[s];
    const double *A = buf + p->off[st->a];
    const double *B = buf + p->off[st->b];
    double *C = buf + st->c_off;
    memset(C, 0, sizeof(double) * ((size_t)1 << st->nc));
    const int64_t n = (int64_t)1 << st->nu;
    int64_t ia = 0, ib = 0, ic = 0;
    for (int64_t u = 0; u < n; ++u) {
      C[ic] += A[ia] * B[ib];
      /* next index in binary counting: clear trailing ones, set next bit */
      int64_t x = u;
      int q = 0;
      while (x & 1) {
        ia -= st->sa[q];
        ib -= st->sb[q];
        ic -= st->sc[q];
        x >>= 1;
        ++q;
      }
      if (q < st->nu) {
        ia += st->sa[q];
        ib += st->sb[q];
        ic += st->sc[q];
      }
    }
  }
  int root = p->T == 1 ? 0 : p->T + p->S - 1;
  const double *R = buf + p->off[root];
  for (int64_t e = 0; e < ((int64_t)1 << p->n_out); ++e) out[p->root_perm[e]] = R[e];
}

/* marg_out: n x 2^n_out float64 marginals in Julia linear order; cls_out
 * (optional): findmax's first maximum.  threads <= 0: all. */
int oracle_contract(const oracle_prog *p, const uint8_t *packed, int64_t n, double *marg_out, int32_t *cls_out,
                    int threads) {
  if (!p) return -1;
  if (threads > 0) omp_set_num_threads(threads);
  const int64_t C = (int64_t)1 << p->n_out;
#pragma omp parallel
  {
    double *buf = (double *)malloc(sizeof(double) * (size_t)p->buf_elems);
#pragma omp for schedule(dynamic, 16)
    for (int64_t r = 0; r < n; ++r) {
      double *o = marg_out + r * C;
      contract_one(p, packed + r * p->syn_bytes, buf, o);
      if (cls_out) {
        int best = 0;
        for (int64_t c = 1; c < C; ++c)
          if (o[c] > o[best]) best = (int)c;
        cls_out[r] = best;
      }
    }
    free(buf);
  }
  return 0;
}

int oracle_max_threads(void) { return omp_get_max_threads(); }

void oracle_destroy(oracle_prog *p) {
  if (!p) return;
  for (int s = 0; s < p->S; ++s) {
    free(p->steps[s].sa);
    free(p->steps[s].sb);
    free(p->steps[s].sc);
  }
  free(p->steps);
  free(p->off);
  free(p->size);
  free(p->syn_leaf);
  free(p->leaf_data);
  free(p->root_perm);
  free(p);
}
