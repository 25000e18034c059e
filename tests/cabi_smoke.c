/* A C caller of the decoder's C ABI (include/tqec_gb300.h), built and run by
 * tests/test_cabi_c.py with a plain C compiler: the header must be valid C99
 * and the library usable without C++ or Python.  No GPU is needed: it plans a
 * small network (the order search, the planner's view of the program, and
 * the error paths); creating a program reports a CUDA error without a GPU and
 * succeeds with one.
 *
 * The network: a distance-3 repetition code under bit flips, as
 * compile(::TNMMAP, ...) builds it (tndecoder.jl:97-139 restricted to one
 * error type): bits 1..3, checks (1,2) and (2,3) with syndrome labels 4 and
 * 5, a logical parity over bit 1 with output label 6, priors [1-p, p] per
 * bit, one-hot syndrome leaves. */
#include <stdio.h>
#include <string.h>

#include "tqec_gb300.h"

static const double P = 0.1;

int main(void) {
  /* tensors: check(1,2,4) check(2,3,5) logical(1,6) prior1 prior2 prior3 leaf4 leaf5 */
  int32_t ix_offsets[9] = {0, 3, 6, 8, 9, 10, 11, 12, 13};
  int32_t ix_labels[13] = {1, 2, 4, 2, 3, 5, 1, 6, 1, 2, 3, 4, 5};
  int64_t data_offsets[9] = {0, 8, 16, 20, 22, 24, 26, 28, 30};
  double data[30];
  int32_t out_labels[1] = {6};
  int32_t syndrome_tensors[2] = {6, 7};
  tqec_network net;
  tqec_order_options oo;
  tqec_tree tree;
  tqec_plan_view view;
  tqec_options opts;
  tqec_program* prog = NULL;
  int32_t steps[14];
  double log2_macs = 0.0;
  int32_t width = 0;
  void* handle = NULL;
  char msg[256];
  int i, rc;

  for (i = 0; i < 8; ++i) { /* rank-3 parity tensors: 1 where the index bits have even parity */
    int par = (i & 1) ^ ((i >> 1) & 1) ^ ((i >> 2) & 1);
    data[i] = par ? 0.0 : 1.0;
    data[8 + i] = data[i];
  }
  data[16] = 1.0; data[17] = 0.0; data[18] = 0.0; data[19] = 1.0; /* logical: label 6 = bit 1 */
  for (i = 0; i < 3; ++i) {
    data[20 + 2 * i] = 1.0 - P;
    data[21 + 2 * i] = P;
  }
  data[26] = 1.0; data[27] = 0.0; data[28] = 1.0; data[29] = 0.0;

  net.n_tensors = 8;
  net.ix_offsets = ix_offsets;
  net.ix_labels = ix_labels;
  net.data_offsets = data_offsets;
  net.data = data;
  net.n_out = 1;
  net.out_labels = out_labels;
  net.n_syndrome = 2;
  net.syndrome_tensors = syndrome_tensors;

  memset(&oo, 0, sizeof(oo));
  oo.trials = 4;
  oo.sweeps = 20;
  oo.width_penalty = 1.0;
  oo.seed = 1;
  rc = tqec_optimize_order(&net, &oo, steps, &log2_macs, &width);
  if (rc != TQEC_OK) {
    tqec_last_error(msg, sizeof(msg));
    printf("order search failed: %d %s\n", rc, msg);
    return 1;
  }
  tree.n_steps = 7;
  tree.steps = steps;
  rc = tqec_plan_inspect(&net, &tree, &view, &handle);
  if (rc != TQEC_OK) {
    tqec_last_error(msg, sizeof(msg));
    printf("plan failed: %d %s\n", rc, msg);
    return 1;
  }
  printf("plan steps=%d classes=%d syndrome=%d arena=%lld width=%d\n", view.n_steps, view.n_classes,
         view.n_syndrome, (long long)view.arena_elems, view.width);
  if (view.n_classes != 2 || view.n_syndrome != 2) return 1;
  tqec_plan_release(handle);

  /* a tree that reuses a node is rejected with a status and a message */
  steps[2] = steps[0];
  steps[3] = steps[1];
  rc = tqec_plan_inspect(&net, &tree, &view, &handle);
  tqec_last_error(msg, sizeof(msg));
  printf("bad tree: %d %s\n", rc, msg);
  if (rc != TQEC_ERR_INVALID || strlen(msg) == 0) return 1;

  /* a program: TQEC_ERR_CUDA without a GPU, TQEC_OK with one */
  rc = tqec_optimize_order(&net, &oo, steps, &log2_macs, &width);
  memset(&opts, 0, sizeof(opts));
  opts.precision = TQEC_F64;
  opts.margin = -1.0;
  rc = tqec_program_create(&net, &tree, &opts, &prog);
  printf("create: %d\n", rc);
  if (rc == TQEC_OK) {
    tqec_program_destroy(prog);
  } else if (rc != TQEC_ERR_CUDA) {
    return 1;
  }
  printf("%s\n", tqec_version());
  return 0;
}
