/*
 * tqec_gb300.h -- C ABI of the GB300 tensor-network decoder for TensorQEC.jl.
 *
 * This library replaces the hot path of TensorQEC's TNMMAP decoder: the
 * contraction `ct.code(ct.tensors...)` of the syndrome-conditioned factor
 * graph followed by `findmax` (src/decoding/tndecoder.jl:160-165 and
 * :248-253 in the TensorQEC.jl project).  The caller hands over the same
 * network the reference builds in `compile` (tndecoder.jl:97-146,
 * :186-219) together with a contraction tree (the reference's OMEinsum
 * `optimize_code` result, tndecoder.jl:140-144), and then decodes whole
 * batches of syndromes on one GPU.
 *
 * Conventions
 *  - Every entry point returns an int status: 0 (TQEC_OK) or a negative
 *    TQEC_ERR_* code; `tqec_last_error` gives the message of the calling
 *    thread's last failure.  No C++ exception crosses this boundary.
 *  - Tensor data are float64 in Julia (column-major) order: for a tensor with
 *    labels (l_0, ..., l_{r-1}) the element with index bits (x_0, ..., x_{r-1})
 *    sits at offset sum_j x_j * 2^j.  All labels have dimension 2, as in the
 *    reference (`uniformsize(code, 2)`).
 *  - Syndromes are bit-packed rows of ceil(n_syndrome/8) bytes, bit j of a
 *    row at byte j/8, bit j%8 (least significant first).  Bit j drives the
 *    j-th syndrome leaf, i.e. the order of `update_syndrome!`
 *    (tndecoder.jl:148-158: all X-check bits, then all Z-check bits).
 *  - Pointers passed to the decode calls may be host or device memory; the
 *    library detects which.  With stream == NULL a call is synchronous.
 *  - Calls on one program are serialised by an internal mutex, like the
 *    reference's compiled decoder, which mutates its tensors per call
 *    (tndecoder.jl:148-158).  Distinct programs are independent.
 */
#ifndef TQEC_GB300_H
#define TQEC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TQEC_OK 0
#define TQEC_ERR_INVALID (-1)     /* bad argument, shape or tree */
#define TQEC_ERR_CUDA (-2)        /* CUDA runtime failure */
#define TQEC_ERR_OOM (-3)         /* device allocation failed */
#define TQEC_ERR_UNSUPPORTED (-4) /* network outside what the kernels support */
#define TQEC_ERR_TIMEOUT (-5)     /* a bounded device wait gave up */
#define TQEC_ERR_IO (-6)          /* file could not be read or written */

/* Arithmetic of a contraction. */
#define TQEC_F64 0 /* float64 throughout (the reference's arithmetic) */
#define TQEC_F32 1 /* float32 with per-tensor power-of-two renormalisation */
/* double-float: each value a pair of float32 (hi + lo, about 48 significant
 * bits), renormalised like TQEC_F32, on the float32 pipes (GB300 runs float64
 * at 1/64 of the float32 rate).  The default arithmetic of the recheck;
 * accepted by tqec_contract_batch. */
#define TQEC_F32X2 2
/* A numerical study of bfloat16 intermediates, for tqec_contract_batch only:
 * the TQEC_F32 program with every stored intermediate rounded to bfloat16's
 * 8 significant bits (kept in float32 words, so no speed is gained).  Its
 * relative error bound is the float32 one plus 2^-9 per runtime step. */
#define TQEC_F32_BF16 3

/* Option flags. */
#define TQEC_FLAG_PLAIN 1u   /* decode one syndrome per kernel launch (drop-in form) */
#define TQEC_FLAG_NORECHECK 2u /* TQEC_F32: skip the recheck of low margins */
#define TQEC_FLAG_MAP 4u      /* most probable configuration (TNMAP): the network's
                                 out_labels name the variables whose values are
                                 reported; the contraction maximises over all */
/* launch shape: keep each syndrome's small intermediates (at most
 * tqec_options.big_elems elements) in shared memory and its large ones in global memory; only for
 * programs that have both kinds (others keep their default shape) */
#define TQEC_FLAG_SPLIT_ARENA 8u
/* TQEC_F32: run GEMM-shaped steps on the SIMT path instead of the tcgen05
 * tensor cores (same results within the same error bound) */
#define TQEC_FLAG_NO_TENSOR_CORES 16u
/* TQEC_F32: recheck low margins in float64 instead of TQEC_F32X2 */
#define TQEC_FLAG_RECHECK_F64 32u
/* launch shape: in blocks of one syndrome, 2-8 lanes share each four-output
 * work item of a step that would leave threads idle, each summing a run of
 * the contracted range (tqec_program_autotune also tries this) */
#define TQEC_FLAG_SHARED_ITEMS 64u

/* The factor graph, as built by compile(::TNMMAP, ...) (tndecoder.jl:97-146
 * for CSS codes, :186-219 for detector error models). */
typedef struct {
  int32_t n_tensors;
  const int32_t* ix_offsets;   /* n_tensors + 1 offsets into ix_labels */
  const int32_t* ix_labels;    /* positive variable labels (the reference's ixs) */
  const int64_t* data_offsets; /* n_tensors + 1 offsets into data */
  const double* data;          /* tensor entries, Julia order (see above) */
  int32_t n_out;
  const int32_t* out_labels;   /* the reference's iy */
  int32_t n_syndrome;
  const int32_t* syndrome_tensors; /* 0-based tensor positions of the one-hot
                                      syndrome leaves, in syndrome-bit order */
} tqec_network;

/* A binary contraction tree: step s merges nodes steps[2s] and steps[2s+1];
 * node ids < n_tensors are the network's tensors, node n_tensors + s is the
 * result of step s.  The last step is the root and every node is used once
 * (the flattened form of OMEinsum's NestedEinsum). */
typedef struct {
  int32_t n_steps;
  const int32_t* steps;
} tqec_tree;

typedef struct {
  int32_t precision;      /* TQEC_F64 or TQEC_F32 */
  uint32_t flags;         /* TQEC_FLAG_* */
  int32_t device;         /* CUDA device ordinal */
  int32_t group;          /* syndromes per thread block (power of two); 0 = auto */
  int32_t threads;        /* threads per block (rounded down to a power of two, >= 32); 0 = auto */
  double margin;          /* TQEC_F32: recheck when the log-probability margin
                             of the top class is below this; < 0 = the
                             rounding-error bound the planner derives */
  int32_t big_elems;      /* intermediates above this many elements go to the
                             big pool (global memory in split layouts); 0 = 1024 */
  int32_t reserved;
} tqec_options;

typedef struct {
  int32_t n_syndrome;        /* syndrome bits per row */
  int32_t syndrome_bytes;    /* bytes per packed row */
  int32_t n_classes;         /* 2^n_out entries of the marginal */
  int32_t n_steps;           /* runtime steps left after constant folding */
  int32_t n_tree_steps;      /* steps of the tree as given */
  int32_t width;             /* log2 of the largest runtime intermediate */
  int64_t arena_elems;       /* per-syndrome working set, elements */
  double flops_per_syndrome; /* 2 x multiply-adds of the runtime steps */
  double flops_tree;         /* 2 x multiply-adds of the whole tree as given */
  double err_bound_f32;      /* relative error bound of a TQEC_F32 marginal */
  double err_bound_f64;      /* relative error bound of a TQEC_F64 marginal */
  int32_t group_f32, threads_f32, smem_f32; /* launch shape chosen for F32 */
  int32_t group_f64, threads_f64, smem_f64; /* launch shape chosen for F64 */
  int32_t resident_f32, resident_f64;       /* most blocks in flight on the device */
  int32_t tables_smem_f32, tables_smem_f64; /* 1: tables staged in shared memory */
  int64_t arena_small;       /* elements of the small-tensor pool (0: one pool) */
  int32_t split_f32, split_f64;             /* 1: small pool in shared, big pool in global memory */
  int32_t tensor_steps;      /* GEMM-shaped steps (tcgen05 tf32 in float32 launches) */
  int32_t tensor_f32;        /* 1: the float32 shape runs them on the tensor cores */
  int32_t recheck_precision; /* TQEC_F32X2 or TQEC_F64: arithmetic of the recheck */
  int32_t cluster_blocks;    /* blocks of the thread-block cluster that contracts one
                                syndrome in single-syndrome launches (the recheck; all
                                launches of a TQEC_FLAG_PLAIN program); 0: one block */
  double err_bound_f32x2;    /* relative error bound of a TQEC_F32X2 marginal */
  int32_t shared_items_f32, shared_items_f64; /* 1: lanes share the work items of steps
                                                 that leave threads idle (TQEC_FLAG_SHARED_ITEMS) */
  int32_t cluster_tuned_steps; /* steps whose cluster-form plan tqec_program_autotune changed
                                  (barrier group on the first block or not, shared items) */
  int32_t info_pad;
} tqec_program_info_t;

typedef struct tqec_program tqec_program;

/* compile(::TNMMAP, problem) -> CompiledTNMMAP (tndecoder.jl:97-146,
 * :186-219).  Host data are copied; the program owns its device memory. */
int tqec_program_create(const tqec_network* net, const tqec_tree* tree,
                        const tqec_options* opts, tqec_program** out);

int tqec_program_destroy(tqec_program* prog);

int tqec_program_info(const tqec_program* prog, tqec_program_info_t* info);

/* decode(ct, syndrome) over a batch (tndecoder.jl:160-165, :248-253):
 * contracts every syndrome, writes the argmax class (findmax's first maximum
 * in Julia linear order), the natural-log marginal of every class
 * (n x n_classes, Julia linear order of `mar`) and a per-syndrome relative
 * error bound.  logp_out and err_bound_out may be NULL.  With TQEC_F32 the
 * syndromes whose class margin is below the bound are contracted again
 * (TQEC_F32X2, or float64 with TQEC_FLAG_RECHECK_F64) before the call
 * returns; their err_bound_out is that arithmetic's bound.  A syndrome that
 * no error produces (an all-zero marginal, where the reference's
 * error_pattern integer program fails) is reported per row rather than by
 * failing the batch: class 0 and every log-marginal -inf. */
int tqec_decode_batch(tqec_program* prog, const uint8_t* syndromes, int64_t n,
                      int32_t* class_out, double* logp_out,
                      float* err_bound_out, void* stream);

/* decode over the rows rows[0 .. *n_rows) of a syndrome array, with the row
 * list and its length in device memory (no reference counterpart: it lets a
 * filter that runs on the device, such as the surrogate's confidence gate,
 * hand its rejected rows to the contraction without a host round trip).
 * class_out[rows[r]] receives row rows[r]'s class, with the float32 recheck
 * as in tqec_decode_batch; other entries are untouched.  Device pointers
 * only; n_max bounds *n_rows; n_hint (the expected row count, e.g. the
 * previous call's) picks the tuned launch shape.  Stream-ordered: returns
 * without waiting and performs no host synchronisation (stream == NULL: the
 * program's own stream).  Not for TQEC_FLAG_PLAIN or TQEC_FLAG_MAP
 * programs. */
int tqec_decode_rows(tqec_program* prog, const uint8_t* syndromes,
                     const int32_t* rows, const int32_t* n_rows, int64_t n_max,
                     int64_t n_hint, int32_t* class_out, void* stream);

/* The contraction alone in a chosen precision, without argmax or recheck:
 * writes n x n_classes natural-log marginals (the reference's
 * `ct.code(ct.tensors...)`, tndecoder.jl:162, in log form). */
int tqec_contract_batch(tqec_program* prog, const uint8_t* syndromes,
                        int64_t n, int32_t precision, double* logp_out,
                        void* stream);

/* decode(ct::CompiledTNMAP, syndrome) over a batch (tndecoder.jl:53-57,
 * TensorInference's most_probable_config): for a program created with
 * TQEC_FLAG_MAP, the values of the reported variables in the most probable
 * configuration consistent with each syndrome (bit-packed rows of
 * ceil(n_out/8) bytes in out_labels order; ties go to the configuration
 * whose maximised labels read smallest as binary numbers, step by step) and
 * the natural log of its probability (n doubles, may be NULL). */
int tqec_map_decode_batch(tqec_program* prog, const uint8_t* syndromes, int64_t n,
                          uint8_t* assignment_out, double* logp_out, void* stream);

/* Count of syndromes the last TQEC_F32 decode call sent to the
 * recheck (a measure of how often the rounding bound was not enough).  After
 * a call that returned before its work ended (a stream given, device
 * outputs), synchronise that stream before asking. */
int tqec_last_recheck_count(const tqec_program* prog, int64_t* count);

/* The form of single-syndrome launches in `precision` (TQEC_F64: the plain
 * form's; TQEC_F32X2 or TQEC_F64: the recheck's): blocks = 0 gives each
 * syndrome one block, blocks = 2, 4, 8 or 16 a thread-block cluster of that
 * many blocks of `threads` threads that share each step's work.
 * small_in_smem = 1 keeps the small intermediates in the first block's
 * shared memory (the others reach them through distributed shared memory),
 * 0 keeps every intermediate in global memory, -1 takes the first where it
 * fits.  Wide programs start with 16 blocks of 128 threads (8 of 256 where
 * 16-block clusters cannot launch); tqec_program_autotune measures the forms
 * and placements.  No reference counterpart (a latency setting). */
int tqec_program_set_cluster(tqec_program* prog, int32_t precision, int32_t blocks, int32_t threads,
                             int32_t small_in_smem);

/* Waits for the program's stream and frees its cached intermediate arenas
 * (the next launch allocates them again).  A program of a wide network
 * holds up to 16 GB of them; the 2^k programs of a sliced contraction run
 * one after another and release theirs in turn.  No reference counterpart. */
int tqec_program_trim(tqec_program* prog);

/* Tries the launch shapes that fit and keeps the fastest for each
 * precision, timing n_probe synthetic syndromes. */
int tqec_program_autotune(tqec_program* prog, int64_t n_probe);

/* Program files.  No direct counterpart in the reference (a compiled Julia
 * decoder is serialised whole); they keep compile's contraction-order search
 * (optimize_code, tndecoder.jl:140-144) and the autotuning out of a new
 * process's start-up.  tqec_program_save writes what the program was compiled
 * from (network, tree, options) and its current launch shapes to `path`
 * (written to path.tmp, then renamed).  tqec_program_load compiles the stored
 * network with the stored tree on `device` (< 0: the stored device), fails
 * with TQEC_ERR_IO when the file cannot be read (or written, on save), with
 * TQEC_ERR_INVALID on a malformed or corrupted file (checksummed) or when
 * the network no longer compiles to the same program, and takes the stored
 * launch shapes when the device has the same SM count and shared-memory limit
 * (otherwise the shapes creation picks; autotune again).  Files use the
 * writer's byte order. */
int tqec_program_save(tqec_program* prog, const char* path);
int tqec_program_load(const char* path, int32_t device, tqec_program** out);

/* The compiled program without a device, for inspection (the counterpart of
 * OMEinsum.contraction_complexity(ct), tndecoder.jl:273-279).  `steps` holds
 * n_steps records of 64 bytes: int32 a_kind, b_kind, a_ref, b_ref, a_prod,
 * b_prod; int8 a_sel[4], b_sel[4]; int32 lh, lfa, lfb, lk, out_off,
 * perm_off, sync_after (1 = block barrier after the step), pad.  Release the
 * view with tqec_plan_release. */
typedef struct {
  int32_t n_steps;
  const void* steps;
  int64_t n_perm;
  const int32_t* perm;
  int64_t n_consts;
  const double* consts;
  int64_t arena_elems;
  int32_t width;
  int32_t n_classes;
  int32_t n_syndrome;
  double flops_per_syndrome;
  double flops_tree;
  double err_terms;
  /* TQEC_FLAG_MAP programs: per-step variable ids (fb, fa, h, k bits; the
   * step record's last field is its offset here), reported variables, and
   * per-variable values fixed on the host (-1 = decided by the search) */
  int32_t map_mode;
  int32_t n_vars;
  int64_t n_vartab;
  const int32_t* vartab;
  int32_t n_report;
  const int32_t* report;
  const int8_t* fixed;
} tqec_plan_view;

int tqec_plan_inspect(const tqec_network* net, const tqec_tree* tree,
                      tqec_plan_view* view, void** handle);
/* The same for a program compiled with option flags (TQEC_FLAG_MAP). */
int tqec_plan_inspect_flags(const tqec_network* net, const tqec_tree* tree, uint32_t flags,
                            tqec_plan_view* view, void** handle);
int tqec_plan_release(void* handle);

/* Contraction-order search, in place of OMEinsum's
 * optimize_code(code, uniformsize(code, 2), TreeSA()) (tndecoder.jl:140-144,
 * :213-217): randomised greedy passes refined by simulated annealing over
 * tree rotations.  Only the network's labels and outputs are read.  Writes
 * 2 * (n_tensors - 1) node ids in the tqec_tree convention, log2 of the
 * tree's multiply-adds and the width of its widest intermediate. */
typedef struct {
  int32_t trials;        /* randomised greedy passes (default 32) */
  int32_t sweeps;        /* annealing sweeps (default 60; 0 = none) */
  int32_t target_width;  /* widths above this are penalised (0 = none) */
  double width_penalty;  /* energy per label above target_width (default 1) */
  uint64_t seed;         /* random seed (0 = 1) */
  double tensor_discount; /* > 1: the multiply-adds of GEMM-shaped steps (>= 2^7 x 2^5
                             outputs per batch index, >= 2^5 contracted, the planner's
                             tensor-core criterion) count this many times less, steering
                             the search toward tensor-core steps (0 or 1: off) */
} tqec_order_options;

int tqec_optimize_order(const tqec_network* net, const tqec_order_options* opts,
                        int32_t* steps_out, double* log2_macs_out,
                        int32_t* width_out);

/* ---- error patterns: error_pattern(pos, ct, syndrome), tndecoder.jl:167-174
 * A syndrome-consistent (ex, ez) of the decoded class for every row, in place
 * of the reference's integer program (ipdecoder.jl:150-169): ex = rz * sz and
 * ez = rx * sx with precomputed GF(2) right inverses (0/1 bytes, row-major
 * nq x n_sz and nq x n_sx), then the reference's fix-up with lx, lz (k x nq).
 * chk_* rows (each over n_s* bits) must all have even overlap with the
 * syndrome half for it to be reachable; ok_out gets 0 for rows that are not.
 * Outputs are bit-packed rows of ceil(nq/8) bytes; host or device memory. */
typedef struct tqec_patterns tqec_patterns;

int tqec_patterns_create(int32_t nq, int32_t n_sx, int32_t n_sz, int32_t k,
                         const uint8_t* rx, const uint8_t* rz, int32_t n_chk_x,
                         const uint8_t* chk_x, int32_t n_chk_z, const uint8_t* chk_z,
                         const uint8_t* lx, const uint8_t* lz, int32_t device,
                         tqec_patterns** out);
int tqec_patterns_destroy(tqec_patterns* p);
int tqec_patterns_decode(tqec_patterns* p, const uint8_t* syndromes, const int32_t* classes,
                         int64_t n, uint8_t* ex_out, uint8_t* ez_out, uint8_t* ok_out,
                         void* stream);

/* ---- learned surrogate (no counterpart in the reference) -----------------
 * A ReLU MLP over the syndrome bits proposes the logical class with a
 * softmax confidence; tqec_gated_decode sends the rows below a confidence
 * threshold to the exact contraction of a program.  Parameters are float32
 * masters (bf16 copies feed the GEMMs, which accumulate in float32); layer l
 * stores W[dout][din] row-major then b[dout], padded to 8 floats, where din
 * of layer 0 is n_in rounded up to 64 (extra columns are zero). */
typedef struct {
  int32_t n_in;      /* syndrome bits */
  int32_t hidden;    /* units per hidden layer (multiple of 32) */
  int32_t n_layers;  /* linear layers (>= 2) */
  int32_t n_out;     /* classes */
  uint64_t seed;     /* initialisation seed */
  int32_t device;
} tqec_mlp_config;

typedef struct tqec_mlp tqec_mlp;

int tqec_mlp_create(const tqec_mlp_config* cfg, tqec_mlp** out);
int tqec_mlp_destroy(tqec_mlp* mlp);
int tqec_mlp_param_count(const tqec_mlp* mlp, int64_t* n);
int tqec_mlp_get_params(tqec_mlp* mlp, float* out, int64_t n);
int tqec_mlp_set_params(tqec_mlp* mlp, const float* in, int64_t n);
/* Gradients of the mean soft-target cross-entropy (targets: n x n_out
 * class probabilities) without updating the parameters. */
int tqec_mlp_gradients(tqec_mlp* mlp, const uint8_t* syndromes, const float* targets, int64_t n,
                       float* grads_out, float* loss_out);
/* One Adam step (beta 0.9/0.999, eps 1e-8) on a batch; loss_out may be NULL. */
int tqec_mlp_train_step(tqec_mlp* mlp, const uint8_t* syndromes, const float* targets, int64_t n,
                        float lr, float* loss_out, void* stream);
/* The same step on rows[0..n) of a training set resident in device memory
 * (n_set packed syndromes and their n_set x n_classes targets): the batch is
 * gathered on the device, and nothing is copied to or from the host unless
 * loss_out is given (then the call synchronises, and reports a row index
 * outside [0, n_set) as TQEC_ERR_INVALID; such a row reads row 0). */
int tqec_mlp_train_step_rows(tqec_mlp* mlp, const uint8_t* syndromes, const float* targets, int64_t n_set,
                             const int32_t* rows, int64_t n, float lr, float* loss_out, void* stream);
/* Argmax class and its softmax probability for each row. */
int tqec_mlp_infer(tqec_mlp* mlp, const uint8_t* syndromes, int64_t n, int32_t* class_out,
                   float* conf_out, void* stream);
/* Surrogate first; rows with confidence < threshold are decoded by `prog`
 * (tqec_decode_batch).  Writes the number of such rows. */
int tqec_gated_decode(tqec_mlp* mlp, tqec_program* prog, float threshold, const uint8_t* syndromes,
                      int64_t n, int32_t* class_out, int64_t* n_fallback_out, void* stream);

/* Rows the last tqec_gated_decode call sent to the exact contraction (the
 * gate's rejections).  A call given a stream and device buffers with
 * n_fallback_out == NULL returns without a host synchronisation; synchronise
 * its stream before asking. */
int tqec_gated_last_fallback(tqec_mlp* mlp, int64_t* n_fallback);
/* How the layers run.  0: SIMT GEMMs.  1, 2: tcgen05 GEMMs layer by layer
 * (hidden a multiple of 256), a 4-stage TMA ring with one block per SM or a
 * 2-stage ring with two blocks per SM.  3, the default: inference (infer,
 * gated decode, logits) by one persistent tcgen05 kernel for the whole
 * forward, activations kept in shared and tensor memory (4 layers, hidden
 * 512, at most 64 inputs and 16 outputs; otherwise as 2), training as 2. */
int tqec_mlp_set_gemm(tqec_mlp* mlp, int use_tensor_cores);
/* Raw output-layer logits (n x n_out float32, host or device memory). */
int tqec_mlp_forward_logits(tqec_mlp* mlp, const uint8_t* syndromes, int64_t n, float* logits_out);
/* Checkpoint: one JSON header line, then the float32 parameters. */
int tqec_mlp_save(tqec_mlp* mlp, const char* path);
int tqec_mlp_load(tqec_mlp* mlp, const char* path);

/* ---- seeded sampling and the Monte-Carlo loop (no counterpart in the
 * reference's decoder path; replaces the host loop of multi_round_qec,
 * threshold.jl:1-19, with check_logical_error, error_model.jl:179-181).
 * Per sample and qubit one Philox4x32-10 uniform picks the Pauli as
 * random_error_pattern does (error_model.jl:97-117); the syndrome is
 * [Hx ez ; Hz ex] bit-packed, the true class the Julia linear index of mar
 * for a = lx.ez, b = lz.ex.  hx/hz are 0/1 bytes (n_s* x nq), lx/lz (k x nq),
 * px/py/pz per qubit.  Sample i of seed s is the same for any batching. */
typedef struct tqec_sampler tqec_sampler;

int tqec_sampler_create(int32_t nq, int32_t n_sx, int32_t n_sz, const uint8_t* hx,
                        const uint8_t* hz, int32_t k, const uint8_t* lx, const uint8_t* lz,
                        const double* px, const double* py, const double* pz, int32_t device,
                        tqec_sampler** out);
int tqec_sampler_destroy(tqec_sampler* s);
/* Samples offset .. offset+n-1 of `seed`; host or device outputs. */
int tqec_sample(tqec_sampler* s, uint64_t seed, uint64_t offset, int64_t n,
                uint8_t* syndromes_out, int32_t* class_out, void* stream);
/* Samples n_total syndromes in batches on the device, decodes them with
 * `prog` (or the gated surrogate `mlp` in front of it when not NULL) and
 * counts decoded classes that differ from the true class (logical errors). */
int tqec_monte_carlo(tqec_sampler* s, tqec_program* prog, tqec_mlp* mlp, float threshold,
                     uint64_t seed, int64_t n_total, int64_t batch, int64_t* n_logical_errors,
                     int64_t* n_fallback);

/* Float64 batch decode that allocates no device memory (no counterpart in
 * the reference).  For callers that cannot allocate while they decode: a
 * real-time decoding loop that must not stall or fail on an allocation, or a
 * process whose device memory is already reserved in full by another
 * allocator.  Same results as tqec_decode_batch with TQEC_F64, whatever the
 * program's own precision; a TQEC_FLAG_MAP program is rejected with
 * TQEC_ERR_INVALID, as tqec_decode_batch rejects it.  All pointers must be
 * device memory of the program's device (host pointers and other GPUs'
 * buffers are rejected, since staging them would allocate); logp_out may be
 * NULL.  The only scratch is a 32 MiB array inside the library, which every
 * GPU that loads the library holds until the process exits; a program whose
 * float64 working set exceeds it (tqec_program_info: arena_elems * 8 bytes per
 * syndrome) is rejected with TQEC_ERR_UNSUPPORTED.  The first call on a device
 * looks up that array's device address on the current device and caches it
 * for the life of the process; make that first call before any stream
 * capture, and do not call this entry point on a device after a
 * cudaDeviceReset of it (the cached address belonged to the old context).  All calls share the one
 * array: calls whose kernels overlap on the GPU (concurrent streams, other
 * threads) race on it and must be serialised by the caller.  Every scratch
 * element a call reads it has written first, so nothing needs clearing.  With
 * stream == NULL the call runs on the default stream and returns when done. */
int tqec_decode_batch_noalloc(tqec_program* prog, const uint8_t* syndromes,
                              int64_t n, int32_t* class_out, double* logp_out,
                              void* stream);

/* Message of the calling thread's last failure (always NUL-terminated). */
int tqec_last_error(char* buf, size_t len);

/* Library version string, e.g. "tqec-gb300 0.1.0 sm_103a". */
const char* tqec_version(void);

/* ---- several programs in one persistent launch (uneven code sizes) ------
 * No reference counterpart (the reference decodes one syndrome of one code at
 * a time).  A batch is a set of rows of every program; decoding it is one
 * float32 persistent launch over all programs' row groups (largest programs
 * first), one recheck launch (TQEC_F32X2, or float64 when every program has
 * TQEC_FLAG_RECHECK_F64; programs must agree) over the rows whose margin is
 * inside the float32 bound, and a counter update, with no host synchronisation and no
 * allocation: one tqec_multi_launch can be captured into a CUDA graph and the
 * graph replayed once per batch.  The programs' own launch shapes are not
 * used; MAP programs are rejected. */
typedef struct tqec_multi tqec_multi;

int tqec_multi_create(tqec_program* const* progs, int32_t n_progs, tqec_multi** out);
int tqec_multi_destroy(tqec_multi* m);
/* batch_end_rows[b * n_progs + i]: end (exclusive) of batch b's rows of
 * program i, non-decreasing in b (batch 0 starts at row 0).  syndromes[i]:
 * device pointer to program i's bit-packed rows; class_out[i]: device int32
 * per row.  The buffers must stay valid while batches are decoded. */
int tqec_multi_set_work(tqec_multi* m, int32_t n_batches, const int64_t* batch_end_rows,
                        const uint8_t* const* syndromes, int32_t* const* class_out);
/* the next launch decodes batch 0 (stream-ordered) */
int tqec_multi_reset(tqec_multi* m, void* stream);
/* decodes the next batch on `stream`; past the last batch it does nothing */
int tqec_multi_launch(tqec_multi* m, void* stream);
/* per program: syndromes per block and whether its arena is in shared memory;
 * and the float32 grid */
int tqec_multi_info(const tqec_multi* m, int32_t* groups, int32_t* arena_in_smem, int32_t* grid);

#ifdef __cplusplus
}
#endif

#endif /* TQEC_GB300_H */
