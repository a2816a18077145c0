/*
 * qxgpu.h -- C ABI of the GB300 (sm_103a) executor for QXTools' contraction programmes.
 *
 * The reference has no FFI: its contraction hot path is Julia code that walks a plan of
 * pairwise contractions (`single_amplitude`, src/simulation.jl:86-91, which calls
 * QXTns.contract_tn!) or a `.qx` DSL programme built by `build_compute_graph`
 * (src/compute_graph/compute_graph.jl:15-98) and run by `QXContexts.execute`
 * (bin/qxrun.jl:83-87).  This header is the boundary that replaces both: a programme is the
 * `.qx` command list (docs/src/users_guide.md:93-165) with tensor symbols mapped to integer
 * ids, leaf data is the TensorCache table (src/compute_graph/tensor_cache.jl:6-111), and an
 * amplitude call takes an explicit list of output bitstrings (the `.yml` `List` method,
 * src/outputs.jl:63-68) and a range of slice ids (qxrun's `--number-slices`,
 * bin/qxrun.jl:36-39).
 *
 * Conventions
 *   - Every entry point returns QXG_OK (0) or a negative qxg_status; no exception crosses
 *     the ABI.  qxg_last_error() returns a thread-local message for the last failure.
 *   - Arrays are column-major (first index fastest), like Julia arrays; complex numbers are
 *     interleaved (re, im) doubles.
 *   - The caller owns every host array; the library copies what it keeps.  Device buffers
 *     belong to the programme handle.  One handle owns one CUDA stream and is not
 *     thread-safe; separate handles may be used from separate threads.
 */
#ifndef QXGPU_H
#define QXGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum qxg_status {
    QXG_OK = 0,
    QXG_ERR_INVALID = -1,      /* malformed programme, bad label, dimension mismatch, bad argument */
    QXG_ERR_CUDA = -2,         /* a CUDA runtime or driver call failed */
    QXG_ERR_OOM = -3,          /* the workspace does not fit in device memory or the set limit */
    QXG_ERR_UNSUPPORTED = -4,  /* valid input outside what the library supports */
    QXG_ERR_TIMEOUT = -5,      /* a bounded device-side wait gave up */
    QXG_ERR_STATE = -6         /* call made in the wrong order (e.g. data not set) */
} qxg_status;

/* One instruction per `.qx` command (docs/src/users_guide.md:93-165; node types built at
 * src/compute_graph/compute_graph.jl:25-35 (load/output), :39-58 (view), :61-90 (ncon),
 * :94 (save)).  Tensor symbols are mapped to dense ids 0..ntensors-1 by the caller. */
typedef enum qxg_opcode {
    QXG_OP_LOAD = 1,    /* dst = leaf data[a]                         ("load t1 data_2 2,2")  */
    QXG_OP_VIEW = 2,    /* dst = a[.., v_b, ..] at rank position pos  ("view t1_s t1 v1 1 2") */
    QXG_OP_OUTPUT = 3,  /* dst = basis vector of output qubit a       ("output t6 1 2")       */
    QXG_OP_NCON = 4,    /* dst = pairwise contraction of a and b      ("ncon I2 1 t1_s 1,2 t4 2") */
    QXG_OP_SAVE = 5     /* the programme's result is tensor a         ("save output t11")     */
} qxg_opcode;

typedef struct qxg_instr {
    int32_t op;        /* qxg_opcode */
    int32_t dst;       /* tensor id written (LOAD, VIEW, OUTPUT, NCON); unused for SAVE */
    int32_t a;         /* LOAD: data id; VIEW: source tensor; OUTPUT: qubit (0-based);
                          NCON: first operand; SAVE: saved tensor */
    int32_t b;         /* VIEW: slice variable id (0-based, `v1` -> 0); OUTPUT: dimension (2);
                          NCON: second operand */
    int32_t pos;       /* VIEW: rank position of the sliced index (0-based) */
    int32_t dim;       /* VIEW: bond dimension of the sliced index */
    int32_t nc;        /* NCON: number of labels of dst (0: scalar) */
    int32_t na;        /* NCON: number of labels of a (0: scalar, the DSL's `0`) */
    int32_t nb;        /* NCON: number of labels of b */
    int32_t label_off; /* NCON: offset into the labels array: nc labels of dst, then na of a,
                          then nb of b.  Labels are positive integers local to the command;
                          a label in a and b but not dst is summed, in a, b and dst batched. */
} qxg_instr;

typedef enum qxg_precision {
    QXG_PREC_FP64 = 0,        /* ComplexF64 storage and arithmetic (the plain executor) */
    QXG_PREC_SPLIT_BF16 = 1,  /* Complex64 storage, FP32 accumulation, 3xBF16 tensor-core products */
    QXG_PREC_SPLIT_TF32 = 2,  /* Complex64 storage, FP32 accumulation, 3xTF32 tensor-core products */
    QXG_PREC_FP32 = 3         /* Complex64 storage, FP32 CUDA-core arithmetic only */
} qxg_precision;

typedef struct qxg_options {
    int32_t precision;            /* qxg_precision */
    int32_t device;               /* CUDA device ordinal */
    int64_t workspace_limit;      /* max bytes of intermediate workspace; 0 = 3/4 of free memory */
    int32_t max_bitstring_batch;  /* bitstrings per pass through the programme; 0 = automatic */
    int32_t max_slice_batch;      /* slices per pass; 0 = automatic */
    int32_t use_graphs;           /* capture each pass in a CUDA graph (1) or launch eagerly (0) */
    int32_t tc_tuning;            /* tensor-core tile variants: 0 = time the candidates of each step
                                     the first time it runs and keep the fastest (default);
                                     k >= 1 = candidate k of every step (1: fused X gather, widest
                                     N tile; then narrower tiles, then the X-planes variants) */
    int32_t tc_plane_budget_mb;   /* packed planes of a tensor-core step's smaller operand beyond which
                                     its free columns are processed in blocks; 0 = 4096 MiB */
    int32_t tc_wait_limit;        /* polls before a tensor-core kernel's bounded wait gives up (0: 2^20).
                                     A wait that gives up ends the call with QXG_ERR_TIMEOUT; the waits
                                     for copies and MMAs already in flight keep the full limit */
    int32_t tc_stall_test;        /* test hook, leave 0: nonzero makes the first CTA of every
                                     tensor-core GEMM issue no operand copies, so its waits run out and
                                     the call returns QXG_ERR_TIMEOUT (exercises the timeout path) */
    int32_t cuda_core_joins;      /* 1: keep the final joins of split-TF32 programmes (32 x 8..32
                                     results per batch value, long sums) on the CUDA cores' batched
                                     small GEMM; 0 = the tensor-core join (default) */
    int32_t reserved[2];
} qxg_options;

typedef struct qxg_program qxg_program;

typedef struct qxg_program_info {
    int64_t num_slices;           /* product of the slice variables' dimensions */
    int64_t output_size;          /* elements of the saved tensor per bitstring (1 = amplitude) */
    int32_t num_qubits;
    int32_t num_steps;            /* ncon instructions */
    int32_t bitstring_batch;      /* chosen bitstrings per pass */
    int32_t slice_batch;          /* chosen slices per pass */
    int64_t workspace_bytes;      /* device workspace in use */
    double flops_per_amplitude;   /* algorithmic FLOPs (8 |C| K per ncon) for one bitstring,
                                     summed over all slices */
    double flops_executed_per_pass;  /* FLOPs one pass executes (shared sub-trees counted once) */
    double bytes_executed_per_pass;  /* algorithmic bytes one pass moves: s(|A|+|B|+|C|) per ncon */
    int32_t num_steps_invariant;  /* ncon steps computed once per call */
    int32_t num_steps_slice;      /* ncon steps computed once per slice batch */
    int32_t num_steps_bitstring;  /* ncon steps computed once per (slice batch, bitstring batch) */
    int32_t num_steps_tensor_core;  /* ncon steps run on the tensor cores (split modes) */
    int32_t num_steps_fused;      /* of those, steps whose GEMM gathers the larger operand itself */
    int32_t num_steps_tuned;      /* tensor-core steps whose variant was chosen by timing */
    int32_t reserved[2];
} qxg_program_info;

/* Build a programme from the `.qx` command list.  data_rank[i] and the concatenated
 * data_dims give the shape of leaf data i (the `load` dims; TensorCache keys `data_N`,
 * src/compute_graph/tensor_cache.jl:90-106).  Replaces parsing a `.qx` file into a
 * QXContexts ComputeGraph (bin/qxrun.jl:83 -> QXContexts.execute). */
int qxg_program_create(const qxg_instr* instrs, int32_t ninstr,
                       const int32_t* labels, int64_t nlabels,
                       const int32_t* data_rank, const int64_t* data_dims, int32_t ndata,
                       int32_t nqubits, const qxg_options* opts, qxg_program** out);

/* Copy leaf data `data_id` (column-major, interleaved complex, `nelem` complex values) to the
 * device.  Replaces loading `data_N` from the `.jld2` file (src/compute_graph/tensor_cache.jl:90-106). */
int qxg_program_set_data(qxg_program* prog, int32_t data_id, const double* re_im, int64_t nelem);

/* Amplitudes of `nbitstrings` bitstrings, summed over slices [slice_begin, slice_end).
 * bitstrings: nbitstrings * nqubits chars from {'0','1','+','-'}, character i is qubit i+1
 * (docs/src/basics.md:55-64).  out_re_im: nbitstrings * output_size complex values, each
 * bitstring's saved tensor in column-major order.  Host buffers; the call is synchronous.
 * Replaces `single_amplitude` (src/simulation.jl:86-91) called once per bitstring, and the
 * slice loop of QXContexts.execute (bin/qxrun.jl:83-87, `max_slices`). */
int qxg_amplitudes(qxg_program* prog, const char* bitstrings, int32_t nbitstrings,
                   int64_t slice_begin, int64_t slice_end, double* out_re_im);

/* As qxg_amplitudes, with device-resident bitstrings and result (d_out_re_im: FP64 complex),
 * enqueued on the programme's stream; returns without synchronising.  No counterpart in the
 * reference (its executor is host-driven); used when inputs already live in HBM. */
int qxg_amplitudes_device(qxg_program* prog, const char* d_bitstrings, int32_t nbitstrings,
                          int64_t slice_begin, int64_t slice_end, double* d_out_re_im);

/* Gradient of a real loss L(amplitudes) with respect to every leaf tensor, by reverse-mode
 * (adjoint) contraction through the same programme: for each `ncon` C = A.B the adjoints are
 * A_bar = ncon(C_bar, conj B) and B_bar = ncon(conj A, C_bar) (X_bar = dL/d conj X).  No
 * counterpart in the reference (its executor is forward only); this is the differentiable form
 * of `single_amplitude` / QXTns.contract_tn!.
 *   amp_bar: nbitstrings * output_size interleaved complex values dL/d conj(amplitude); NULL
 *            means L = sum |amplitude|^2 (then the slice range must fit one slice batch).
 *   out_re_im: the amplitudes (as qxg_amplitudes), or NULL.
 *   leaf_grads: dL/d conj(leaf) for every `load` command in programme order, each its data's
 *            elements in column-major order (interleaved complex doubles).
 * Each (slice batch, bitstring batch) pass recomputes the forward sub-trees it needs and runs its
 * backward steps; gradients are summed over passes in FP64.  Every command's result must be read
 * by at most one command (true of programmes built by build_compute_graph). */
int qxg_gradient(qxg_program* prog, const char* bitstrings, int32_t nbitstrings,
                 int64_t slice_begin, int64_t slice_end, const double* amp_bar,
                 double* out_re_im, double* leaf_grads);

/* Wait for work enqueued on the programme's stream. */
int qxg_program_synchronize(qxg_program* prog);

/* The programme's CUDA stream (a cudaStream_t), for callers that order their own work. */
void* qxg_program_stream(qxg_program* prog);

/* Sizes, chosen batches and FLOP counts of a created programme. */
int qxg_program_info_get(const qxg_program* prog, qxg_program_info* info);

/* Per-kernel timing of a programme: the reference times its executor with TimerOutputs
 * sections ("Simulation", bin/qxrun.jl:50-52 and the warm re-run at :89-96); here every
 * launch can be bracketed with CUDA events on the programme's own stream. */
typedef enum qxg_kernel_kind {
    QXG_KERNEL_CONTRACT_FP64 = 0,   /* CUDA-core contraction, ComplexF64 */
    QXG_KERNEL_CONTRACT_FP32 = 1,   /* CUDA-core contraction, Complex64 / FP32 */
    QXG_KERNEL_CONTRACT_TC = 2,     /* tensor-core (tcgen05) split-precision GEMM of a contraction */
    QXG_KERNEL_VIEW = 3,            /* slice-batch view materialisation */
    QXG_KERNEL_OUTPUT = 4,          /* bitstring-batch output vectors */
    QXG_KERNEL_REDUCE = 5,          /* FP64 sum over the slice batch */
    QXG_KERNEL_TC_PACK = 6,         /* gather + hi/lo split of both operands for the tensor cores */
    QXG_KERNEL_CONTRACT_BATCH = 7   /* several small independent CUDA-core contractions, one launch */
} qxg_kernel_kind;

typedef struct qxg_step_profile {
    int32_t instr;      /* instruction index of the command (-1: the slice reduction, -2: batches
                           of small contractions, QXG_KERNEL_CONTRACT_BATCH) */
    int32_t kernel;     /* qxg_kernel_kind */
    int64_t launches;
    double ms;          /* summed CUDA-event time of those launches */
    double flops;       /* algorithmic FLOPs (8 |C| K) summed over the launches */
    double bytes;       /* algorithmic bytes (s (|A|+|B|+|C|)) summed over the launches */
} qxg_step_profile;

/* enable = 1: record CUDA events around every launch from now on (clears earlier records);
 * enable = 0: stop recording.  No counterpart in the reference beyond its timers. */
int qxg_program_profile(qxg_program* prog, int32_t enable);

/* Synchronise and aggregate the records per command: up to max_entries entries are written to
 * out, *n_entries receives their count, *kernel_launches the number of kernels this programme
 * launched since it was created (counted whether or not profiling is on). */
int qxg_program_profile_read(qxg_program* prog, qxg_step_profile* out, int32_t max_entries,
                             int32_t* n_entries, int64_t* kernel_launches);

/* Describe, as one line of text, how the current forward plan executes command `instr`: the
 * kernel path (tensor-core variant, row form or general CUDA-core contraction), the batch / free /
 * summed bit counts, and for tensor-core steps which index bit of the larger operand lies at each
 * of its address bits (from the lowest).  Writes at most len bytes (NUL-terminated) to buf and
 * returns 0; QXG_ERR_INVALID when the command is not an executed `ncon` of the plan (no plan is
 * built before the first amplitudes call).  A diagnostic with no counterpart in the reference. */
int qxg_program_explain(const qxg_program* prog, int32_t instr, char* buf, int32_t len);

/* The autotuner's decisions (tensor-core tile variant per step shape), as text, so that a later
 * programme -- in another process -- runs the same variants without timing them again.
 * qxg_program_tuning_get writes at most len bytes (NUL-terminated) and returns the length the
 * whole text needs (excluding the NUL), or a negative status; qxg_program_tuning_set merges a
 * text written by qxg_program_tuning_get (unknown shapes are ignored when planning).  No
 * counterpart in the reference. */
int qxg_program_tuning_get(const qxg_program* prog, char* buf, int64_t len);
int qxg_program_tuning_set(qxg_program* prog, const char* text);

/* Free the device buffers, graphs and stream of a programme.  Accepts NULL. */
void qxg_program_destroy(qxg_program* prog);

/* One pairwise contraction on device buffers: C = ncon(A, B) with the labels and dimensions
 * of one `ncon` command (a ContractCommand, src/compute_graph/compute_graph.jl:61-74;
 * QXTns.contract_pair! semantics).  A, B, C are column-major interleaved complex arrays of
 * the given precision's storage type (QXG_PREC_FP64: double2 with FP64 arithmetic; the other
 * modes: float2 with FP32 arithmetic); `stream` is a cudaStream_t or NULL for the default
 * stream.  Dimensions must be powers of two.  Enqueues one kernel; a float2 contraction with
 * few results and a sum of 2^12 or more terms enqueues two, with their partial sums in scratch
 * taken and returned in stream order (cudaMallocAsync / cudaFreeAsync on `stream`). */
int qxg_ncon(int32_t precision,
             void* C, int32_t nc, const int32_t* c_labels,
             const void* A, int32_t na, const int32_t* a_labels, const int64_t* a_dims,
             const void* B, int32_t nb, const int32_t* b_labels, const int64_t* b_dims,
             void* stream);

/* Bytes of the library's static device scratch used by qxg_ncon_tc_static (64 MiB). */
#define QXG_TC_STATIC_SCRATCH_BYTES (64ll << 20)

/* One pairwise contraction on the tensor cores (3xBF16 or 3xTF32 split products, FP32
 * accumulation) that allocates no device memory.  No counterpart in the reference: it exists for
 * callers that cannot call cudaMalloc -- code running while a CUDA graph is being captured, hosts
 * whose allocator is owned by another runtime, or allocation-free real-time loops.  The packed
 * hi/lo operand planes live in one file-scope device array of QXG_TC_STATIC_SCRATCH_BYTES that
 * every GPU loading the library holds until the process exits; a shape whose planes do not fit
 * is rejected with QXG_ERR_UNSUPPORTED and a message, and so is a shape the tensor cores do not
 * serve (fewer than 128 free rows on the larger operand -- 16 when the summed extent is above
 * 1024 --, a summed extent below 8, or a smaller operand with fewer than 4 free columns); sums
 * longer than 1024 are cut into blocks whose partial results are added in a fixed order.  Arguments are those of qxg_ncon with precision
 * QXG_PREC_SPLIT_BF16 or QXG_PREC_SPLIT_TF32 (float2 storage).  The first call on a device looks
 * up the array's device address (make that first call before any stream capture).  Every call on
 * a device shares that device's array, which keeps the last call's contents: calls that can
 * overlap on one GPU (issued on different streams or from different threads) race, so the caller
 * must order them. */
int qxg_ncon_tc_static(int32_t precision,
                       void* C, int32_t nc, const int32_t* c_labels,
                       const void* A, int32_t na, const int32_t* a_labels, const int64_t* a_dims,
                       const void* B, int32_t nb, const int32_t* b_labels, const int64_t* b_dims,
                       void* stream);

/* Sizes of the arrays qxg_parse_qx fills (capacities on input when it fills them). */
typedef struct qxg_qx_sizes {
    int32_t ninstr;       /* commands */
    int32_t ndata;        /* distinct data keys */
    int64_t nlabels;      /* ncon labels, concatenated */
    int64_t ndims;        /* data dimensions, concatenated over the data keys */
    int64_t key_bytes;    /* bytes of the data keys, each NUL-terminated, one after another */
    int32_t nqubits;      /* largest output qubit: the bitstring length */
    int32_t reserved[3];
} qxg_qx_sizes;

/* Parse `.qx` DSL text (docs/src/users_guide.md:93-165, the file generate_simulation_files
 * writes, src/simulation.jl:52-77) into qxg_program_create's arguments: one qxg_instr per
 * command, the concatenated ncon labels, and per data key (numbered in order of first `load`)
 * its rank and dims and its name (the `data_N` key of the leaf data file).  Replaces the parse
 * QXContexts performs in `execute` (bin/qxrun.jl:83-87).  Host code only, no device.
 * With instrs, labels, data_rank, data_dims and data_keys all NULL it only sets *sizes; else
 * *sizes holds the capacities of those arrays on input (too small: QXG_ERR_INVALID) and the sizes
 * used on output.  A malformed line, an unknown command, a tensor defined twice or used before
 * its definition, or a data key loaded with two shapes gives QXG_ERR_INVALID with the line
 * number in qxg_last_error. */
int qxg_parse_qx(const char* text, qxg_qx_sizes* sizes, qxg_instr* instrs, int32_t* labels,
                 int32_t* data_rank, int64_t* data_dims, char* data_keys);

/* Output methods of a `.yml` parameter file (output_params_dict, src/outputs.jl:47-78). */
typedef enum qxg_output_method {
    QXG_OUTPUT_LIST = 0,       /* params.bitstrings, explicit */
    QXG_OUTPUT_UNIFORM = 1,    /* params.num_samples bitstrings drawn uniformly from params.seed */
    QXG_OUTPUT_REJECTION = 2   /* rejection sampling with params.M, params.fix_M, params.seed */
} qxg_output_method;

/* The `output:` block of a `.yml` parameter file. */
typedef struct qxg_yml_output {
    int32_t method;        /* qxg_output_method */
    int32_t num_qubits;    /* List: length of its bitstrings; Uniform, Rejection: params.num_qubits */
    int64_t num_samples;   /* params.num_samples (List without it: the number of bitstrings) */
    int64_t nbitstrings;   /* List: bitstrings listed; 0 for the other methods */
    int64_t seed;          /* params.seed when has_seed */
    double M;              /* Rejection: params.M (1e-4 when absent) */
    int32_t has_seed;      /* 0 when the seed is absent or ~ */
    int32_t fix_M;         /* Rejection: params.fix_M (0 when absent) */
    int32_t reserved[4];
} qxg_yml_output;

/* Read the `output:` block of the `.yml` parameter file that generate_parameter_file writes
 * (src/simulation.jl:149-155; layout docs/src/users_guide.md:22-35), the List bitstrings that
 * QXContexts' `execute` reads in bin/qxrun.jl:83-87.  The YAML read is the subset those writers
 * produce: block mappings, block (`- x`) or flow (`[x, y]`) sequences of scalars, plain or quoted
 * scalars, `~`, `#` comment lines.  Fills *out; for a List with `bitstrings` non-NULL it also
 * writes the bitstrings packed, nbitstrings x num_qubits characters with no separators (the
 * layout qxg_amplitudes takes); capacity is that buffer's size in bytes.  Bitstring characters
 * are `0 1 + -`, all of one length, taken as written (a plain `010` stays "010").  Host code
 * only, no device.  A missing `output:` block, method or params, an unknown method, a malformed
 * line, or a bitstring of another length or character gives QXG_ERR_INVALID with the line
 * number in qxg_last_error. */
int qxg_parse_yml_output(const char* text, qxg_yml_output* out, char* bitstrings, int64_t capacity);

/* Options of qxg_plan_contraction (zero-initialised: the defaults). */
typedef struct qxg_plan_options {
    int32_t trials;          /* recursive-bisection trees tried (0: 64) */
    int32_t greedy_trials;   /* random-greedy trees tried besides them (0: 16; negative: none) */
    int64_t seed;            /* the search is deterministic for a seed */
    double max_log2;         /* slice labels until every intermediate has <= 2^max_log2 elements
                                (<= 0: no width target) */
    int32_t num_sliced;      /* slice at least this many labels (number_bonds_to_slice; 0: none) */
    int32_t max_sliced;      /* slice at most this many labels (0: no limit) */
    double flops_per_s;      /* step model: max(FLOPs / flops_per_s, bytes / bytes_per_s); 0: 1e14 */
    double bytes_per_s;      /* 0: 5e12 (Complex64 bytes of A, B and C) */
    const uint8_t* tensor_batched;  /* ntensors flags (NULL: none): the tensors that change with the
                                       bitstring (the `output` tensors); every step that depends on
                                       one runs once per bitstring of a batch */
    double batch_log2;       /* log2 of the bitstrings run together, for the step model */
    int32_t reserved[6];
} qxg_plan_options;

typedef struct qxg_plan_stats {
    double log2_flops;        /* FLOPs of one slice (8 |A u B| per step, complex), log2 */
    double log2_flops_total;  /* FLOPs of all slices, log2 */
    double max_log2;          /* elements of the largest intermediate of one slice, log2 */
    double time;              /* modelled seconds of one slice */
    double log2_slices;       /* number of slices, log2 */
    int32_t num_sliced;       /* labels sliced */
    int32_t trees_tried;
    int32_t reserved[6];
} qxg_plan_stats;

/* Contraction tree and sliced labels for a tensor network given as a hypergraph: tensor v holds
 * labels[label_off[v] .. label_off[v+1]) (ids 0..nlabels-1), label l has dimension
 * 2^label_log2dim[l] and is kept to the end when label_open[l] (NULL: none open).  A label is
 * summed by the contraction that encloses all its holders (QXTns contraction_indices, called at
 * src/compute_graph/compute_graph.jl:65).  Writes ntensors-1 steps to pairs: step k contracts
 * nodes pairs[2k] and pairs[2k+1] into node ntensors+k (nodes 0..ntensors-1 are the tensors); the
 * steps in order are an `(A, B, C)` plan (src/contraction_planning.jl:386-448).  label_sliced
 * (optional, nlabels bytes) marks the labels to slice (contraction_scheme's bond groups,
 * :219-299).  Replaces FlowCutter (flow_cutter_contraction_plan, :90-113), which QXTools calls
 * but does not ship, by recursive hypergraph bisection and randomised greedy trees scored by the
 * executor's step model, then greedy slicing.  Host code only, no device. */
int qxg_plan_contraction(int32_t ntensors, const int64_t* label_off, const int32_t* labels, int32_t nlabels,
                         const int32_t* label_log2dim, const uint8_t* label_open,
                         const qxg_plan_options* opts, int32_t* pairs, uint8_t* label_sliced,
                         qxg_plan_stats* stats);

/* Thread-local description of the last error ("" when none). */
const char* qxg_last_error(void);

/* Library version string, e.g. "qxgpu 0.1.0 sm_103a". */
const char* qxg_version(void);

#ifdef __cplusplus
}
#endif

#endif /* QXGPU_H */
