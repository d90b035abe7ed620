/*
 * fpg.h -- C ABI of the GB300 Pauli apply / expectation engine (libfpg.so).
 *
 * This is the drop-in boundary for the hot path of qognitive/fast-pauli:
 * PauliString / PauliOp / SummedPauliOp apply, apply_weighted and
 * expectation_value.  The reference's bindings call its header-only C++
 * templates directly (fast_pauli/cpp/src/include/__*_bindings.hpp); here the
 * C++ host classes (fast-pauli_gb300/cpp/include/fast_pauli_gb300.hpp) and the
 * Python module fast_pauli._fast_pauli call these entry points instead.
 *
 * Conventions
 *  - Every function returns an int status: FPG_OK (0) or an FPG_ERR_* code;
 *    nothing aborts.  fpg_last_error() gives the message of the calling
 *    thread's last failure.  Argument errors map to the reference's
 *    std::invalid_argument (Python ValueError).
 *  - Array arguments are DEVICE pointers owned by the caller, row-major.
 *    States are (2^n_qubits, n_states): states are columns, the state index is
 *    the fastest-varying, exactly the reference's layout.
 *  - Outputs ACCUMULATE (+=) like the reference (e.g.
 *    fast_pauli/cpp/include/__pauli_string.hpp:338,432,534,
 *    __summed_pauli_op.hpp:609): callers zero them first.
 *  - Work is ordered on `stream` (a cudaStream_t, NULL = legacy default
 *    stream); functions return once the work is enqueued.  Scratch memory is
 *    drawn from the library's stream-ordered pool (fpg_device_alloc).
 *  - dtype FPG_C128: complex128 data, float64 arithmetic (the reference's
 *    precision).  dtype FPG_C64: complex64 data, float32 arithmetic with
 *    compensated float32 partial sums, float64 cross-block reduction, 3xTF32
 *    tensor-core coefficient contraction.
 *  - Pauli strings are passed as characters 'I','X','Y','Z', n_qubits
 *    characters per string, concatenated.  The leftmost character acts on the
 *    most significant bit of the row index (reference: __pauli_string.hpp:54).
 */
#ifndef FPG_H
#define FPG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FPG_ABI_VERSION 1

enum fpg_status
{
    FPG_OK = 0,
    FPG_ERR_INVALID = 1,     /* bad argument: shapes, characters, null pointers  */
    FPG_ERR_CUDA = 2,        /* a CUDA runtime call failed                        */
    FPG_ERR_NOMEM = 3,       /* device or host allocation failed                  */
    FPG_ERR_UNSUPPORTED = 4, /* e.g. n_qubits beyond the supported range          */
    FPG_ERR_TIMEOUT = 5,     /* a bounded device wait gave up                     */
    FPG_ERR_BUSY = 6         /* admission refused (serving loop)                  */
};

enum fpg_dtype
{
    FPG_C128 = 0,
    FPG_C64 = 1
};

/* Opaque, device-resident encoding of a list of Pauli strings:
 * per string (x mask, z mask, #Y), grouped by x mask. */
typedef struct fpg_operator fpg_operator;

/* ABI version (FPG_ABI_VERSION). */
int fpg_abi_version(void);

/* Message for the calling thread's most recent failure ("" if none). */
const char *fpg_last_error(void);

/* Running total of kernels this library has launched (all devices, all
 * threads); lets a caller count the kernels inside a timed region. */
int fpg_kernel_launches(uint64_t *total);

/* Status of the library's bounded device waits since the last call: *code = 0
 * if every wait completed, FPG_ERR_TIMEOUT-class failure (nonzero) if a
 * tensor-core kernel gave up waiting on an mbarrier (its results are then
 * invalid).  Synchronises `stream` and clears the flag. */
int fpg_device_error(int *code, void *stream);

/* Measured fused multiply-add rate of the current device, lane operations
 * per second (one FMA = 1; multiply by 2 for FLOP/s): dtype FPG_C64 the
 * float32 pipe, FPG_C128 the float64 pipe.  Runs a ~10 ms kernel of
 * independent FMA chains on `stream` and synchronises it.  The roof of the
 * float64 expectation stage, which runs as double-float on the float32
 * pipes.  No reference counterpart (used to report rooflines). */
int fpg_measure_peak(int32_t dtype, double *fma_per_s, void *stream);

/* Number of visible CUDA devices (0 on a machine without a GPU). */
int fpg_device_count(int *count);

/* 1 if ptr is device (or managed) memory on some device, else 0. */
int fpg_pointer_is_device(const void *ptr, int *is_device);

/* Stream-ordered device memory from the library's pool on the current
 * device (the pool the entry points take their scratch from).  Freed memory
 * stays mapped for reuse up to FPG_POOL_KEEP_BYTES (environment, bytes;
 * default 4 GiB), so calls that synchronise do not remap their buffers.
 * bytes = 0 allocates a minimal block.  FPG_ERR_NOMEM when the device is
 * full.  No reference counterpart: the reference's CPU path allocates with
 * std::vector per call (__summed_pauli_op.hpp). */
int fpg_device_alloc(void **ptr, size_t bytes, void *stream);
int fpg_device_free(void *ptr, void *stream);
/* Give the pool's unused memory back to the device (all devices). */
int fpg_release_cached_memory(void);

/*
 * Encode n_strings Pauli strings of n_qubits characters each and upload the
 * encoding to the current device.  Replaces the per-call get_sparse_repr of
 * the reference (__pauli_string.hpp:49-118), which the reference rebuilds for
 * every string on every apply/expectation call.  Raises FPG_ERR_INVALID on a
 * character outside IXYZ (reference: PauliString(std::string),
 * __pauli_string.hpp:193-194).  1 <= n_qubits <= 40.
 */
int fpg_operator_create(const char *strings, int64_t n_strings, int32_t n_qubits, fpg_operator **out);
int fpg_operator_destroy(fpg_operator *op);
int fpg_operator_info(const fpg_operator *op, int32_t *n_qubits, int64_t *n_strings, int64_t *n_groups);

/*
 * Work of one expectation pass per state column: number of chunks (CTA work
 * units), row visits summed over chunks (a visit loads a row pair and forms
 * conj(psi_i) psi_{i^x}), and signed accumulations (string slots x visits).
 * Used to report arithmetic rooflines; no counterpart in the reference.
 */
int fpg_operator_stats(const fpg_operator *op, int64_t *n_chunks, int64_t *row_visits, int64_t *sign_adds);

/*
 * The same work split by the kernel family that does it: row_visits[f] and
 * sign_adds[f] for f in FPG_FAMILY_DIRECT .. FPG_FAMILY_TILE (arrays of
 * FPG_FAMILY_COUNT entries).  The families compute with different float32
 * costs per float64 operation in the df64 form, which bench.py's roofline
 * counts.  No counterpart in the reference.
 */
enum
{
    FPG_FAMILY_DIRECT = 0,    /* direct-kernel chunks */
    FPG_FAMILY_TRANSFORM = 1, /* 16-point Walsh-Hadamard transform kernel */
    FPG_FAMILY_PAIR = 2,      /* pair kernel */
    FPG_FAMILY_MARGINAL = 3,  /* marginal kernel */
    FPG_FAMILY_TILE = 4,      /* tile kernel (two-position groups, four row bits per unit) */
    FPG_FAMILY_COUNT = 5
};
int fpg_operator_family_stats(const fpg_operator *op, int64_t *row_visits, int64_t *sign_adds);

/*
 * Sparse pattern of one Pauli string on the device: cols[i] = column of the
 * non-zero in row i, vals[i] = its value (complex128 interleaved), i < 2^n.
 * Bit-exact replacement for get_sparse_repr<double>
 * (__pauli_string.hpp:49-118; Python helpers.pauli_string_sparse_repr,
 * fast_pauli/cpp/src/fast_pauli.cpp:92).
 */
int fpg_sparse_repr(const char *string, int32_t n_qubits, uint64_t *cols, void *vals, void *stream);

/*
 * out(D,S) += sum_j coeffs[j] * P_j * states        (coeffs: n_strings complex)
 * Replaces PauliOp::apply (__pauli_op.hpp:399-468) and, with one string,
 * PauliString::apply_batch (__pauli_string.hpp:378-436).
 * Scratch (this call and fpg_summed_apply): FPG_C128 takes double-float
 * copies of the states and coefficients (16 bytes per complex element); with
 * 4 or more states and 2 or more strings per x-group on average, a table of
 * the x-groups' diagonals (16 bytes per group and state row for FPG_C128,
 * 8 for FPG_C64; at most 1 GiB; left out when the pool cannot supply it).
 */
int fpg_apply(const fpg_operator *op, const void *coeffs, const void *states, void *out, int64_t n_states,
              int32_t dtype, void *stream);

/*
 * Per-string expectation values ev(j,t) = <psi_t| P_j |psi_t> (real; Pauli
 * strings are Hermitian), float64, shape (n_strings, n_states); ev is
 * OVERWRITTEN.  The per-string stage of SummedPauliOp::expectation_value
 * (__summed_pauli_op.hpp:572-577) and of PauliString::expectation_value
 * (__pauli_string.hpp:471-538).
 */
int fpg_expect_strings(const fpg_operator *op, const void *states, double *ev, int64_t n_states, int32_t dtype,
                       void *stream);

/*
 * out(K,S) += sum_j coeffs(j,k) * <psi_t|P_j|psi_t>   (coeffs: (n_strings, K) complex)
 * Replaces SummedPauliOp::expectation_value (__summed_pauli_op.hpp:520-614);
 * with K = 1 it is PauliOp::expectation_value (__pauli_op.hpp:482-549).
 */
int fpg_summed_expect(const fpg_operator *op, const void *coeffs, int64_t n_operators, const void *states, void *out,
                      int64_t n_states, int32_t dtype, void *stream);

/*
 * out(D,S) += sum_j (sum_k coeffs(j,k)) P_j states
 * Replaces SummedPauliOp::apply (__summed_pauli_op.hpp:277-349).
 */
int fpg_summed_apply(const fpg_operator *op, const void *coeffs, int64_t n_operators, const void *states, void *out,
                     int64_t n_states, int32_t dtype, void *stream);

/*
 * out(:,t) += sum_j w(j,t) P_j states(:,t),  w(j,t) = sum_k coeffs(j,k) data(k,t)
 * data is real, shape (K, S): float64 for FPG_C128, float32 for FPG_C64.
 * Replaces SummedPauliOp::apply_weighted (__summed_pauli_op.hpp:365-503).
 */
int fpg_summed_apply_weighted(const fpg_operator *op, const void *coeffs, int64_t n_operators, const void *states,
                              const void *data, void *out, int64_t n_states, int32_t dtype, void *stream);

/*
 * Product of two operators with equal strings merged:
 *   (sum_i coeffs_a(i) A_i) (sum_j coeffs_b(j) B_j) = sum_k c_k C_k
 * over the distinct strings C_k among the products A_i B_j.  Replaces
 * PauliOp operator* (__pauli_op.hpp:237-281) and PauliString::operator*
 * (__pauli_string.hpp:228-247) inside it.  coeffs_a (n_strings(a)) and
 * coeffs_b (n_strings(b)) are complex128 device arrays; the results go to
 * device arrays of n_strings(a) * n_strings(b) entries: out_x, out_z the
 * (x, z) masks of C_k (bit n-1-q is character q: I (0,0), X (1,0), Y (1,1),
 * Z (0,1)), sorted by (x, z), and out_coeffs the complex128 c_k; *n_out
 * (host) receives the number of distinct strings.  Coefficients are summed
 * in pair order (i, j), so results are deterministic.  Synchronises
 * `stream`.  FPG_ERR_UNSUPPORTED when n_strings(a) * n_strings(b) >= 2^31.
 */
int fpg_op_product(const fpg_operator *a, const void *coeffs_a, const fpg_operator *b, const void *coeffs_b,
                   uint64_t *out_x, uint64_t *out_z, void *out_coeffs, int64_t *n_out, void *stream);

/*
 * Coefficients of the squares A_k^2 of a SummedPauliOp's operators
 * A_k = sum_j coeffs(j,k) P_j:
 *   out(a,k) = sum_{i,j: P_i P_j = phase * Q_a} phase * coeffs(i,k) * coeffs(j,k)
 * over the strings Q_a of `sq` (normally all strings of weight up to
 * min(n, 2 * max weight), calculate_pauli_strings_max_weight).  coeffs
 * (n_strings(op), K) and out (n_strings(sq), K) are device arrays of dtype;
 * out is OVERWRITTEN.  Returns FPG_ERR_INVALID if some product P_i P_j is not
 * a string of sq.  Synchronises `stream` before returning.
 * Replaces SummedPauliOp::square (__summed_pauli_op.hpp:197-268).
 */
int fpg_summed_square(const fpg_operator *op, const void *coeffs, int64_t n_operators, const fpg_operator *sq,
                      void *out, int32_t dtype, void *stream);

/*
 * Dense matrices of the operators A_k = sum_j coeffs(j,k) P_j:
 *   out(k, i, j) += A_k(i, j),   out (K, 2^n, 2^n) complex, coeffs (n_strings, K),
 * both device arrays of dtype.  Outputs accumulate, as in the reference.
 * Replaces SummedPauliOp::to_tensor (__summed_pauli_op.hpp:644-665) and, with
 * K = 1, PauliOp::to_tensor (__pauli_op.hpp:558-571).
 */
int fpg_to_tensor(const fpg_operator *op, const void *coeffs, int64_t n_operators, void *out, int32_t dtype,
                  void *stream);

/* ------------------------------------------------------------------------
 * Batches: many expectation problems of uneven size (qubits, strings,
 * states, operators) run as one persistent work-queue launch per chunk class
 * plus a reduction and a contraction -- no allocation at run time, so a run
 * can be captured into a CUDA graph.  No counterpart in the reference (its
 * equivalent is a loop of PauliOp/SummedPauliOp::expectation_value calls,
 * __pauli_op.hpp:482-549, __summed_pauli_op.hpp:520-614).
 * Each problem: out(K,S) = sum_j coeffs(j,k) <psi_t|P_j|psi_t>; a run
 * OVERWRITES the outputs (so repeated runs and autotuning are idempotent).
 * All arrays are device arrays of the batch's dtype and must stay valid
 * while the batch is used.  Runs of one batch must not overlap on the GPU.
 * ------------------------------------------------------------------------ */
typedef struct fpg_batch fpg_batch;

typedef struct fpg_batch_tuning
{
    int32_t threads_per_cta; /* 128 or 256                                          */
    int32_t ctas_per_sm;     /* CTAs per SM of each persistent grid, 1..8; 0 = as
                                many as the kernel's residency allows (default);
                                -1 = item grid: one CTA per work item, drained by
                                the hardware block scheduler                        */
    int32_t rows_per_item;   /* row window of one work item when a problem's column
                                tile exceeds tile_mb (power of two >= 32)          */
    int32_t tile_mb;         /* column-tile budget (MiB) for L2 residency, >= 1   */
} fpg_batch_tuning;

int fpg_batch_create(int32_t dtype, fpg_batch **out);
int fpg_batch_add(fpg_batch *batch, const fpg_operator *op, const void *coeffs, int64_t n_operators,
                  const void *states, void *out, int64_t n_states);
/* Build the work queue and per-problem partial tables (allocates device memory).
 * tuning NULL: the batch's current tuning (defaults 256 / 0 / 32768 / 40). */
int fpg_batch_plan(fpg_batch *batch, const fpg_batch_tuning *tuning);
/* Enqueue one run on stream (plans first if needed). */
int fpg_batch_run(fpg_batch *batch, void *stream);
/* Same, through a CUDA graph captured on first use and replayed afterwards. */
int fpg_batch_run_graph(fpg_batch *batch, void *stream);
/* Times every candidate tuning on this batch (runs it 3x per candidate),
 * re-plans with the fastest and reports it. */
int fpg_batch_autotune(fpg_batch *batch, void *stream, fpg_batch_tuning *best, double *best_ms);
int fpg_batch_info(const fpg_batch *batch, int64_t *n_problems, int64_t *n_items, fpg_batch_tuning *tuning);
int fpg_batch_destroy(fpg_batch *batch);

/* ------------------------------------------------------------------------
 * Serving: a device-resident request loop with continuous admission.  No
 * counterpart in the reference.  Requests reference resident operators and
 * device arrays; a scheduler thread admits queued requests as soon as a slot
 * (one CUDA stream) is free and the request's scratch fits the remaining HBM
 * budget, so requests arriving while others run are started immediately and
 * overlap on the device.  A request needing more than the whole budget, or
 * arriving at a full queue, is refused with FPG_ERR_BUSY.  Outputs are
 * overwritten.  Small expectation requests (n_strings x 2^n x n_states <= 4e9)
 * admitted in the same scheduling round run as one merged batch (one
 * work-queue kernel per chunk class, one reduction, one contraction) on one
 * slot; alone, such a request runs as a merge of one.  Results do not depend
 * on the mix (a request runs the same kernels, in the same summation order,
 * alone and in the mix).
 * ------------------------------------------------------------------------ */
enum fpg_request_kind
{
    FPG_REQ_EXPECT = 0,        /* out(K,S) = sum_j coeffs(j,k) <psi_t|P_j|psi_t>               */
    FPG_REQ_APPLY_WEIGHTED = 1 /* out(D,S) = sum_j (sum_k coeffs(j,k) data(k,t)) P_j psi_t   */
};

typedef struct fpg_request
{
    int32_t kind;
    int32_t reserved;
    const fpg_operator *op;
    const void *coeffs; /* (n_strings, n_operators) complex, device             */
    int64_t n_operators;
    const void *states; /* (2^n, n_states) complex, device                        */
    const void *data;   /* (n_operators, n_states) real, APPLY_WEIGHTED only      */
    void *out;          /* (K, S) or (2^n, S) complex, device                     */
    int64_t n_states;
} fpg_request;

typedef struct fpg_server_config
{
    int32_t dtype;            /* FPG_C128 or FPG_C64 for every request            */
    int32_t n_slots;          /* concurrent requests (streams), 1..64             */
    int64_t hbm_budget_bytes; /* scratch memory all running requests may hold   */
    int64_t max_queue;        /* queued requests before refusing (<= 0: 2^20)   */
} fpg_server_config;

typedef struct fpg_ticket_info
{
    int32_t status; /* 2 done, 3 failed                                        */
    int32_t reserved;
    int64_t scratch_bytes;
    double submit_us, start_us, done_us; /* steady clock, microseconds since server creation */
} fpg_ticket_info;

typedef struct fpg_server_stats_t
{
    int64_t completed, failed, refused, queued;
    int32_t peak_running;
    int32_t reserved;
    int64_t peak_reserved_bytes;
    int64_t merged_runs;     /* merged launch sequences of small expectation requests */
    int64_t merged_requests; /* requests those runs served                            */
} fpg_server_stats_t;

typedef struct fpg_server fpg_server;

int fpg_server_create(const fpg_server_config *config, fpg_server **out);
int fpg_server_submit(fpg_server *server, const fpg_request *request, uint64_t *ticket);
/* Block until the ticket finishes (timeout_ms < 0: no limit); fills info. */
int fpg_server_wait(fpg_server *server, uint64_t ticket, int32_t timeout_ms, fpg_ticket_info *info);
/* Forget a finished ticket. */
int fpg_server_release(fpg_server *server, uint64_t ticket);
int fpg_server_stats(fpg_server *server, fpg_server_stats_t *stats);
/* Drains queued and running requests, then stops the scheduler. */
int fpg_server_destroy(fpg_server *server);

/*
 * fpg_summed_expect_noalloc: the same result as fpg_summed_expect
 * (out(K,S) += sum_j coeffs(j,k) <psi_t|P_j|psi_t>), for callers that cannot
 * allocate device memory: processes living inside a framework that has
 * already reserved almost all of the GPU for its own pool (where cudaMalloc
 * fails or bypasses that pool), and latency-bound request loops that may not
 * allocate because an allocation can block or synchronise the device.  It
 * takes the strings themselves (no fpg_operator, whose creation allocates),
 * allocates nothing, and keeps its scratch -- the encoded strings and the
 * n_strings x n_states float64 table of per-string expectation values -- in
 * one 16 MiB static device array that every GPU loading libfpg.so holds until
 * exit.
 * Limits: n_strings <= 8192 and n_strings * n_states up to about 2 million
 * (the table must fit the array); larger requests return FPG_ERR_INVALID.
 * The first call on a device resolves the array's address and keeps it for
 * the life of the process (so not for processes that call cudaDeviceReset);
 * calls whose GPU work overlaps race on the shared array.  The encoding is
 * copied from static host arrays, so a call made while `stream` is being
 * captured returns FPG_ERR_UNSUPPORTED.  Rows are not split: an operator of
 * a few strings on a large state runs on few CTAs (slower than
 * fpg_summed_expect).
 * No counterpart in the reference.
 */
int fpg_summed_expect_noalloc(const char *strings, int64_t n_strings, int32_t n_qubits, const void *coeffs,
                              int64_t n_operators, const void *states, void *out, int64_t n_states, int32_t dtype,
                              void *stream);

#ifdef __cplusplus
}
#endif

#endif /* FPG_H */
