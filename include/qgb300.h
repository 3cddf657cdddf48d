/*
 * qgb300.h — C ABI of the GB300 (sm_103a) state-vector engine behind the
 * qibo backend plugin ``qibo_gb300``.
 *
 * The reference (qibo 0.3.5) is pure Python and has no FFI of its own; its
 * backend interface is the Python class ``qibo.backends.abstract.Backend``.
 * Each entry point below states which reference method it replaces
 * (paths relative to the reference's ``src/qibo/``).  A Python, C or C++
 * host binds these symbols with plain pointers and sizes (ctypes in
 * ``qibo_gb300/_lib.py``).
 *
 * Conventions
 *  - Every function returns an int status: QGB_OK (0) or one of the
 *    QGB_ERR_* codes; ``qgb_last_error()`` gives the message of the last
 *    failure on the calling host thread.
 *  - A state is a device buffer of 2^nqubits interleaved complex amplitudes:
 *    QGB_C128 = 2 x double (16 B), QGB_C64 = 2 x float (8 B), allocated with
 *    ``qgb_malloc`` (or any cudaMalloc'ed buffer with 256-byte alignment).
 *  - Qubit numbering is qibo's: qubit 0 is the most significant bit of the
 *    amplitude index (backends/abstract.py:2327-2355), i.e. qubit q has
 *    stride 2^(nqubits-1-q).
 *  - Gate matrices are host arrays of 2*4^k doubles (re, im interleaved,
 *    row-major, rows = outputs), whose index bits follow the order of the
 *    ``qubits`` array: qubits[0] is the most significant matrix-index bit
 *    (the reference's ``matrix @ state`` after moving ``gate.qubits`` to the
 *    front, backends/abstract.py:2350-2355).  Matrices travel by value in the
 *    kernel parameters: no device allocation, no host-device copy.
 *  - ``stream`` is a cudaStream_t (NULL = legacy default stream).  All
 *    calls are asynchronous and stream-ordered unless stated otherwise.
 */
#ifndef QGB300_H
#define QGB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QGB_OK 0
#define QGB_ERR_INVALID 1     /* bad argument (qubit out of range, size, dtype) */
#define QGB_ERR_OOM 2         /* device allocation failed (backends/abstract.py:2500-2510) */
#define QGB_ERR_CUDA 3        /* any other CUDA runtime error */
#define QGB_ERR_TIMEOUT 4     /* a bounded device wait gave up */
#define QGB_ERR_UNSUPPORTED 5 /* valid request the library does not handle */

#define QGB_C64 0
#define QGB_C128 1

/* ---- library / device ------------------------------------------------- */
const char* qgb_last_error(void);
int qgb_version(void);
/* Number of kernels this library has launched in the process so far. */
int64_t qgb_launch_count(void);
/* Select the device and report its SM count. */
int qgb_device_init(int device, int* sm_count);
int qgb_mem_info(size_t* free_bytes, size_t* total_bytes);
int qgb_malloc(void** ptr, size_t bytes);              /* OOM -> QGB_ERR_OOM */
int qgb_free(void* ptr);
int qgb_memcpy_h2d(void* dst, const void* src, size_t bytes, void* stream);
int qgb_memcpy_d2h(void* dst, const void* src, size_t bytes, void* stream);
int qgb_memcpy_d2d(void* dst, const void* src, size_t bytes, void* stream);
int qgb_memset_zero(void* ptr, size_t bytes, void* stream);
/* Page-locked host memory (asynchronous device->host result copies). */
int qgb_host_alloc(void** ptr, size_t bytes);
int qgb_host_free(void* ptr);
int qgb_stream_sync(void* stream);

/* ---- state creation: Backend.zero_state (backends/abstract.py:2243-2273),
 *      NumpyBackend.cast (backends/numpy.py:38-64) ----------------------- */
int qgb_state_zero(void* state, int nqubits, int dtype, void* stream);
int qgb_state_basis(void* state, int nqubits, int dtype, int64_t index, void* stream);
/* dst = src converted between QGB_C128 and QGB_C64 (same n). */
int qgb_state_cast(const void* src, int src_dtype, void* dst, int dst_dtype, int nqubits, void* stream);
/* state *= scale (real); used for renormalisation. */
int qgb_state_scale(void* state, int nqubits, int dtype, double scale, void* stream);

/* ---- gate application: Backend.apply_gate (backends/abstract.py:2322-2361)
 *      and Backend._apply_gate_controlled_by (:3176-3197) ---------------- */
/* Apply the 2^k x 2^k ``matrix`` on ``qubits[0..k)`` (k <= 5), active only
 * where every qubit in ``controls[0..ncontrols)`` is 1 (ncontrols may be 0).
 * The engine classifies the matrix (hidden controls, diagonal, permutation
 * with phases, dense) and launches the matching kernel. */
int qgb_apply_gate(void* state, int nqubits, int dtype, const int* qubits, int k,
                   const int* controls, int ncontrols, const double* matrix, void* stream);
/* Specialised entry points (no classification).  Dense 2x2 on ``target``. */
int qgb_apply_1q(void* state, int nqubits, int dtype, int target, const double* matrix, void* stream);
/* Dense 4x4 on (q0, q1); q0 is the most significant matrix bit. */
int qgb_apply_2q(void* state, int nqubits, int dtype, int q0, int q1, const double* matrix, void* stream);
/* Multiply by phase (re, im) every amplitude whose qubits[0..nq) are all 1
 * (CZ, CU1, CCZ, Z, S, T, U1 after control extraction). */
int qgb_apply_phase(void* state, int nqubits, int dtype, const int* qubits, int nq,
                    double phase_re, double phase_im, void* stream);
/* SWAP (models/qft.py:56-58 uses it), optionally controlled. */
int qgb_apply_swap(void* state, int nqubits, int dtype, int q0, int q1,
                   const int* controls, int ncontrols, void* stream);

/* Apply a whole gate list (a circuit, or a fused block sequence) in order.
 * ``ops`` is an array of ``nops`` qgb_op records, ``coefs`` holds their
 * matrices (each op's ``coef_offset`` indexes doubles).  The engine plans
 * shared-memory passes that apply many gates per read+write of the state
 * when ``flags & QGB_PLAN_BLOCKED``, otherwise it runs gate by gate.  Gate
 * by gate, complex128 dense gates of one or two qubits compute in
 * double-float too (the doubles split and joined with integer operations),
 * unless ``flags & QGB_PLAN_STRICT_FP64``; qgb_apply_gate keeps IEEE FP64.
 * Complex128 passes compute in double-float (two FP32 words per double,
 * about 48 significant bits) on the FP32 pipe unless
 * ``flags & QGB_PLAN_STRICT_FP64`` asks for IEEE FP64 arithmetic.  With
 * QGB_PLAN_BLOCKED, uncontrolled 5-qubit dense blocks (fused gates) run on
 * the tensor cores (qgb_apply_fused5_tc; complex128 from 12 qubits) unless
 * ``flags & QGB_PLAN_NO_TC``. */
typedef struct qgb_op {
    int32_t k;              /* number of gate qubits (<= 5) */
    int32_t ncontrols;      /* number of controls (<= 8) */
    int32_t qubits[5];      /* gate qubits, most significant matrix bit first */
    int32_t controls[8];
    int64_t coef_offset;    /* offset (in doubles) of the 2*4^k matrix in coefs */
} qgb_op;
#define QGB_PLAN_BLOCKED 1
#define QGB_PLAN_STRICT_FP64 2
#define QGB_PLAN_NO_TC 8       /* fused 5-qubit blocks in shared-memory passes instead of on the tensor cores */
#define QGB_PLAN_FUSE 16       /* with QGB_PLAN_BLOCKED: fuse the gate list into blocks of <= 5 qubits first
                                  (greedy forward scan, Circuit.fuse's role, models/circuit.py:954-1003),
                                  kept when it has at most 11 ops per pass of the unfused plan (circuits
                                  of mostly diagonal gates, such as QFT, run faster unfused) */
int qgb_apply_circuit(void* state, int nqubits, int dtype, const qgb_op* ops, int nops,
                      const double* coefs, int flags, void* stream);
/* What QGB_PLAN_FUSE makes of a gate list (host only): the number of ops
 * after fusion and how many of them are uncontrolled 5-qubit blocks (the
 * ones the tensor cores take).  pad_nqubits: the state's qubit count when
 * qgb_apply_circuit widens every block to 5 qubits (tensor cores in use and
 * nqubits >= 12), else 0. */
int qgb_fuse_stats(const qgb_op* ops, int nops, const double* coefs, int pad_nqubits, int* nops_out, int* nblocks5);
/* Number of state passes QGB_PLAN_BLOCKED would launch for this gate list
 * (host only, no device work). */
int qgb_plan_passes(int nqubits, int dtype, const qgb_op* ops, int nops, const double* coefs, int* npasses);

/* A fused 5-qubit block (FusedGate, gates/special.py:28-153, applied by
 * Backend.apply_gate with Backend.matrix_fused, backends/abstract.py:
 * 2680-2717) computed on the tensor cores, 128 groups of 32 amplitudes per
 * tcgen05 MMA tile.  complex64 (nqubits >= 5): 3xTF32 split (A_hi*B_hi +
 * A_hi*B_lo + A_lo*B_hi) with FP32 accumulation in tensor memory.
 * complex128 (nqubits >= 12): Ozaki scheme on the BF16 tensor cores, six
 * 8-bit digits per value in 47-bit fixed point, six exact FP32 level
 * accumulators, combined into IEEE doubles (error per output about 2^-45 of
 * the tile scale).  ``matrix`` as for qgb_apply_gate (32x32, qubits[0] most
 * significant).  QGB_ERR_UNSUPPORTED below the qubit minimum. */
int qgb_apply_fused5_tc(void* state, int nqubits, int dtype, const int* qubits, const double* matrix, void* stream);
/* *timed_out = 1 if a tensor-core launch since the previous call gave up
 * waiting for its MMAs or copies (that launch stopped early and its output
 * is invalid); clears the flag.  Not synchronising: it reads a flag in
 * mapped host memory, so call it after synchronising the streams whose
 * launches it should cover. */
int qgb_tc_status(int* timed_out);

/* ---- measurement: Backend.calculate_probabilities (:2734-2758,
 *      _order_probabilities :3371-3381), sample_shots / sample_frequencies
 *      (:2760-2801) --------------------------------------------------------- */
/* out[2^nq] (device, float64) = marginal probabilities of qubits[0..nq) in
 * the given order (qubits[0] is the most significant output bit),
 * accumulated in FP64.  ``scratch`` is a device buffer of at least
 * qgb_probs_scratch_bytes(nqubits, nq) bytes (may be NULL when that is 0). */
size_t qgb_probs_scratch_bytes(int nqubits, int nq);
int qgb_probabilities(const void* state, int nqubits, int dtype, const int* qubits, int nq,
                      double* out, void* scratch, void* stream);
/* Sum of |psi|^2 in FP64 written to *out (device pointer); ``scratch`` is a
 * device buffer of qgb_norm_scratch_bytes() bytes. */
size_t qgb_norm_scratch_bytes(void);
int qgb_norm2(const void* state, int nqubits, int dtype, double* out, void* scratch, void* stream);
/* Draw ``nshots`` outcomes from the (unnormalised) FP64 distribution
 * probs[0..2^m) with a Philox4x32-10 stream keyed by ``seed``; the CDF is an
 * FP64 prefix sum built in ``scratch`` (qgb_sample_scratch_bytes).  Writes
 * either samples[nshots] (int64, outcome index) or counts[2^m] (int64
 * histogram), whichever pointer is non-NULL (device pointers). */
size_t qgb_sample_scratch_bytes(int m);
int qgb_sample(const double* probs, int m, int64_t nshots, uint64_t seed, int64_t* samples,
               int64_t* counts, void* scratch, void* stream);
/* Shots on every qubit drawn straight from the state, without a 2^n
 * probability vector (for states that fill the GPU): FP64 chunk sums of
 * |psi|^2 over 64 amplitudes, their prefix scan, and an in-chunk recompute.
 * Draws follow the same Philox4x32-10 protocol as qgb_sample; samples[nshots]
 * (device, int64).  Scratch: qgb_sample_state_scratch_bytes(nqubits). */
size_t qgb_sample_state_scratch_bytes(int nqubits);
int qgb_sample_state(const void* state, int nqubits, int dtype, int64_t nshots, uint64_t seed, int64_t* samples,
                     void* scratch, void* stream);
/* qgb_sample without a scratch argument and without allocating: this entry
 * point has no counterpart in the reference.  It is for callers that cannot
 * allocate device memory when they need shots (a state that fills the GPU
 * leaves no room for a CDF buffer; a serving loop must not call
 * cudaMalloc/cudaFree, which can synchronise the device).  The CDF lives in a
 * fixed array inside the library (131 584 bytes held by every GPU that loads
 * it, until exit), so m is limited to 20 (2^20 outcomes); larger m returns
 * QGB_ERR_INVALID.  Same outputs as qgb_sample for the same arguments.  The
 * first call on a device looks up that array's device address (do it before
 * any stream capture); the address is kept per device, for the device's
 * primary context (the one the CUDA runtime uses), the only context this
 * entry point supports.  All calls share the one array: calls that can
 * overlap on the GPU (different streams without ordering) race and must not
 * be issued. */
int qgb_sample_noalloc(const double* probs, int m, int64_t nshots, uint64_t seed, int64_t* samples,
                       int64_t* counts, void* stream);
/* Raw Philox4x32-10 words: out[4t+e] = word e of philox(counter = (t_lo,
 * t_hi, c2, c3), key = (k0, k1)), t < n4 (device buffer).  Exposes the
 * generator behind qgb_sample for known-answer tests. */
int qgb_philox_fill(uint32_t* out, int64_t n4, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
                    void* stream);

/* ---- measurement outcomes: expectation values from samples
 *      (Backend.exp_value_diagonal_observable_symbolic_from_samples,
 *      backends/abstract.py:2873-2926) and state collapse
 *      (Backend.collapse_state / _collapse_statevector, :2424-2440,
 *      :3279-3304) ---------------------------------------------------------- */
/* odd[t] (device, int64) = number of samples[0..nshots) (device, int64
 * outcome indices) whose bits under masks[t] have odd parity, for
 * t < nterms (host masks).  Bit b of an outcome is bit b of the sampled
 * index: for probabilities over qubits[0..m), qubit qubits[i] is bit m-1-i.
 * Term t's mean of (-1)^parity over the shots is (nshots - 2 odd[t]) /
 * nshots, the reference's frequency-weighted sum; integer counts make it
 * independent of the reduction order. */
#define QGB_PARITY_MAX_TERMS 256
int qgb_parity_counts(const int64_t* samples, int64_t nshots, const uint64_t* masks, int nterms, int64_t* odd,
                      void* stream);
/* Collapse onto the outcome *outcome (device int64) of measuring qubits[0..nq)
 * (qubits[0] is the most significant outcome bit, as in qgb_probabilities):
 * amplitudes whose bits differ become 0; with ``normalize`` the kept ones are
 * divided by the FP64 norm of the kept slice (a slice of norm 0 gives NaN,
 * as in the reference).  The outcome is read on the device, so a shot drawn
 * by qgb_sample collapses the state without a host round trip.  ``scratch``:
 * qgb_norm_scratch_bytes() bytes (unused without ``normalize``). */
int qgb_collapse(void* state, int nqubits, int dtype, const int* qubits, int nq, const int64_t* outcome,
                 int normalize, void* scratch, void* stream);

/* ---- expectation values: Backend.exp_value_observable_symbolic
 *      (backends/abstract.py:2946-3054) ------------------------------------ */
/* out (device, float64) = sum_t coef[t] * <psi| P_t |psi> for Pauli strings
 * given as bit masks over qibo qubits (bit q of the mask = qubit q):
 * xmask = qubits carrying X or Y, zmask = qubits carrying Z or Y.  One pass
 * over the state for all terms, FP64 accumulation. */
int qgb_expect_pauli(const void* state, int nqubits, int dtype, const uint64_t* xmask,
                     const uint64_t* zmask, const double* coef, int nterms, double* out,
                     void* scratch, void* stream);
size_t qgb_expect_scratch_bytes(int nqubits, int nterms);
/* out (device) = Re sum_i conj(psi_i) (H psi)_i for a dense Hermitian H
 * (device, complex128 interleaved, row-major 2^n x 2^n, n <= 20):
 * Backend.expectation_value (backends/abstract.py:2807-2825) without the
 * normalisation, which the caller applies with qgb_norm2.  ``scratch``:
 * qgb_expect_scratch_bytes(nqubits, 1) bytes. */
int qgb_expect_dense(const void* state, int nqubits, int dtype, const double* hamiltonian, double* out,
                     void* scratch, void* stream);

/* ---- density matrices ------------------------------------------------------
 * A density matrix rho of n qubits (n <= 20) is the 2n-qubit "state"
 * v[i * 2^n + j] = rho[i, j] (row-major, the reference's rho.ravel()): row
 * qubit q is vector qubit q, column qubit q is vector qubit n + q.  A gate U
 * on qubits T is qgb_apply_circuit of U on T and conj(U) on T + n (the two
 * einsums of Backend.apply_gate with a density matrix,
 * backends/abstract.py:2322-2361, and _apply_gate_controlled_by_density_
 * matrix, :3199-3247, with the controls shifted likewise); a channel on T is
 * one dense superoperator on (T, T + n).  ``nqubits`` below is n. */
/* out[0..2^nq) (device, FP64) = marginal probabilities of ``qubits`` from
 * the diagonal (Backend.calculate_probabilities with density_matrix=True,
 * backends/abstract.py:2734-2758), qubits[0] the most significant outcome
 * bit; nq = 0 gives the real trace.  Fixed reduction order. */
size_t qgb_density_scratch_bytes(void);
int qgb_density_probabilities(const void* rho, int nqubits, int dtype, const int* qubits, int nq, double* out,
                              void* scratch, void* stream);
/* Backend.collapse_state with density_matrix=True (_collapse_density_matrix,
 * backends/abstract.py:3249-3277): entries whose row or column bits on
 * ``qubits`` differ from outcome *outcome (device int64) become 0; with
 * ``normalize`` the kept block is divided by its real trace.  ``scratch``:
 * qgb_density_scratch_bytes() bytes. */
int qgb_density_collapse(void* rho, int nqubits, int dtype, const int* qubits, int nq, const int64_t* outcome,
                         int normalize, void* scratch, void* stream);
/* out (device, FP64) = sum_t coef[t] Re Tr(P_t rho), Pauli strings as in
 * qgb_expect_pauli (Backend.exp_value_observable_symbolic on a density
 * matrix, backends/abstract.py:2975-3054).  ``scratch``:
 * qgb_density_scratch_bytes() bytes. */
int qgb_density_expect_pauli(const void* rho, int nqubits, int dtype, const uint64_t* xmask, const uint64_t* zmask,
                             const double* coef, int nterms, double* out, void* scratch, void* stream);
/* y = a x + b y over 2^nqubits amplitudes (b = 0: y is only written): the
 * weighted sum of Backend.apply_channel (backends/abstract.py:2297-2312) for
 * channels wider than one superoperator, and the mean of the final density
 * matrices of repeated execution (:2603-2607). */
int qgb_state_axpby(void* y, const void* x, int nqubits, int dtype, double a, double b, void* stream);

/* ---- gradients: the reference has parameter shift and finite differences
 *      only (derivative.py:7-226); these implement the adjoint method ----- */
/* dst = sum_t coef[t] P_t src for Pauli strings given as qubit bit masks
 * (as qgb_expect_pauli); src and dst are distinct states of the same n.
 * At most 256 terms in at most 64 distinct X/Y patterns. */
int qgb_apply_pauli_sum(const void* src, void* dst, int nqubits, int dtype, const uint64_t* xmask,
                        const uint64_t* zmask, const double* coef, int nterms, void* stream);
/* out[0..2) (device, FP64) = <a|b> (real, imaginary); scratch of
 * qgb_inner_scratch_bytes() bytes. */
size_t qgb_inner_scratch_bytes(void);
int qgb_inner(const void* a, const void* b, int nqubits, int dtype, double* out, void* scratch, void* stream);
/* <a|b> for states of possibly different precision (complex64 results are
 * compared against complex128 ones with it: infidelity 1 - |<a|b>|^2). */
int qgb_inner_mixed(const void* a, int dtype_a, const void* b, int dtype_b, int nqubits, double* out, void* scratch,
                    void* stream);
/* Reverse sweep of the adjoint method.  On entry psi = U_L...U_1 psi_0 and
 * lam = H psi; ``ops`` lists U_L^dagger, ..., U_1^dagger (matrices in
 * ``coefs`` as for qgb_apply_circuit).  For op i with nder[i] > 0 (at most 3,
 * gates on at most 2 qubits), coefs + der_offset[i] holds nder[i] matrices
 * dU/dtheta (of U, not of U^dagger) and the derivatives are written to
 * grads[grad_index[i] + j] (device, FP64): dE/dtheta = 2 Re <lam|dU psi>.
 * Each parameter slot belongs to one op.  On return psi = psi_0.  Scratch:
 * qgb_adjoint_scratch_bytes(nparams) bytes. */
size_t qgb_adjoint_scratch_bytes(int nparams);
int qgb_adjoint_sweep(void* psi, void* lam, int nqubits, int dtype, const qgb_op* ops, int nops,
                      const double* coefs, const int* nder, const int64_t* der_offset, const int* grad_index,
                      int nparams, double* grads, void* scratch, void* stream);

/* ---- serving: many independent circuits (replaces the joblib thread pools
 *      of Backend.execute_circuits / parallel_circuits_execution,
 *      backends/abstract.py:2514-2530, parallel.py:60-121) ----------------- */
#define QGB_NOT_READY 6      /* qgb_event_query: work still in flight */
int qgb_stream_create(void** stream);  /* non-blocking stream */
int qgb_stream_destroy(void* stream);
int qgb_event_query(void* ev);         /* QGB_OK when complete, else QGB_NOT_READY */

/* A program is a planned circuit whose pass parameters and state pointer
 * live in device memory: its first qgb_program_run captures the launches as
 * a CUDA graph, later runs (any state of the same size, any stream) replay
 * it.  qgb_program_update swaps in new matrices for the same gate shape (same
 * gates on the same qubits).  A program must not run on two streams at once.
 * On the legacy default stream (NULL), which cannot be captured, the passes
 * are launched directly.  flags: QGB_PLAN_STRICT_FP64, QGB_PROGRAM_NO_GRAPH. */
#define QGB_PROGRAM_NO_GRAPH 4
int qgb_program_create(int nqubits, int dtype, const qgb_op* ops, int nops, const double* coefs, int flags,
                       void** prog);
int qgb_program_passes(void* prog, int* npasses);
int qgb_program_update(void* prog, const qgb_op* ops, int nops, const double* coefs, void* stream);
int qgb_program_run(void* prog, void* state, void* stream);
int qgb_program_destroy(void* prog);

/* Batched small circuits: one launch runs many circuits of at most 13
 * (complex64) or 12 (complex128) qubits, one CTA per circuit with the whole
 * state in shared memory, and produces each circuit's output in the same
 * kernel: the final state (written back), ``nshots`` samples from |psi|^2
 * (Philox4x32-10 keyed by ``seed``, FP64 CDF in shared memory), or the
 * expectation of a Z string (qubit mask ``zmask``).  A batch context owns a
 * device workspace and pinned staging of ``capacity`` bytes. */
#define QGB_OUT_STATE 0
#define QGB_OUT_SAMPLES 1
#define QGB_OUT_ZEXP 2
typedef struct qgb_batch_item {
    void* state;            /* device state, 2^nqubits amplitudes (in/out) */
    int32_t nqubits;
    int32_t nops;
    const qgb_op* ops;      /* host gate list, as for qgb_apply_circuit */
    const double* coefs;    /* host matrices */
    int32_t init_zero;      /* 1: start from |0...0> */
    int32_t out_kind;       /* QGB_OUT_* */
    int64_t nshots;
    uint64_t seed;
    uint64_t zmask;
    void* out;              /* device int64[nshots] or double[1]; unused for QGB_OUT_STATE */
} qgb_batch_item;
#define QGB_BATCH_MAX_QUBITS_C64 13
#define QGB_BATCH_MAX_QUBITS_C128 12
int qgb_batch_create(size_t capacity, void** ctx);
int qgb_batch_run(void* ctx, const qgb_batch_item* items, int nitems, int dtype, void* stream);
int qgb_batch_destroy(void* ctx);

/* ---- timing helpers (events on the caller's stream) ------------------- */
int qgb_event_create(void** ev);
int qgb_event_destroy(void* ev);
int qgb_event_record(void* ev, void* stream);
int qgb_event_elapsed_ms(void* start, void* stop, float* ms);

#ifdef __cplusplus
}
#endif
#endif /* QGB300_H */
