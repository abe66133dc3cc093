/*
 * qmprs_gb300 — C ABI of the GB300 (sm_103a) MPS-encoding library.
 *
 * The library replaces the numerical core of the reference project
 * Qualition/qmprs (pure Python over quimb/numpy) behind its own Python API
 * (qmprs_gb300.primitives.MPS, qmprs_gb300.synthesis.mps_encoding.Sequential).
 * Every entry point below names the reference function it replaces.
 *
 * Conventions
 *   - All buffers are DEVICE pointers owned by the caller unless stated;
 *     sizes and offsets come from the plan (qmprs_plan_layout).
 *   - Statevectors are complex64 (interleaved float re, im); amplitude index
 *     bit (n-1-q) is qubit q (the reference's MSB order).
 *   - Gates, MPS tensors and fidelities are complex128 / double.
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *     stream-ordered; a call returns after its work is enqueued, except where
 *     it says it synchronises.
 *   - Return value: QMPRS_OK or an error code; qmprs_last_error() gives the
 *     message.  Error classes mirror the reference's exceptions: INVALID
 *     maps to ValueError/TypeError, NONUNITARY to the ValueError raised at
 *     qmprs/primitives/mps.py:837-839.
 *   - One handle per host thread; handles hold no global state.
 */
#ifndef QMPRS_GB300_H
#define QMPRS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QMPRS_OK 0
#define QMPRS_ERR_INVALID 1
#define QMPRS_ERR_UNSUPPORTED 2
#define QMPRS_ERR_CUDA 3
#define QMPRS_ERR_NUMERIC 4
#define QMPRS_ERR_NONUNITARY 5

typedef struct qmprs_ctx* qmprs_handle_t;
typedef struct qmprs_plan* qmprs_plan_t;

/* Library version (major * 10000 + minor * 100 + patch). */
int qmprs_version(void);

/* Number of kernel launches the library has issued in this process.
 * No reference counterpart (instrumentation). */
int64_t qmprs_launch_count(void);

/*
 * Per-kernel profiling of qmprs_optimize_layers (instrumentation, no
 * reference counterpart).  When enabled, every launch of the sweep kernel
 * classes is bracketed by CUDA events on the caller's stream;
 * qmprs_plan_profile returns, for kernel 0 (group pass: apply the previous
 * group's gates and reduce the cross matrix of the next), 2 (circuit
 * rebuild) or 3 (per-group step algebra and polar updates; class 1 is
 * unused), the launches, the summed event time in ms and the algorithmic
 * bytes moved (complex64 reads and writes of the states active in each
 * launch; 0 for kernel 3).  Enabling resets the counters; profiling
 * synchronises once per sweep.
 */
int qmprs_plan_set_profiling(qmprs_plan_t p, int enable);
int qmprs_plan_profile(qmprs_plan_t p, int kernel, int64_t* launches, double* milliseconds, double* bytes);

/* Create a handle on the current CUDA device. */
int qmprs_create(qmprs_handle_t* out);
void qmprs_destroy(qmprs_handle_t h);
/* Message of the last failing call on this handle (never NULL). */
const char* qmprs_last_error(qmprs_handle_t h);

/*
 * Plan a batch of `num_states` states with the given qubit counts (host
 * array, 2 <= n <= 30), at most `max_layers` unitary layers and MPS bond
 * dimension `max_bond`.  Allocates the plan's device scratch.
 * Replaces: the per-call set-up the reference performs implicitly in
 * MPSEncoder.prepare_state (qmprs/synthesis/mps_encoding/base.py:58-106);
 * the reference encodes one state per call, the plan batches many.
 */
int qmprs_plan_create(qmprs_handle_t h, int num_states, const int* num_qubits, int max_layers,
                      int max_bond, qmprs_plan_t* out);
void qmprs_plan_destroy(qmprs_plan_t p);

/*
 * Sizes (in elements) of the caller-owned buffers and per-state offsets
 * (host arrays of num_states entries, any may be NULL):
 *   vec_elems    complex64 elements of a statevector batch
 *   gate_elems   complex128 elements of the gate store (16 per gate slot)
 *   tensor_elems complex128 elements of the MPS tensor store
 *   vec_off / gate_off / tensor_off   start of state b in those buffers
 * The arity store has gate_elems / 16 int8 entries, the bond store
 * num_states * (max_qubits + 1) int32 entries (see qmprs_plan_max_qubits).
 */
int qmprs_plan_layout(qmprs_plan_t p, int64_t* vec_elems, int64_t* gate_elems, int64_t* tensor_elems,
                      int64_t* vec_off, int64_t* gate_off, int64_t* tensor_off);
int qmprs_plan_max_qubits(qmprs_plan_t p);

/*
 * Arithmetic of a plan's stages.  QMPRS_PRECISION_FAST (the default):
 * complex64 statevector buffers, complex64 working states, split-FP16
 * tensor-core products in the sweep.  QMPRS_PRECISION_EXACT: every
 * statevector-sized caller buffer (the input of qmprs_mps_from_statevector
 * and qmprs_plan_upload, the target, the circuit state, the inputs of
 * qmprs_overlap and the vector of qmprs_apply_layer) is complex128, and the
 * working states are double-float (about 2^-46 relative), so per-layer and
 * per-sweep fidelities follow an FP64 run of the reference's algorithm to
 * about 1e-9 even through deep layer stacks, whose bond-2 truncations
 * amplify rounding by a few times per layer.  Set the precision before the
 * first stage call; gates, tensors and fidelities keep their formats.
 * Replaces: the complex128 numpy/quimb arithmetic of the reference
 * (qmprs/primitives/mps.py, qmprs/synthesis/mps_encoding/sequential.py).
 */
#define QMPRS_PRECISION_FAST 0
#define QMPRS_PRECISION_EXACT 1
int qmprs_plan_set_precision(qmprs_plan_t p, int precision);
int qmprs_plan_precision(qmprs_plan_t p);

/*
 * CUDA graphs of the layer stage (qmprs_unitary_layers) and the sweep stage
 * (qmprs_optimize_layers), on by default.  A stage's launch sequence is
 * fixed by its arguments (buffer addresses, sizes, layer and sweep counts,
 * thresholds) and, for the sweeps, by the group counts of the gates it is
 * given.  The first call with a given set runs launch by launch; the second
 * records the stage on a stream private to the plan and replays it as one
 * graph on the caller's stream, and later calls replay it.  In a graph every
 * layer and sweep is enqueued without host synchronisation: states that
 * reach the early-exit or stop fidelity are skipped on the device, so the
 * results are bit-identical to the launch-by-launch path, which stops at
 * the first layer or sweep after which no state is left.  A plan keeps at
 * most 16 graphs (oldest dropped first).  qmprs_plan_graph_stats returns
 * the graphs cached and the replays so far.
 * Replaces: the reference's per-layer and per-sweep Python loops
 * (qmprs/synthesis/mps_encoding/sequential.py:384-391, 532-539).
 */
int qmprs_plan_set_graphs(qmprs_plan_t p, int enable);
int qmprs_plan_graph_stats(qmprs_plan_t p, int* cached, int64_t* replays);

/*
 * Counters of the eigensolver for Grams wider than 128 (bonds above 64) in
 * qmprs_mps_from_statevector, summed over the plan's calls: Grams solved,
 * FP32 block-Jacobi sweeps, FP64 refinement steps, and the largest
 * first-order correction of the last step of any Gram (the error left is
 * about its square).
 * Replaces: nothing (a diagnostic of the SVD that quimb's compression runs
 * in qmprs/primitives/mps.py:242,247).
 */
int qmprs_plan_wide_stats(qmprs_plan_t p, int* grams, int* sweeps, int* refine_steps, float* last_correction);

/*
 * Autotuner of the sweep's tile passes (on by default).  The grouped sweep
 * and the circuit rebuild run grid-stride loops over chunks of 32 tiles of
 * 2^11 amplitudes; how many blocks take them decides how evenly states of
 * uneven size and group count spread over the 152 SMs.  On a batch whose
 * signature (qubit-count histogram, bond dimension, layer count) the handle
 * has not seen, the first sweeps of qmprs_optimize_layers each run one
 * candidate grid (4 blocks per SM, the resident maximum; one block per
 * chunk, balanced by the hardware scheduler; 2 blocks per SM), timed with
 * events and divided by the states active in that sweep; the fastest is
 * used for the rest of the call, by the layer stage's passes, and by every
 * later plan with the same signature on the handle.  The grid changes no
 * result (each chunk is reduced in a fixed order whichever block takes
 * it).  qmprs_plan_tuning returns the grid in use and whether it came from
 * the autotuner.
 * Replaces: nothing in the reference (its sweep runs one state on the CPU).
 */
int qmprs_plan_set_autotune(qmprs_plan_t p, int enable);
int qmprs_plan_tuning(qmprs_plan_t p, int* pass_grid, int* tuned);

/*
 * Copy a packed complex64 statevector batch (`bytes` = vec_elems * 8, from
 * host memory, ideally pinned) into the plan's own device input buffer on
 * `stream` and return that buffer in *dev_out, ready for
 * qmprs_mps_from_statevector and qmprs_overlap.  The buffer is allocated
 * once, on the first call, and reused by later calls on the same plan; it
 * lives until qmprs_plan_destroy.  Work that still reads it must be
 * ordered before the next upload.  Pinned (device-mapped) host memory is
 * read by a copy kernel on the SMs, which keeps many address translations
 * in flight over the coherent host link; other host memory goes through
 * cudaMemcpyAsync.
 * Replaces: the host-to-device move of the input the reference leaves to
 * its array library (qmprs/synthesis/mps_encoding/base.py:58-106 takes the
 * statevector as a host array).
 */
int qmprs_plan_upload(qmprs_plan_t p, const void* host, int64_t bytes, void* stream, void** dev_out);

/*
 * (a) Statevector -> MPS truncated to `max_bond` (<= the plan's), with the
 * quimb default cutoff `cutoff` (1e-10, rsum2).  Writes the site tensors
 * (l, p, r) of state b, site s at tensor_off[b] + s * 2 * chi_b^2 with
 * chi_b = min(max_bond, 2^floor(n_b/2)), the bonds, and the dense
 * statevector of the truncated MPS into `target`.
 * Replaces: MPS.from_statevector (qmprs/primitives/mps.py:219-249), i.e.
 * quimb MatrixProductState.from_dense + tensor_network_1d_compress.
 */
int qmprs_mps_from_statevector(qmprs_plan_t p, const void* sv, int max_bond, double cutoff, void* tensors,
                               int* bonds, void* target, void* stream);

/*
 * Dense statevector of an MPS held in the plan's tensor layout (site s of
 * state b at tensor_off[b] + s * 2 * chi_b^2, bonds as written by
 * qmprs_mps_from_statevector; every bond <= 1024).
 * Replaces: MPS.to_statevector (qmprs/primitives/mps.py:252-270), i.e.
 * quimb MatrixProductState.to_dense.
 */
int qmprs_mps_to_statevector(qmprs_plan_t p, const void* tensors, const int* bonds, void* out, void* stream);

/*
 * (b)+(c) Disentangling layers.  From the dense target (normalised inside),
 * generates up to `num_layers` layers: bond-2 truncation + Ran completion,
 * then the adjoint layer applied to the working state, stopping a state
 * early when |<0|psi> - 1| <= (1 - fidelity_threshold) + 1e-5.  Writes the
 * gates (generation order), their arity (1 or 2), the number of layers per
 * state and the complex zero-state overlap after each layer
 * (num_states x num_layers complex128).  Synchronises the stream.
 * Replaces: Sequential._get_unitary_layers
 * (qmprs/synthesis/mps_encoding/sequential.py:330-398) with
 * MPS.generate_bond_D_unitary_layer (qmprs/primitives/mps.py:849-891),
 * MPS.apply_unitary_layer(inverse=True) (mps.py:973-995) and
 * MPS.fidelity_with_zero_state (mps.py:1020-1039).
 */
int qmprs_unitary_layers(qmprs_plan_t p, const void* target, int num_layers, double fidelity_threshold,
                         void* gates, int8_t* arity, int* layers_out, void* layer_fid, void* stream);

/*
 * (d) Environment sweeps.  Runs up to `num_sweeps` sweeps over every gate
 * (last to first) of each state, replacing each gate by the conjugate of the
 * polar factor of its environment.  After each sweep writes
 * |<target|C|0>| / ||target|| into sweep_fid[b * num_sweeps + s]; if
 * stop_fidelity > 0 a state stops sweeping once it reaches it.
 * sweeps_done[b] receives the number of sweeps run.  Synchronises the
 * stream once per sweep when stop_fidelity > 0, otherwise at the end.
 * Replaces: Sequential._optimize_unitary_layers and _sweep_unitary_layers
 * (qmprs/synthesis/mps_encoding/sequential.py:400-541).
 */
int qmprs_optimize_layers(qmprs_plan_t p, const void* target, void* gates, const int8_t* arity,
                          const int* num_layers, int num_sweeps, double stop_fidelity, double* sweep_fid,
                          int* sweeps_done, void* stream);

/*
 * (d) Gate environments at a fixed circuit.  One backward pass over every
 * gate, as a sweep makes it but without replacing any gate: env (the gate
 * store's layout and size, complex128) receives at each gate's slot the
 * m x m environment E with <target|C|0> = sum_{a,c} G[a,c] E[a,c] for that
 * gate G; entries outside the gates are zero.  E is the derivative of the
 * circuit overlap with respect to the gate's entries, which trains the
 * learned warm start on circuit fidelity.  Fast precision only
 * (QMPRS_ERR_INVALID for an exact plan).  Synchronises the stream.
 * Replaces: the environment contraction of
 * Sequential._sweep_unitary_layers (qmprs/synthesis/mps_encoding/
 * sequential.py:463-477) with the update left out.
 */
int qmprs_layer_environments(qmprs_plan_t p, const void* target, const void* gates, const int8_t* arity,
                             const int* num_layers, void* env, void* stream);

/*
 * Dense circuit state C|0...0> of the stored layers (circuit order = reverse
 * generation order).
 * Replaces: Sequential._tensor_network_from_unitary_layers(...).to_dense()
 * (qmprs/synthesis/mps_encoding/sequential.py:216-292, 443-447) and the
 * statevector of the emitted circuit.
 */
int qmprs_circuit_state(qmprs_plan_t p, const void* gates, const int8_t* arity, const int* num_layers,
                        void* out, void* stream);

/*
 * Per-state inner products <a|b> (complex128 out[num_states]) in fp64.
 * Replaces: the np.dot(conj(sv), sv') fidelity of the reference tests
 * (tests/synthesis/mps_encoding/test_sequential_encoding.py:67).
 */
int qmprs_overlap(qmprs_plan_t p, const void* a, const void* b, void* out, void* stream);

/*
 * Per-state inner products <a|b> like qmprs_overlap, for callers that
 * cannot allocate device memory (their GPU memory belongs to another
 * allocator, or cudaMalloc's implicit synchronisation is not acceptable on
 * their stream).  No plan and no cudaMalloc/cudaFree: the states are packed
 * back to back (state i of 2^num_qubits[i] complex64 amplitudes, host array
 * num_qubits), out is a device complex128[num_states], and the reduction
 * scratch is a 1 MiB static device array inside the library.  Limits: at most
 * QMPRS_NOALLOC_MAX_STATES states and QMPRS_NOALLOC_MAX_TILES tiles of 4096
 * amplitudes in total (2^25 amplitudes); larger requests return
 * QMPRS_ERR_UNSUPPORTED.  The first call on a device looks up the scratch
 * address (make it before any stream capture); calls share the scratch, so
 * calls that overlap on the GPU race and must be serialised by the caller.
 * A CUDA error already pending on the calling thread is left in place and
 * the call returns QMPRS_ERR_CUDA without launching.
 * No counterpart in the reference (which has no device code).
 */
#define QMPRS_NOALLOC_MAX_STATES 64
#define QMPRS_NOALLOC_MAX_TILES 8192
int qmprs_overlap_noalloc(const void* a, const void* b, int num_states, const int* num_qubits, void* out,
                          void* stream);

/*
 * Apply the adjoint (inverse != 0) or the gate itself of one generated layer
 * to a statevector batch, in the reference's order.
 * Replaces: MPS.apply_unitary_layer (qmprs/primitives/mps.py:893-995).
 */
int qmprs_apply_layer(qmprs_plan_t p, void* vec, const void* gates, const int8_t* arity, int layer,
                      int inverse, void* stream);

/*
 * Learned warm start (no reference counterpart: the reference initialises
 * the layers analytically only).  Building blocks of the BF16 multilayer
 * perceptron that predicts a block's converged gate from its analytic
 * initial gate; qmprs_gb300.warmstart composes them into training and
 * inference.  All matrices are row-major device buffers.
 *
 * qmprs_gemm_bf16: C = A B^T on the tensor cores (tcgen05.mma, BF16
 * operands, FP32 accumulation in tensor memory).  A is M x K (leading
 * dimension lda), B is N x K (ldb); M a multiple of 128, N a multiple of 16
 * in [16, 256], K a multiple of 16, lda and ldb multiples of 8, A and B
 * 16-byte aligned.  ksplit < K splits K over blocks (multiple of 16), which
 * needs `part` (ceil(K / ksplit) * M * N floats) and reduces in fixed order.
 * Epilogue: z = C + bias + resid (bias [N] and resid [M x ldr], fp32, may
 * be NULL); Cf (fp32, ldc) receives z; Cb (bf16, ldc) and CbT (bf16,
 * N x ldt, transposed) receive act(z), act 0 = identity, 1 = GELU (tanh
 * form).  Any output may be NULL.  `err` is a device int; bit 16 is raised
 * if a tensor-core completion wait ran out.
 */
int qmprs_gemm_bf16(const void* A, int lda, const void* B, int ldb, int M, int N, int K, int ksplit,
                    const float* bias, const float* resid, int ldr, int act, float* Cf, int ldc, void* Cb,
                    void* CbT, int ldt, float* part, int* err, void* stream);

/*
 * Gate loss of a batch of B predictions: Y and U are B x 32 floats (4 x 4
 * complex, row-major, interleaved re/im), w the per-sample weights.
 * loss[s] = w[s] min_phi |Y_s - e^{i phi} U_s|_F^2; dY = d(sum loss) / dY
 * scaled by inv_wsum, also as bf16 (B x 32) and transposed bf16 (32 x ldt).
 */
int qmprs_mlp_loss(const float* Y, const float* U, const float* w, int B, float inv_wsum, float* loss, float* dY,
                   void* dYb, void* dYT, int ldt, void* stream);

/* dZ = dH * GELU'(Z) for B x N; also bf16 and transposed bf16 (N x ldt). */
int qmprs_mlp_act_back(const float* dH, const float* Z, int B, int N, float* dZ, void* dZb, void* dZT, int ldt,
                       void* stream);

/* out[c] = sum over the B rows of X[r][c] (B x N), fixed order. */
int qmprs_mlp_col_sum(const float* X, int B, int N, float* out, void* stream);

/*
 * One Adam step (bias-corrected, step >= 1, decoupled weight decay wd) on
 * fp32 master weights W (rows x cols) with gradient G (the same layout, or
 * cols x rows when gT != 0); refreshes the bf16 copies Wb (rows x cols) and
 * WTb (cols x rows) when given.
 */
int qmprs_mlp_adam(float* W, const float* G, int gT, float* m, float* v, int rows, int cols, float lr, float b1,
                   float b2, float eps, int step, float wd, void* Wb, void* WTb, void* stream);

/*
 * Test of the bounded tensor-core completion wait of qmprs_gemm_bf16: one
 * block allocates tensor memory and waits on an mbarrier at which nothing
 * will arrive.  After its limit (about one second of wall time) the wait
 * gives up, bit 16 of `err` (a device int) is raised and the tensor memory
 * is freed, as qmprs_gemm_bf16 does after a timeout; the context stays
 * usable.  No reference counterpart (error handling of this library).
 */
int qmprs_tc_wait_selftest(int* err, void* stream);

/*
 * Circuit-overlap loss of the warm start.  For rows r < rows: slots[r] and
 * kind[r] as in qmprs_mlp_project; `gates` holds the projected outputs and
 * `env` their environments from qmprs_layer_environments (both complex128,
 * the gate store's layout).  fid[r] = |f|^2 tinv[r] with
 * f = sum_ac U[a,c] E[a,c] the state's circuit overlap (tinv[r] =
 * 1 / <t|t> of the row's state).  dY (B x 32 fp32, also bf16 and
 * transposed bf16 32 x ldt) = the gradient of -gscale fid[r] with respect
 * to the network output, through the tangent map of the polar factor at U;
 * rows rows..B-1 get zero gradient.  No reference counterpart (the
 * reference has no learned part).
 */
int qmprs_mlp_overlap_grad(const void* env, const void* gates, const int64_t* slots, const int8_t* kind,
                           const float* tinv, int rows, int B, float gscale, float* fid, float* dY, void* dYb,
                           void* dYT, int ldt, void* stream);

/*
 * Project network outputs to gates: row r of Y (4 x 4 complex, interleaved
 * fp32; for kind[r] == 1 the 2 x 2 in its first four entries) becomes its
 * unitary polar factor, written to the complex128 gate slot slots[r] (units
 * of 16 entries) of `gates`; singular directions below 1e-6 of the largest
 * are completed towards the gate already in the slot.  Rows with non-finite
 * entries leave the slot unchanged.
 */
int qmprs_mlp_project(const float* Y, int rows, const int64_t* slots, const int8_t* kind, void* gates,
                      void* stream);

#ifdef __cplusplus
}
#endif

#endif /* QMPRS_GB300_H */
