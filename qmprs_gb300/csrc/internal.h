// Internal declarations of the qmprs_gb300 CUDA library.
//
// Layout in HBM (all caller buffers are contiguous):
//   vectors  complex64, state b occupies [vec_off[b], vec_off[b] + 2^n_b);
//            amplitude index bit (n-1-q) is qubit q (MSB order, the
//            reference's convention).
//   gates    complex128, state b, generated layer l, site s at
//            gate_off[b] + (l * n_b + s) * 16; a two-qubit gate is a
//            row-major 4x4 (rows = outputs), a one-qubit gate uses the first
//            four entries as a row-major 2x2.  Layers are stored in the order
//            they are generated; the circuit applies them in reverse.
//   arity    int8, same indexing as gates without the factor 16 (1 or 2).
//   tensors  complex128 MPS site tensors (l, p, r), site s of state b at
//            tensor_off[b] + s * 2 * chi * chi.
//   bonds    int32, state b at b * (max_n + 1): bonds[c] is the bond between
//            sites c-1 and c, bonds[0] = bonds[n] = 1.
//
// Work decomposition: every state is cut into tiles of 2^tile_bits
// amplitudes (one tile if the state is smaller); the plan picks tile_bits in
// [TILE_BITS_MIN, TILE_BITS_MAX] so that the batch has about 16 tiles per SM.
// A launch runs a grid-stride loop over the tiles of all states of the
// batch, so states of uneven size share one launch.  Per-state reductions
// write one fp64 partial per warp of each tile; a second kernel (one block
// or warp per state) sums them in a fixed order, which keeps every result
// deterministic.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "qm_complex.h"

#define TILE_BITS_MIN 12
#define TILE_BITS_MAX 17
#define WARPS_PER_BLOCK 8   // BLOCK_THREADS / 32; per-warp partials per tile
#define BLOCK_THREADS 256
#define MAX_QUBITS 30
#define TT_MAXW 128   // widest Gram of stage (a)'s one-block kernels: 2 * bond
#define TT_MAXB 64    // largest bond of stage (a)'s one-block kernels (wider: ttsvd_wide.cu)
#define TT_WIDE_MAXB 1024   // largest bond of stage (a) overall

enum {
  QM_OK = 0,
  QM_ERR_INVALID = 1,
  QM_ERR_UNSUPPORTED = 2,
  QM_ERR_CUDA = 3,
  QM_ERR_NUMERIC = 4,
  QM_ERR_NONUNITARY = 5,
};

// error flags raised by kernels (bit mask in dev_err)
enum {
  KERR_NONUNITARY = 1,
  KERR_EIG_WIDTH = 2,
  KERR_NONFINITE = 4,
  KERR_BAD_GATE = 8,
  KERR_TC_TIMEOUT = 16,   // a tensor-core completion wait ran out
  KERR_BAD_INPUT = 32,    // an input statevector has a non-finite or zero norm
};

struct BatchDev {
  int B;
  int ntiles;
  int max_n;
  const int* n;            // [B] qubits
  const int64_t* vec_off;  // [B]
  const int64_t* gate_off; // [B]
  const int64_t* tensor_off;  // [B]
  const int* tile_state;   // [ntiles]
  const int* tile_idx;     // [ntiles] tile index within its state
  const int* state_tile0;  // [B]
  const int* state_ntiles; // [B]
  int* ticket;             // [B] last-tile tickets (kept at zero between launches)
  int* err;                // [1] error flag bits
  int tt_w;                // stage (a): Gram stride (>= TT_MAXW, 2 x the largest bond)
  int tt_b;                // stage (a): largest bond / selected-column stride (>= TT_MAXB)
  int eig_wmax;            // stage (a): widest Gram of the one-block eigensolver; wider ones
                           // take the blocked solver (ttsvd_wide.cu)
};
// Batches of at most this many states send Grams wider than 64 to the
// blocked multi-SM solver: one block per state would leave the GPU idle
#define BJ_SMALL_BATCH 8

// Gate selection modes for the per-step gate launches.
enum {
  SEL_REBUILD = 0,   // forward circuit order, gate j of C (circuit state)
  SEL_SWEEP = 1,     // backward circuit order, gate j from the end
  SEL_INVERSE = 2,   // adjoint of generated layer `layer`, sites n-1 .. 0
  SEL_LAYER_FWD = 3, // generated layer `layer` itself, sites 0 .. n-1
};

struct GateSel {
  int mode;
  int step;             // j
  int layer;            // for SEL_INVERSE
  int adjoint;          // apply G^H instead of G
  const double2* gates;
  const signed char* arity;
  const int* nlayers;   // [B] generated layers per state
  const int* active;    // [B] state participates (may be null)
};

// Grouped backward sweep (sweep_group.cu): a group is a run of consecutive
// backward steps whose qubits fit a window of GW qubits; one pass over the
// vectors per group, shared-memory tiles of 2^GT amplitudes, one partial
// cross matrix per chunk of GCHUNK tiles.
#define GW 4
#define GM (1 << GW)
#define GMM (GM * GM)
#define GT 11
#define GCHUNK 32
#define GMAXSTEPS 8
#define PASS_GRID_DEFAULT (4 * 152)   // resident blocks of the tile passes (4 per SM)

struct GroupEnt {
  int j0;     // first backward step
  int cnt;    // steps in the group
  int qmask;  // window qubits (bit q = qubit q), exactly u of them
  int u;      // window size min(GW, n)
};

struct GroupDev {
  int nchunks;
  int gmax;                  // group slots per state (max_layers * max_n)
  const int* chunk_state;    // [nchunks]
  const int* chunk_idx;      // [nchunks] chunk index within its state
  const int* state_chunk0;   // [B]
  const int* state_nchunks;  // [B]
  GroupEnt* grp;             // [B * gmax]
  int* ngroups;              // [B]
  double2* old_gates;        // [B * GMAXSTEPS * 16] gates replaced by the last group
  double2* partials;         // [nchunks * GMM]
  GroupEnt* rgrp;            // [B * gmax] forward-order groups (circuit rebuild)
  int* nrgroups;             // [B]
  int grid;                  // blocks of the tile-pass launches (0: min(nchunks, 4 per SM)); set by the autotuner
};

// ---- launches (defined in the .cu files) ---------------------------------
void launch_set_zero_state(const BatchDev& bd, float2* vec, const int* active, cudaStream_t s);
void launch_apply_gate(const BatchDev& bd, float2* vec, const GateSel& sel, cudaStream_t s);
void launch_upload(void* dst, const void* src_dev, int64_t bytes, cudaStream_t s);
void launch_overlap(const BatchDev& bd, const float2* a, const float2* b, double2* partials,
                    double2* out, cudaStream_t s);
// out[b] = sum of one partial per tile of state b (fixed order)
void launch_reduce_tiles(const BatchDev& bd, const double2* partials, double2* out, cudaStream_t s);
void launch_copy_normalize(const BatchDev& bd, const float2* src, float2* dst, double2* partials,
                           double2* sq_norms, cudaStream_t s);

// (b) layer generation
void launch_layer_gram(const BatchDev& bd, int step, const float2* work, const float2* src,
                       const int* bonds, double2* partials, double2* vsel, int* bonds_out,
                       double2* site_t, const int* active, cudaStream_t s);
void launch_layer_eig(const BatchDev& bd, int step, const double2* partials, double2* vsel, int* bonds,
                      double2* site_t, const int* active, cudaStream_t s);
void launch_layer_project(const BatchDev& bd, int step, const float2* work, const float2* src,
                          float2* dst, const int* bonds, const double2* vsel, const int* active,
                          cudaStream_t s);
void launch_layer_build(const BatchDev& bd, int layer, const float2* rem0, const float2* rem1,
                        const int* bonds, double2* site_t, double2* gates, signed char* arity,
                        const int* active, cudaStream_t s);
void launch_layer_fidelity(const BatchDev& bd, int layer, const float2* work, int num_layers,
                           double atol, double2* layer_fid, int* nlayers, int* active,
                           cudaStream_t s);

// (d) sweep
void launch_group_plan(const BatchDev& bd, const GroupDev& gd, const signed char* arity, const int* nlayers,
                       cudaStream_t s);
// step orders of the group plan and the tile passes
enum { ORDER_BWD = 0, ORDER_FWD = 1, ORDER_LAYER_INV = 2, ORDER_LAYER_FWD = 3 };
void launch_rebuild_pass(const BatchDev& bd, const GroupDev& gd, int pass, float2* psi, const double2* gates,
                         const signed char* arity, const int* nlayers, const int* active, cudaStream_t s,
                         int mode = ORDER_FWD, int layer = 0, bool exact = false);
void launch_layer_plan(const BatchDev& bd, const GroupDev& gd, const signed char* arity, int mode, int layer,
                       const int* active, cudaStream_t s);
int layer_pass_bound(int max_n);
// znorm: per-state <z|z> (x has unit norm), for the tensor-core scales
int launch_group_pass(const BatchDev& bd, const GroupDev& gd, int g, float2* psi, const float2* z_in, float2* z_out,
                      const double2* gates, const signed char* arity, const int* nlayers, const int* active,
                      const double2* znorm, cudaStream_t s);
// env_out: write each gate's environment there (gate-store layout) and
// leave the gates unchanged (one pass at a fixed circuit)
void launch_group_polar(const BatchDev& bd, const GroupDev& gd, int g, double2* gates, const signed char* arity,
                        const int* nlayers, const int* active, double* nuc, cudaStream_t s,
                        double2* env_out = nullptr);
void launch_sweep_finish(int B, int sweep, int num_sweeps, const double* nuc, const double2* tnorm2,
                         double* sweep_fid, int* sweeps_done, int* active, double stop_fid,
                         int* num_active, cudaStream_t s);

// (a) statevector -> MPS
void launch_tt_gram(const BatchDev& bd, int step, const float2* sv, const float2* src, const int* bonds,
                    double2* partials, double2* gram, cudaStream_t s);
void launch_tt_eig(const BatchDev& bd, int step, int* bonds, double2* gram, double2* vwork, int max_bond,
                   double cutoff, double2* vsel, double2* tensors, int chi, double2* scratch, double fine,
                   cudaStream_t s);
void launch_tt_project(const BatchDev& bd, int step, const float2* sv, const float2* src, float2* dst,
                       const int* bonds, const double2* vsel, cudaStream_t s);
void launch_tt_site0(const BatchDev& bd, const float2* rem0, const float2* rem1, const int* bonds,
                     double2* tensors, int chi, const double2* in_sq, cudaStream_t s);
// Scratch of the blocked eigensolver for Grams wider than TT_MAXW (one
// state at a time): FP32 matrix and eigenvectors (W x W, W = width rounded
// up to 32), the subproblem rotations, the FP64 basis X, the input of a
// deflated subproblem H, two FP64 work matrices, the conjugate transpose
// of a remainder for the row-Gram path, and the refinement
// products [H X_K | X_K] and [S | X^H X_K] (n x 2K).
struct BJScratch {
  int W = 0, kmax = 0;
  float2 *A = nullptr, *V = nullptr, *J = nullptr;
  double2 *X = nullptr, *H = nullptr, *T = nullptr, *T2 = nullptr, *Mt = nullptr, *YX = nullptr, *SR = nullptr;
  int *perm = nullptr, *order = nullptr, *count = nullptr;
  double *lamA = nullptr, *lamK = nullptr, *lsort = nullptr, *stats = nullptr, *part = nullptr;
  unsigned* emax = nullptr;
};
// refinement tolerance on max |E| (the error after a step is about its
// square): exact mode to FP64 level, fast mode to about 1e-8
#define BJ_TOL_EXACT 1e-7
#define BJ_TOL_FAST 1e-4
// eigenvalues above this fraction of the largest count as resolved by the
// FP32 sweeps; the rest form the deflated subproblem when it holds columns
// that may be kept
#define BJ_RESOLVED 1e-5
struct BJStats {
  int calls = 0, sweeps = 0, refine_steps = 0;
  float last_emax = 0.f;
};
int bj_alloc(BJScratch& sc, int tt_w, int tt_b);
void bj_free(BJScratch& sc);
// Diagonalise stage (a)'s Gram of state b at cut c and emit the cut: the
// w x w column Gram already in `gram`, or, with rowsrc (the 2^c x w
// complex64 remainder, 2^c < w), the row Gram M M^H built here, whose kept
// right singular vectors are M^H U Sigma^-1.
int tt_block_eig(const BatchDev& bd, int b, int c, int w, double2* gram, const float2* rowsrc,
                 BJScratch& sc, BJScratch& sub, int* bonds, double2* vsel, double2* tensors, int chi, int max_bond,
                 double cutoff, double refine_tol, cudaStream_t s, BJStats* st);
void launch_cgemm(const float2* A, int64_t lda, const double2* B, int64_t ldb, float2* C, int64_t ldc, int64_t M,
                  int N, int K, cudaStream_t s);
void launch_mps_contract(const BatchDev& bd, int step, const double2* tensors, const int* bonds, int chi,
                         const float2* src, float2* dst_buf, float2* target, cudaStream_t s);

// every sweep of a batch of states of at most SWEEP_FUSED_MAXN qubits in one
// launch (sweep_fused.cu): one block per state, psi and t in shared memory
#define SWEEP_FUSED_MAXN 13
int launch_sweep_fused(const BatchDev& bd, int max_n, const float2* target, double2* gates, const signed char* arity,
                       const int* nlayers, int* active, const double2* tnorm2, int num_sweeps, double stop_fid,
                       double* sweep_fid, int* sweeps_done, cudaStream_t s, double2* env_out = nullptr);

// misc
void qm_note_launch();   // counts every kernel launch the library issues
void launch_fill_int(int* p, int64_t count, int value, cudaStream_t s);
void launch_count_active(int B, const int* active, int* num_active, cudaStream_t s);
// raise KERR_BAD_INPUT unless every sq[b].x is finite and positive
void launch_check_norms(int B, const double2* sq, int* err, cudaStream_t s);

#define TT_SPLIT 8

// helpers
__host__ __device__ inline int64_t ipow2(int k) { return (int64_t)1 << k; }
