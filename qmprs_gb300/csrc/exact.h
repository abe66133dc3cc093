// Launchers of the exact precision mode (exact.cu): double-float working
// states, one float4 (re hi, im hi, re lo, im lo) per complex amplitude.
#pragma once

#include <algorithm>

#include "internal.h"

typedef float4 xc;

void launch_x_from_d(const BatchDev& bd, const double2* src, xc* dst, cudaStream_t s);
void launch_x_to_d(const BatchDev& bd, const xc* src, double2* dst, cudaStream_t s);
void launch_x_copy(const BatchDev& bd, const xc* src, xc* dst, const int* active, cudaStream_t s);
void launch_x_zero(const BatchDev& bd, xc* vec, const int* active, cudaStream_t s);
// per-state <a|b> (complex128 out[B]) of double-float / complex128 vectors
void launch_x_dot(const BatchDev& bd, const xc* a, const xc* b, double2* partials, double2* out, cudaStream_t s);
void launch_d_dot(const BatchDev& bd, const double2* a, const double2* b, double2* partials, double2* out,
                  cudaStream_t s);
// dst = src / ||src||, sq[b].x = ||src||^2
void launch_x_normalize(const BatchDev& bd, const xc* src, xc* dst, double2* partials, double2* sq, cudaStream_t s);

// stage (a), one state at a time: Gram of a rows x w remainder into gram
// (row-major, stride w), through `part` (TT_SPLIT x WW complex128 partials)
void launch_x_gram(const xc* m, int64_t rows, int w, double2* part, int64_t WW, double2* gram, cudaStream_t s);
// C = A B (A double-float M x K, B complex128 K x N, C double-float M x N)
void launch_x_gemm(const xc* A, int64_t lda, const double2* B, int64_t ldb, xc* C, int64_t ldc, int64_t M, int N,
                   int K, cudaStream_t s);
void launch_x_site0(const xc* rem, int r1, double in_sq, double2* t0, double* f_out, cudaStream_t s);
void launch_x_scale_flat(const xc* src, xc* dst, int64_t count, const double* f, cudaStream_t s);
void launch_x_from_d_flat(const double2* src, xc* dst, int64_t count, cudaStream_t s);

// (b) layer stage (the FP64 eigen kernel is launch_layer_eig)
void launch_x_layer_gram(const BatchDev& bd, int step, const xc* work, const xc* src, const int* bonds,
                         double2* partials, const int* active, cudaStream_t s);
void launch_x_layer_project(const BatchDev& bd, int step, const xc* work, const xc* src, xc* dst, const int* bonds,
                            const double2* vsel, const int* active, cudaStream_t s);
void launch_x_layer_build(const BatchDev& bd, int layer, const xc* rem0, const xc* rem1, const int* bonds,
                          double2* site_t, double2* gates, signed char* arity, const int* active, cudaStream_t s);
void launch_x_layer_fidelity(const BatchDev& bd, int layer, const xc* work, int num_layers, double atol,
                             double2* layer_fid, int* nlayers, int* active, cudaStream_t s);

// (c)/(d) gates and sweeps
void launch_x_apply_gate(const BatchDev& bd, xc* vec, const GateSel& sel, cudaStream_t s);
// every sweep of every state in one launch, one block per state (states of
// at most X_FUSED_MAXN qubits: psi and t in shared memory)
#define X_FUSED_MAXN 12
int launch_x_sweep_fused(const BatchDev& bd, int max_n, const xc* target, double2* gates, const signed char* arity,
                         const int* nlayers, int* active, const double2* tnorm2, int num_sweeps, double stop_fid,
                         double* sweep_fid, int* sweeps_done, cudaStream_t s);
void launch_x_sweep_step(const BatchDev& bd, int step, xc* psi, const xc* t, double2* gates, const signed char* arity,
                         const int* nlayers, const int* active, double2* partials, double* nuc, cudaStream_t s);
