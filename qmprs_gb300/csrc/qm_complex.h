// Complex arithmetic shared by device kernels and the host-side check build.
//
// The same header compiles under nvcc (device + host) and under plain g++
// (host only), so the small dense linear algebra that decides gauges and
// gates can be checked on a CPU against the oracle before it runs on a GPU.
#pragma once

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#include <cuda_runtime.h>
#define QM_HD __host__ __device__ __forceinline__
#else
#define QM_HD inline
struct double2 { double x, y; };
struct float2 { float x, y; };
#endif

QM_HD double2 cd(double re, double im) { double2 r; r.x = re; r.y = im; return r; }
QM_HD double2 cadd(double2 a, double2 b) { return cd(a.x + b.x, a.y + b.y); }
QM_HD double2 csub(double2 a, double2 b) { return cd(a.x - b.x, a.y - b.y); }
QM_HD double2 cmul(double2 a, double2 b) { return cd(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
QM_HD double2 cconj(double2 a) { return cd(a.x, -a.y); }
// conj(a) * b
QM_HD double2 cmulc(double2 a, double2 b) { return cd(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x); }
QM_HD double2 cscale(double2 a, double s) { return cd(a.x * s, a.y * s); }
QM_HD double cnorm2(double2 a) { return a.x * a.x + a.y * a.y; }
QM_HD double cabs_(double2 a) { return hypot(a.x, a.y); }
QM_HD double2 czero() { return cd(0.0, 0.0); }

QM_HD float2 cf(float re, float im) { float2 r; r.x = re; r.y = im; return r; }
QM_HD double2 f2d(float2 a) { return cd((double)a.x, (double)a.y); }
