// Gate application on a window of U qubits held in registers.
//
// A window is U distinct qubits wq[0] < ... < wq[U-1]; local index bit
// (U-1-i) stands for qubit wq[i], so the window keeps the MSB order of the
// full state.  A thread owns the 2^U amplitudes of one window position
// ("group"): global index = base(r) + off[li].  Gates act on local bits; the
// local bit positions are template parameters so every register index is a
// compile-time constant, and small switch statements map the runtime
// positions onto the instantiations.
#pragma once

#include "device_common.cuh"

struct WinSpec {
  int u;           // window size
  int qubit[4];    // ascending qubit indices
  int bitpos[4];   // global bit positions n-1-qubit, same order (descending)
};

// Add `want` qubits to the window: first the given ones, then the least
// significant qubits not present (highest index), keeping it sorted.
// Returns false (window unusable) if the given qubits are more than `want`.
__device__ __forceinline__ bool win_build(WinSpec& w, int n, const int* qs, int nq, int want) {
  int cnt = 0;
  int sel[4];
  for (int i = 0; i < nq; ++i) {
    bool dup = false;
    for (int j = 0; j < cnt; ++j) dup |= sel[j] == qs[i];
    if (dup) continue;
    if (cnt >= want) return false;
    sel[cnt++] = qs[i];
  }
  for (int q = n - 1; q >= 0 && cnt < want; --q) {
    bool dup = false;
    for (int j = 0; j < cnt; ++j) dup |= sel[j] == q;
    if (!dup) sel[cnt++] = q;
  }
  // insertion sort ascending
  for (int i = 1; i < cnt; ++i) {
    int k = sel[i], j = i - 1;
    while (j >= 0 && sel[j] > k) { sel[j + 1] = sel[j]; --j; }
    sel[j + 1] = k;
  }
  w.u = cnt;
  for (int i = 0; i < 4; ++i) {
    w.qubit[i] = i < cnt ? sel[i] : 0;
    w.bitpos[i] = i < cnt ? n - 1 - sel[i] : 0;
  }
  return true;
}

// local bit of qubit q in the window
__device__ __forceinline__ int win_local(const WinSpec& w, int q) {
  for (int i = 0; i < w.u; ++i)
    if (w.qubit[i] == q) return w.u - 1 - i;
  return -1;
}

// Group base: insert a zero bit at every window bit position into r
// (positions processed in ascending order).
__device__ __forceinline__ int64_t win_base(const WinSpec& w, int64_t r) {
  int64_t x = r;
  for (int i = w.u - 1; i >= 0; --i) {   // bitpos ascending as i descends
    const int p = w.bitpos[i];
    x = ((x >> p) << (p + 1)) | (x & ((((int64_t)1) << p) - 1));
  }
  return x;
}

template <int U>
__device__ __forceinline__ void win_offsets(const WinSpec& w, int (&off)[1 << U]) {
#pragma unroll
  for (int li = 0; li < (1 << U); ++li) {
    int o = 0;
#pragma unroll
    for (int i = 0; i < U; ++i)
      if ((li >> (U - 1 - i)) & 1) o |= 1 << w.bitpos[i];
    off[li] = o;
  }
}

// index of the o-th combination of the bits other than HI and LO
template <int U, int HI, int LO>
__device__ __forceinline__ constexpr int win_other2(int o) {
  int base = 0, k = 0;
  for (int b = 0; b < U; ++b) {
    if (b == HI || b == LO) continue;
    base |= ((o >> k) & 1) << b;
    ++k;
  }
  return base;
}

template <int U, int B>
__device__ __forceinline__ constexpr int win_other1(int o) {
  int base = 0, k = 0;
  for (int b = 0; b < U; ++b) {
    if (b == B) continue;
    base |= ((o >> k) & 1) << b;
    ++k;
  }
  return base;
}

// y = G x on local bits (HI, LO); g is a row-major 4x4 (fp32 complex)
template <int U, int HI, int LO>
__device__ __forceinline__ void win_apply2_t(float2 (&a)[1 << U], const float2* g) {
#pragma unroll
  for (int o = 0; o < (1 << (U - 2)); ++o) {
    const int b = win_other2<U, HI, LO>(o);
    const int i0 = b, i1 = b | (1 << LO), i2 = b | (1 << HI), i3 = b | (1 << HI) | (1 << LO);
    const float2 x0 = a[i0], x1 = a[i1], x2 = a[i2], x3 = a[i3];
    float2 y[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      float2 acc = cf(0.f, 0.f);
      acc = fmac(acc, g[r * 4 + 0], x0);
      acc = fmac(acc, g[r * 4 + 1], x1);
      acc = fmac(acc, g[r * 4 + 2], x2);
      acc = fmac(acc, g[r * 4 + 3], x3);
      y[r] = acc;
    }
    a[i0] = y[0];
    a[i1] = y[1];
    a[i2] = y[2];
    a[i3] = y[3];
  }
}

template <int U, int B>
__device__ __forceinline__ void win_apply1_t(float2 (&a)[1 << U], const float2* g) {
#pragma unroll
  for (int o = 0; o < (1 << (U - 1)); ++o) {
    const int b = win_other1<U, B>(o);
    const int i0 = b, i1 = b | (1 << B);
    const float2 x0 = a[i0], x1 = a[i1];
    a[i0] = fmac(fmac(cf(0.f, 0.f), g[0], x0), g[1], x1);
    a[i1] = fmac(fmac(cf(0.f, 0.f), g[2], x0), g[3], x1);
  }
}

// E[r][c] += sum_other conj(t[r, other]) y[c, other] on local bits (HI, LO)
template <int U, int HI, int LO>
__device__ __forceinline__ void win_env2_t(const float2 (&t)[1 << U], const float2 (&y)[1 << U], float2 (&e)[16]) {
#pragma unroll
  for (int o = 0; o < (1 << (U - 2)); ++o) {
    const int b = win_other2<U, HI, LO>(o);
    const int idx[4] = {b, b | (1 << LO), b | (1 << HI), b | (1 << HI) | (1 << LO)};
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const float2 ct = cf(t[idx[r]].x, -t[idx[r]].y);
#pragma unroll
      for (int c = 0; c < 4; ++c) e[r * 4 + c] = fmac(e[r * 4 + c], ct, y[idx[c]]);
    }
  }
}

template <int U, int B>
__device__ __forceinline__ void win_env1_t(const float2 (&t)[1 << U], const float2 (&y)[1 << U], float2 (&e)[16]) {
#pragma unroll
  for (int o = 0; o < (1 << (U - 1)); ++o) {
    const int b = win_other1<U, B>(o);
    const int idx[2] = {b, b | (1 << B)};
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const float2 ct = cf(t[idx[r]].x, -t[idx[r]].y);
#pragma unroll
      for (int c = 0; c < 2; ++c) e[r * 2 + c] = fmac(e[r * 2 + c], ct, y[idx[c]]);
    }
  }
}

// ---- runtime dispatch (uniform over the block) ---------------------------------
template <int U>
__device__ __forceinline__ void win_apply(float2 (&a)[1 << U], const float2* g, int k, int hi, int lo) {
  if (k == 2) {
    if (U == 2) {
      win_apply2_t<U, 1, 0>(a, g);
    } else if (U == 3) {
      if (hi == 2 && lo == 1) win_apply2_t<U, 2, 1>(a, g);
      else if (hi == 1 && lo == 0) win_apply2_t<U, 1, 0>(a, g);
      else win_apply2_t<U, 2, 0>(a, g);
    } else {
      switch (hi * 4 + lo) {
        case 3 * 4 + 2: win_apply2_t<U, 3, 2>(a, g); break;
        case 3 * 4 + 1: win_apply2_t<U, 3, 1>(a, g); break;
        case 3 * 4 + 0: win_apply2_t<U, 3, 0>(a, g); break;
        case 2 * 4 + 1: win_apply2_t<U, 2, 1>(a, g); break;
        case 2 * 4 + 0: win_apply2_t<U, 2, 0>(a, g); break;
        default: win_apply2_t<U, 1, 0>(a, g); break;
      }
    }
  } else {
    switch (hi) {
      case 0: win_apply1_t<U, 0>(a, g); break;
      case 1: win_apply1_t<U, 1>(a, g); break;
      case 2: if (U > 2) win_apply1_t<U, (U > 2 ? 2 : 0)>(a, g); break;
      default: if (U > 3) win_apply1_t<U, (U > 3 ? 3 : 0)>(a, g); break;
    }
  }
}

template <int U>
__device__ __forceinline__ void win_env(const float2 (&t)[1 << U], const float2 (&y)[1 << U], float2 (&e)[16],
                                        int k, int hi, int lo) {
  if (k == 2) {
    if (U == 2) {
      win_env2_t<U, 1, 0>(t, y, e);
    } else if (U == 3) {
      if (hi == 2 && lo == 1) win_env2_t<U, 2, 1>(t, y, e);
      else if (hi == 1 && lo == 0) win_env2_t<U, 1, 0>(t, y, e);
      else win_env2_t<U, 2, 0>(t, y, e);
    } else {
      switch (hi * 4 + lo) {
        case 3 * 4 + 2: win_env2_t<U, 3, 2>(t, y, e); break;
        case 3 * 4 + 1: win_env2_t<U, 3, 1>(t, y, e); break;
        case 3 * 4 + 0: win_env2_t<U, 3, 0>(t, y, e); break;
        case 2 * 4 + 1: win_env2_t<U, 2, 1>(t, y, e); break;
        case 2 * 4 + 0: win_env2_t<U, 2, 0>(t, y, e); break;
        default: win_env2_t<U, 1, 0>(t, y, e); break;
      }
    }
  } else {
    switch (hi) {
      case 0: win_env1_t<U, 0>(t, y, e); break;
      case 1: win_env1_t<U, 1>(t, y, e); break;
      case 2: if (U > 2) win_env1_t<U, (U > 2 ? 2 : 0)>(t, y, e); break;
      default: if (U > 3) win_env1_t<U, (U > 3 ? 3 : 0)>(t, y, e); break;
    }
  }
}
