// Shared-memory tile layout of the pass kernels: the swizzle, the bit
// deposits, and the rest / position orders that keep the tensor-core
// fragment loads on distinct banks.  Plain integer functions, compiled into
// the CUDA library and into the host check build, so their bijectivity and
// bank properties are tested on a CPU.
#pragma once

#include "qm_complex.h"

#if defined(__CUDA_ARCH__)
#define QM_FFS(x) __ffs(x)
#else
#define QM_FFS(x) __builtin_ffs(x)
#endif

// Shared-memory swizzle of a tile index: the low four bits (the float2
// slot within a 128-byte bank row) are XORed with bits 4-7 and 8-11, so
// that warps walking low, middle or high tile bits hit distinct banks.  The
// map is linear over XOR, so for disjoint bit sets swz(a | b) =
// swz(a) ^ swz(b) and the offset tables hold swizzled values.
QM_HD int swz(int li) { return li ^ (((li >> 4) ^ (li >> 8)) & 15); }

// Place the low bits of v, in order, at the set bits of mask (ascending).
QM_HD int deposit32(int v, int mask) {
  int r = 0;
  while (mask) {
    const int bit = mask & (-mask);
    if (v & 1) r |= bit;
    v >>= 1;
    mask ^= bit;
  }
  return r;
}

// bank residue (one-hot) of a single-bit mask; 0 for no bit
QM_HD int bank_res(int bit) { return bit ? 1 << ((QM_FFS(bit) - 1) & 3) : 0; }

// lowest bit of `left` whose residue is not in `avoid`, else the lowest bit
QM_HD int pick_res(int left, int avoid) {
  for (int m = left; m; m &= m - 1) {
    const int bit = QM_FFS(m) - 1;
    if (!((avoid >> (bit & 3)) & 1)) return 1 << bit;
  }
  return left & (-left);
}

// the i-th lowest set bit of a mask (0 when it has fewer bits)
QM_HD int nth_bit(int mask, int i) {
  for (int k = 0; k < i && mask; ++k) mask &= mask - 1;
  return mask & (-mask);
}

// Tile offset of rest index r for the tensor-core cross matrix.  A
// half-warp's fragment loads cover window entries 0-3 (window bits 0-1)
// times rest indices 2t (rest bits 1-2), so rest bits 1 and 2 take tile
// bits whose bank residues (bit position mod 4: the swizzle folds tile bits
// 4-7 and 8-11 onto 0-3) differ from each other and from those of window
// bits 0-1; the other rest bits follow in ascending order.  The reduction
// over rests does not depend on their order.  Needs at least three rest
// bits (T >= 8 with 4-qubit windows).
QM_HD int rest_offset(int r, int wmask, int rmask) {
  const int cov = bank_res(nth_bit(wmask, 0)) | bank_res(nth_bit(wmask, 1));
  int left = rmask;
  const int b1 = pick_res(left, cov);
  left &= ~b1;
  const int b2 = pick_res(left, cov | bank_res(b1));
  left &= ~b2;
  const int b0 = left & (-left);
  left &= ~b0;
  return ((r & 1) ? b0 : 0) | ((r & 2) ? b1 : 0) | ((r & 4) ? b2 : 0) | deposit32(r >> 3, left);
}

// Tile offset of window position p for the tensor-core gate application.
// Its loads put window bits 1-2 and position bits 0-1 on a half-warp, its
// stores window bits 0-1 and position bits 1-2; positions bits 0-2 take
// residues distinct from those, where the tile has them.  Needs at least
// three position bits.
QM_HD int apply_pos_offset(int p, int wmask, int rmask) {
  const int r0 = bank_res(nth_bit(wmask, 0)), r1 = bank_res(nth_bit(wmask, 1)), r2 = bank_res(nth_bit(wmask, 2));
  int left = rmask;
  const int p1 = pick_res(left, r0 | r1 | r2);
  left &= ~p1;
  const int p0 = pick_res(left, r1 | r2 | bank_res(p1));
  left &= ~p0;
  const int p2 = pick_res(left, r0 | r1 | bank_res(p1));
  left &= ~p2;
  return ((p & 1) ? p0 : 0) | ((p & 2) ? p1 : 0) | ((p & 4) ? p2 : 0) | deposit32(p >> 3, left);
}

// Tensor-core scale of a state vector with 2^n amplitudes and norm `nrm`:
// 2^k with 2^k nrm <= 2^min(n/2 + 4, 15), so every |v s| <= 2^15 (below
// the FP16 maximum 65504) and typical amplitudes (nrm 2^-n/2) land near 16,
// where the low half of the FP16 split is a normal number.
QM_HD float vec_scale(int n, double nrm) {
  int e = 0;
  frexp(nrm, &e);   // nrm < 2^e
  const int top = n / 2 + 4 < 15 ? n / 2 + 4 : 15;
  return ldexpf(1.f, top - e);
}
