// Gate application kernels: dense k-qubit operators (k <= 12) on batches of
// states, the per-qubit loop of apply_all_qubits, and apply_phase.
//
// unitair applies a gate as permute -> contiguous copy -> einsum -> permute
// -> contiguous copy (src/unitair/simulation/operations.py:151-186, :322),
// three read+write passes over the state.  Here one kernel reads each
// amplitude once and writes it once: the amplitudes a gate mixes are found
// by inserting zero bits at the target positions of a compressed index
// ("bit insertion"), so no permuted copy is ever made.
//
// Work unit of the chunked kernel: a "chunk" is V consecutive amplitudes
// (32 bytes: V = 4 for complex64, 2 for complex128) so every load and store
// is a full 32-byte sector issued as 16-byte vectors.  Target qubits whose
// bit position is >= log2(V) ("high" targets) select which chunks a thread
// loads together (2 for one high target, 4 for two); targets below log2(V)
// ("low" targets) pair amplitudes inside a chunk, in registers.
//
// complex128 with one operator for every state (n >= 7) runs in
// dense_c128_stream_kernel instead: warp steps of 128 amplitudes streamed
// through shared memory, with the arithmetic in double-float pairs
// (dfloat.cuh); the chunked kernel keeps complex128 per-state operators,
// small states and unaligned views.
#include <stdio.h>

#include <algorithm>
#include <atomic>

#include "common.cuh"
#include "dfloat.cuh"

namespace gbsv {

struct DenseArgs {
  uint64_t total_units;  // num_states << log_units
  int log_units;         // log2(units per state)
  int n;                 // qubits per state
  int64_t in_stride;     // amplitudes between input states (0 = broadcast)
  int64_t op_stride;     // complex elements between operators (0 = shared)
  int nins;              // number of high targets (zero bits to insert)
  int ins_pos[2];        // their bit positions, ascending
  int64_t hstride[2];    // amplitude offset selected by chunk bit 0 / 1
  int log_v;             // log2(V)
  int df;                // complex128: double-float pairs (1) or FP64 (0)
};

template <typename C, int NR, int K, int RB0, int RB1>
__device__ __forceinline__ void apply_regs(C* r, const C* m) {
  if constexpr (K == 1) {
#pragma unroll
    for (int i = 0; i < NR; ++i) {
      if ((i >> RB0) & 1) continue;
      const int i1 = i | (1 << RB0);
      C a0 = r[i], a1 = r[i1];
      C o0 = cmad(m[1], a1, cmul(m[0], a0));
      C o1 = cmad(m[3], a1, cmul(m[2], a0));
      r[i] = o0;
      r[i1] = o1;
    }
  } else {
    constexpr int M0 = 1 << RB0, M1 = 1 << RB1;
#pragma unroll
    for (int i = 0; i < NR; ++i) {
      if (i & (M0 | M1)) continue;
      const int idx[4] = {i, i | M1, i | M0, i | M0 | M1};
      C v[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) v[j] = r[idx[j]];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        C acc = cmul(m[4 * j], v[0]);
        acc = cmad(m[4 * j + 1], v[1], acc);
        acc = cmad(m[4 * j + 2], v[2], acc);
        acc = cmad(m[4 * j + 3], v[3], acc);
        r[idx[j]] = acc;
      }
    }
  }
}

// complex128: GB300 issues FP64 at about 1/64 of its FP32 rate, so a gate
// whose 2x2 update runs in FP64 is bound by the FP64 pipe, not by HBM.
// The kernel therefore (1) finds the shared operator's structure once per
// block (warp 0 classifies the entries from their bit patterns and splits
// them into exact float triples in shared memory), (2) runs each kind's own
// loop, so permutations and the entries 0, +-1, +-i cost no arithmetic at
// all, and (3) does the remaining arithmetic in double-float pairs on the
// FP32 pipe (dfloat.cuh), with native FP64 kept for threads whose
// amplitudes lie outside the pair range, for per-state operators, and for
// the whole engine when gbsv_set_c128_arith selects it.
constexpr int EC_ZERO = 0, EC_ONE = 1, EC_MONE = 2, EC_I = 3, EC_MI = 4,
              EC_REAL = 5, EC_IMAG = 6, EC_FULL = 7;
// classes up to EC_MI need no arithmetic
__device__ __forceinline__ bool ec_real(int c) {
  return c <= EC_MONE || c == EC_REAL;
}
__device__ __forceinline__ bool ec_imag(int c) {
  return c == EC_I || c == EC_MI || c == EC_IMAG;
}

// From the bit patterns (integer compares: an FP64 compare costs an FP64
// issue slot; +0 and -0 are both zero)
template <typename C>
__device__ __forceinline__ int entry_class(const C& m) {
  constexpr unsigned long long P1 = 0x3FF0000000000000ull;  // +1.0
  constexpr unsigned long long M1 = 0xBFF0000000000000ull;  // -1.0
  const unsigned long long xb = __double_as_longlong(m.x);
  const unsigned long long yb = __double_as_longlong(m.y);
  const bool xz = (xb << 1) == 0, yz = (yb << 1) == 0;
  if (yz)
    return xz ? EC_ZERO : xb == P1 ? EC_ONE : xb == M1 ? EC_MONE : EC_REAL;
  if (xz) return yb == P1 ? EC_I : yb == M1 ? EC_MI : EC_IMAG;
  return EC_FULL;
}

// -x by flipping the sign bit (an integer operation)
__device__ __forceinline__ double dneg(double x) {
  return __hiloint2double(__double2hiint(x) ^ (int)0x80000000,
                          __double2loint(x));
}

// r *= m for the classes that need no arithmetic (cls <= EC_MI); the
// results equal the FP64 products.
template <typename C>
__device__ __forceinline__ void scale_exact(C& r, int cls) {
  const double x = r.x, y = r.y;
  switch (cls) {
    case EC_ZERO:
      r.x = r.y = 0;
      return;
    case EC_MONE:
      r.x = dneg(x);
      r.y = dneg(y);
      return;
    case EC_I:  // i (x + iy) = -y + ix
      r.x = dneg(y);
      r.y = x;
      return;
    case EC_MI:
      r.x = y;
      r.y = dneg(x);
      return;
    default:
      return;
  }
}

// r[i] *= m for the registers i with (i & MASK) == PAT; FP64 form
template <typename C, int NR, int MASK, int PAT>
__device__ __forceinline__ void scale_sel(C* r, const C& m, int cls) {
  switch (cls) {
    case EC_REAL:
#pragma unroll
      for (int i = 0; i < NR; ++i)
        if ((i & MASK) == PAT) {
          r[i].x = m.x * r[i].x;
          r[i].y = m.x * r[i].y;
        }
      return;
    case EC_IMAG:
#pragma unroll
      for (int i = 0; i < NR; ++i)
        if ((i & MASK) == PAT) {
          const C t = r[i];
          r[i].x = -(m.y * t.y);
          r[i].y = m.y * t.x;
        }
      return;
    case EC_FULL:
#pragma unroll
      for (int i = 0; i < NR; ++i)
        if ((i & MASK) == PAT) r[i] = cmul(m, r[i]);
      return;
    default:
      if (cls == EC_ONE) return;
#pragma unroll
      for (int i = 0; i < NR; ++i)
        if ((i & MASK) == PAT) scale_exact(r[i], cls);
      return;
  }
}

// the same in double-float pairs (e: the entry's exact triple)
template <typename C, int NR, int MASK, int PAT>
__device__ __forceinline__ void scale_sel_df(C* r, const DEC& e, int cls) {
  switch (cls) {
    case EC_REAL:
#pragma unroll
      for (int i = 0; i < NR; ++i)
        if ((i & MASK) == PAT) {
          const DC y = df_rmul(e.re, df_split2(r[i].x, r[i].y));
          r[i].x = df_join(y.re);
          r[i].y = df_join(y.im);
        }
      return;
    case EC_IMAG:
#pragma unroll
      for (int i = 0; i < NR; ++i)
        if ((i & MASK) == PAT) {
          const DC y = df_imul(e.im, df_split2(r[i].x, r[i].y));
          r[i].x = df_join(y.re);
          r[i].y = df_join(y.im);
        }
      return;
    case EC_FULL:
#pragma unroll
      for (int i = 0; i < NR; ++i)
        if ((i & MASK) == PAT) {
          const DC y = df_cmul(e, df_split2(r[i].x, r[i].y));
          r[i].x = df_join(y.re);
          r[i].y = df_join(y.im);
        }
      return;
    default:
      if (cls == EC_ONE) return;
#pragma unroll
      for (int i = 0; i < NR; ++i)
        if ((i & MASK) == PAT) scale_exact(r[i], cls);
      return;
  }
}

constexpr int K1_PERM = 0, K1_DIAG = 1, K1_ANTI = 2, K1_REAL = 3,
              K1_RX = 4, K1_FULL = 5;

__device__ __forceinline__ int kind_2x2(int c0, int c1, int c2, int c3) {
  if (c1 == EC_ZERO && c2 == EC_ZERO) return K1_DIAG;
  if (c0 == EC_ZERO && c3 == EC_ZERO)
    return c1 == EC_ONE && c2 == EC_ONE ? K1_PERM : K1_ANTI;
  if (ec_real(c0) && ec_real(c1) && ec_real(c2) && ec_real(c3))
    return K1_REAL;
  if (ec_real(c0) && ec_real(c3) && ec_imag(c1) && ec_imag(c2)) return K1_RX;
  return K1_FULL;
}

// Does a 2x2 of this kind and these classes need arithmetic?
__device__ __forceinline__ bool arith_2x2(int kind, const int* c) {
  switch (kind) {
    case K1_PERM:
      return false;
    case K1_DIAG:
      return c[0] > EC_MI || c[3] > EC_MI;
    case K1_ANTI:
      return c[1] > EC_MI || c[2] > EC_MI;
    default:
      return true;
  }
}

// The 2x2 (m0 m1; m2 m3) on register bit T, for the registers i with
// (i & CM) == CV (a control pattern; 0, 0 for none); c: the entries'
// classes.  FP64 form.
template <typename C, int NR, int T, int CM, int CV>
__device__ __forceinline__ void apply_2x2(C* r, const C& m0, const C& m1,
                                          const C& m2, const C& m3, int kind,
                                          const int* c) {
  constexpr int B = 1 << T;
  switch (kind) {
    case K1_PERM:
#pragma unroll
      for (int i = 0; i < NR; ++i) {
        if ((i & B) || (i & CM) != CV) continue;
        const C t = r[i];
        r[i] = r[i | B];
        r[i | B] = t;
      }
      return;
    case K1_DIAG:
      scale_sel<C, NR, B | CM, CV>(r, m0, c[0]);
      scale_sel<C, NR, B | CM, B | CV>(r, m3, c[3]);
      return;
    case K1_ANTI:  // swap, then scale by m1 (row 0) and m2 (row 1)
#pragma unroll
      for (int i = 0; i < NR; ++i) {
        if ((i & B) || (i & CM) != CV) continue;
        const C t = r[i];
        r[i] = r[i | B];
        r[i | B] = t;
      }
      scale_sel<C, NR, B | CM, CV>(r, m1, c[1]);
      scale_sel<C, NR, B | CM, B | CV>(r, m2, c[2]);
      return;
    case K1_REAL:
#pragma unroll
      for (int i = 0; i < NR; ++i) {
        if ((i & B) || (i & CM) != CV) continue;
        const C a0 = r[i], a1 = r[i | B];
        r[i].x = fma(m1.x, a1.x, m0.x * a0.x);
        r[i].y = fma(m1.x, a1.y, m0.x * a0.y);
        r[i | B].x = fma(m3.x, a1.x, m2.x * a0.x);
        r[i | B].y = fma(m3.x, a1.y, m2.x * a0.y);
      }
      return;
    case K1_RX:
#pragma unroll
      for (int i = 0; i < NR; ++i) {
        if ((i & B) || (i & CM) != CV) continue;
        const C a0 = r[i], a1 = r[i | B];
        r[i].x = fma(-m1.y, a1.y, m0.x * a0.x);
        r[i].y = fma(m1.y, a1.x, m0.x * a0.y);
        r[i | B].x = fma(m3.x, a1.x, -(m2.y * a0.y));
        r[i | B].y = fma(m3.x, a1.y, m2.y * a0.x);
      }
      return;
    default:
#pragma unroll
      for (int i = 0; i < NR; ++i) {
        if ((i & B) || (i & CM) != CV) continue;
        const C a0 = r[i], a1 = r[i | B];
        r[i] = cmad(m1, a1, cmul(m0, a0));
        r[i | B] = cmad(m3, a1, cmul(m2, a0));
      }
      return;
  }
}

// The same in double-float pairs, entries from their exact triples.
template <typename C, int NR, int T, int CM, int CV>
__device__ __forceinline__ void apply_2x2_df(C* r, const DEC& e0,
                                             const DEC& e1, const DEC& e2,
                                             const DEC& e3, int kind,
                                             const int* c) {
  constexpr int B = 1 << T;
  switch (kind) {
    case K1_PERM:
#pragma unroll
      for (int i = 0; i < NR; ++i) {
        if ((i & B) || (i & CM) != CV) continue;
        const C t = r[i];
        r[i] = r[i | B];
        r[i | B] = t;
      }
      return;
    case K1_DIAG:
      scale_sel_df<C, NR, B | CM, CV>(r, e0, c[0]);
      scale_sel_df<C, NR, B | CM, B | CV>(r, e3, c[3]);
      return;
    case K1_ANTI:
#pragma unroll
      for (int i = 0; i < NR; ++i) {
        if ((i & B) || (i & CM) != CV) continue;
        const C t = r[i];
        r[i] = r[i | B];
        r[i | B] = t;
      }
      scale_sel_df<C, NR, B | CM, CV>(r, e1, c[1]);
      scale_sel_df<C, NR, B | CM, B | CV>(r, e2, c[2]);
      return;
    default:
#pragma unroll
      for (int i = 0; i < NR; ++i) {
        if ((i & B) || (i & CM) != CV) continue;
        const DC a0 = df_split2(r[i].x, r[i].y);
        const DC a1 = df_split2(r[i | B].x, r[i | B].y);
        DC y0, y1;
        if (kind == K1_REAL) {
          y0 = df_row2_real(e0.re, a0, e1.re, a1);
          y1 = df_row2_real(e2.re, a0, e3.re, a1);
        } else if (kind == K1_RX) {
          y0 = df_row2_rx(e0.re, a0, e1.im, a1);
          y1 = df_row2_rx(e3.re, a1, e2.im, a0);
        } else {
          y0 = df_row2(e0, a0, e1, a1);
          y1 = df_row2(e2, a0, e3, a1);
        }
        r[i].x = df_join(y0.re);
        r[i].y = df_join(y0.im);
        r[i | B].x = df_join(y1.re);
        r[i | B].y = df_join(y1.im);
      }
      return;
  }
}

// Structure of a complex128 operator, found once per block.
struct OpKind {
  int kind;     // K1_* for 2x2; for 4x4: 0 general, 1 monomial (one
                // nonzero entry per row and column), 2 diagonal,
                // 3 controlled 2x2
  int sub;      // 4x4 controlled: K1_* of the 2x2 block
  int c[4];     // classes of the 2x2's entries m0..m3 / of the 4x4's
                // row entries (monomial) or diagonal / of the controlled
                // block's entries
  int perm;     // 4x4 monomial: column of row j's entry in bits 2j..2j+1
  int arith;    // 1 if applying it needs arithmetic
};

template <int K>
__device__ __forceinline__ OpKind classify_classes(const int* cl) {
  OpKind k{};
  if constexpr (K == 1) {
    k.kind = kind_2x2(cl[0], cl[1], cl[2], cl[3]);
#pragma unroll
    for (int j = 0; j < 4; ++j) k.c[j] = cl[j];
    k.arith = arith_2x2(k.kind, k.c);
    return k;
  } else {
    bool diag = true, mono = true, ctrl = true;
    int pm = 0, cols = 0, rc[4];
#pragma unroll
    for (int row = 0; row < 4; ++row) {
      int nz = 0, col = 0;
      rc[row] = EC_ZERO;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = cl[4 * row + j];
        if (c != EC_ZERO) {
          ++nz;
          col = j;
          rc[row] = c;
          if (j != row) diag = false;
          // controlled: identity on rows 0, 1; rows 2, 3 inside cols 2, 3
          if (row < 2 ? (j != row || c != EC_ONE) : j < 2) ctrl = false;
        } else if (row < 2 && j == row) {
          ctrl = false;
        }
      }
      if (nz != 1) mono = false;
      cols |= 1 << col;
      pm |= col << (2 * row);
    }
    if (cols != 15) mono = false;
    if (mono && !diag) {
      k.kind = 1;
      k.perm = pm;
      k.arith = 0;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        k.c[j] = rc[j];
        if (rc[j] > EC_MI) k.arith = 1;
      }
    } else if (diag) {
      k.kind = 2;
#pragma unroll
      for (int j = 0; j < 4; ++j) k.c[j] = cl[5 * j];
      k.arith = k.c[0] > EC_MI || k.c[1] > EC_MI || k.c[2] > EC_MI ||
                k.c[3] > EC_MI;
    } else if (ctrl) {
      k.kind = 3;
      k.c[0] = cl[10];
      k.c[1] = cl[11];
      k.c[2] = cl[14];
      k.c[3] = cl[15];
      k.sub = kind_2x2(k.c[0], k.c[1], k.c[2], k.c[3]);
      k.arith = arith_2x2(k.sub, k.c);
    } else {
      k.kind = 0;
      k.arith = 1;
    }
    return k;
  }
}

template <typename C>
__device__ __forceinline__ C pick4(const C* v, int j) {
  const C lo = (j & 1) ? v[1] : v[0];
  const C hi = (j & 1) ? v[3] : v[2];
  return (j & 2) ? hi : lo;
}

template <typename C, int NR, int RB0, int RB1>
__device__ __forceinline__ void permute4(C* r, int perm) {
  constexpr int M0 = 1 << RB0, M1 = 1 << RB1;
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if (i & (M0 | M1)) continue;
    const int idx[4] = {i, i | M1, i | M0, i | M0 | M1};
    C v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) v[j] = r[idx[j]];
#pragma unroll
    for (int j = 0; j < 4; ++j) r[idx[j]] = pick4(v, (perm >> (2 * j)) & 3);
  }
}

// Matrix index bit 1 (K = 2: the first target) is register bit RB0, bit 0
// register bit RB1.  FP64 form.
template <typename C, int NR, int K, int RB0, int RB1>
__device__ __forceinline__ void apply_c128(C* r, const C* m,
                                           const OpKind& k) {
  if constexpr (K == 1) {
    apply_2x2<C, NR, RB0, 0, 0>(r, m[0], m[1], m[2], m[3], k.kind, k.c);
  } else {
    constexpr int M0 = 1 << RB0, M1 = 1 << RB1;
    switch (k.kind) {
      case 1: {  // monomial: row j takes column perm_j, times its entry
        permute4<C, NR, RB0, RB1>(r, k.perm);
        if (k.c[0] != EC_ONE || k.c[1] != EC_ONE || k.c[2] != EC_ONE ||
            k.c[3] != EC_ONE) {
          scale_sel<C, NR, M0 | M1, 0>(r, pick4(m, k.perm & 3), k.c[0]);
          scale_sel<C, NR, M0 | M1, M1>(r, pick4(m + 4, (k.perm >> 2) & 3),
                                        k.c[1]);
          scale_sel<C, NR, M0 | M1, M0>(r, pick4(m + 8, (k.perm >> 4) & 3),
                                        k.c[2]);
          scale_sel<C, NR, M0 | M1, M0 | M1>(
              r, pick4(m + 12, (k.perm >> 6) & 3), k.c[3]);
        }
        return;
      }
      case 2:  // diagonal
        scale_sel<C, NR, M0 | M1, 0>(r, m[0], k.c[0]);
        scale_sel<C, NR, M0 | M1, M1>(r, m[5], k.c[1]);
        scale_sel<C, NR, M0 | M1, M0>(r, m[10], k.c[2]);
        scale_sel<C, NR, M0 | M1, M0 | M1>(r, m[15], k.c[3]);
        return;
      case 3:  // controlled: the lower-right 2x2 where bit RB0 is set
        apply_2x2<C, NR, RB1, M0, M0>(r, m[10], m[11], m[14], m[15], k.sub,
                                      k.c);
        return;
      default:
        apply_regs<C, NR, K, RB0, RB1>(r, m);
        return;
    }
  }
}

// The same in double-float pairs (e: the entries' exact triples).
template <typename C, int NR, int K, int RB0, int RB1>
__device__ __forceinline__ void apply_c128_df(C* r, const DEC* e,
                                              const OpKind& k) {
  if constexpr (K == 1) {
    apply_2x2_df<C, NR, RB0, 0, 0>(r, e[0], e[1], e[2], e[3], k.kind, k.c);
  } else {
    constexpr int M0 = 1 << RB0, M1 = 1 << RB1;
    switch (k.kind) {
      case 1:
        permute4<C, NR, RB0, RB1>(r, k.perm);
        if (k.c[0] != EC_ONE || k.c[1] != EC_ONE || k.c[2] != EC_ONE ||
            k.c[3] != EC_ONE) {
          scale_sel_df<C, NR, M0 | M1, 0>(r, e[k.perm & 3], k.c[0]);
          scale_sel_df<C, NR, M0 | M1, M1>(r, e[4 + ((k.perm >> 2) & 3)],
                                           k.c[1]);
          scale_sel_df<C, NR, M0 | M1, M0>(r, e[8 + ((k.perm >> 4) & 3)],
                                           k.c[2]);
          scale_sel_df<C, NR, M0 | M1, M0 | M1>(
              r, e[12 + ((k.perm >> 6) & 3)], k.c[3]);
        }
        return;
      case 2:
        scale_sel_df<C, NR, M0 | M1, 0>(r, e[0], k.c[0]);
        scale_sel_df<C, NR, M0 | M1, M1>(r, e[5], k.c[1]);
        scale_sel_df<C, NR, M0 | M1, M0>(r, e[10], k.c[2]);
        scale_sel_df<C, NR, M0 | M1, M0 | M1>(r, e[15], k.c[3]);
        return;
      case 3:
        apply_2x2_df<C, NR, RB1, M0, M0>(r, e[10], e[11], e[14], e[15],
                                         k.sub, k.c);
        return;
      default:
#pragma unroll
        for (int i = 0; i < NR; ++i) {
          if (i & (M0 | M1)) continue;
          const int idx[4] = {i, i | M1, i | M0, i | M0 | M1};
          DC a[4];
#pragma unroll
          for (int j = 0; j < 4; ++j)
            a[j] = df_split2(r[idx[j]].x, r[idx[j]].y);
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const DC y = df_row4(e + 4 * j, a);
            r[idx[j]].x = df_join(y.re);
            r[idx[j]].y = df_join(y.im);
          }
        }
        return;
    }
  }
}

// The shared operator of a complex128 launch, one copy per warp in shared
// memory.
template <int D>
struct C128Op {
  OpKind k;
  int pairs_ok;     // entries within the pair range
  DEC e[D * D];     // exact triples, for the pairs
  double2 raw[D * D];  // the entries, for the FP64 form
};

// Each warp fills its own copy (no block barrier): lane j loads entry j,
// classifies and splits it; the classes reach every lane as three ballots
// (one per class bit).
template <typename C, int K>
__device__ __forceinline__ void c128_prologue(const C* ops,
                                              C128Op<1 << K>& op) {
  constexpr int D = 1 << K;
  const int lane = threadIdx.x & 31;
  int cls = EC_ZERO;
  uint32_t mag = 0;
  if (lane < D * D) {
    const C mj = __ldg(ops + lane);
    cls = entry_class(mj);
    op.e[lane] = df_entry2(mj.x, mj.y);
    op.raw[lane] = mj;
    mag = max(df_hiword(mj.x) & 0x7fffffffu, df_hiword(mj.y) & 0x7fffffffu);
  }
  const uint32_t mx = __reduce_max_sync(0xffffffffu, mag);
  const uint32_t p0 = __ballot_sync(0xffffffffu, cls & 1);
  const uint32_t p1 = __ballot_sync(0xffffffffu, cls & 2);
  const uint32_t p2 = __ballot_sync(0xffffffffu, cls & 4);
  int cl[D * D];
#pragma unroll
  for (int j = 0; j < D * D; ++j)
    cl[j] = ((p0 >> j) & 1) | (((p1 >> j) & 1) << 1) | (((p2 >> j) & 1) << 2);
  if (lane == 0) {
    op.k = classify_classes<K>(cl);
    op.pairs_ok = mx >= (DF_EMIN << 20) && mx < ((DF_EMAX + 1) << 20);
  }
  __syncwarp();
}

// Every amplitude component of the thread's registers within the pair
// range (or zero).
template <typename C, int NR>
__device__ __forceinline__ bool pairs_in_range(const C* r) {
  uint32_t mx = 0;  // largest exponent field (the split computes the same)
#pragma unroll
  for (int i = 0; i < NR; ++i)
    mx = max(mx, max(df_hiword(r[i].x) & 0x7ff00000u,
                     df_hiword(r[i].y) & 0x7ff00000u));
  return mx < ((DF_EMAX + 1) << 20) && (mx == 0 || mx >= (DF_EMIN << 20));
}

// NH high targets (chunks per unit = 2^NH); RB0 / RB1 are the register-index
// bits of the first / second target in matrix order.
template <typename R, int V, int K, int NH, int RB0, int RB1>
__global__ void __launch_bounds__(256, 3)
    dense_chunk_kernel(const Cx<R>* in, Cx<R>* out, const Cx<R>* ops,
                       DenseArgs a) {
  using C = Cx<R>;
  constexpr int NCH = 1 << NH;
  constexpr int NR = NCH * V;
  constexpr int D = 1 << K;
  // amplitudes per thread: complex128 keeps four so that the pair
  // arithmetic fits the 85 registers of three blocks per SM
  constexpr int TARGET = sizeof(R) == 4 ? 16 : 4;
  constexpr int UNROLL = NR >= TARGET ? 1 : TARGET / NR;
  constexpr bool kC128 = sizeof(R) == 8;
  const bool shared_op = a.op_stride == 0;

  C m[D * D];
  if (!kC128 && shared_op) {
#pragma unroll
    for (int j = 0; j < D * D; ++j) m[j] = __ldg(ops + j);
  }

  C reg[UNROLL][NR];
  uint64_t obase[UNROLL];
  uint64_t state[UNROLL];
  const uint64_t first =
      (uint64_t)blockIdx.x * (UNROLL * blockDim.x) + threadIdx.x;
  const uint64_t lmask = (uint64_t(1) << a.log_units) - 1;

#pragma unroll
  for (int u = 0; u < UNROLL; ++u) {
    const uint64_t g = first + (uint64_t)u * blockDim.x;
    if (g >= a.total_units) break;
    const uint64_t s = g >> a.log_units;
    uint64_t x = (g & lmask) << a.log_v;
#pragma unroll
    for (int j = 0; j < NH; ++j) x = insert_zero(x, a.ins_pos[j]);
    state[u] = s;
    obase[u] = (s << a.n) + x;
    const C* src = in + s * a.in_stride + x;
#pragma unroll
    for (int c = 0; c < NCH; ++c) {
      int64_t off = 0;
      if (NH > 0 && (c & 1)) off += a.hstride[0];
      if (NH > 1 && (c & 2)) off += a.hstride[1];
      load_chunk<V>(src + off, &reg[u][c * V]);
    }
  }

  // complex128 with a shared operator: warp 0 classifies it while the
  // state loads are in flight, then one structured pass over every unit's
  // registers (the target bits index within each unit's NR block;
  // registers of units past the end are computed and not stored)
  if constexpr (kC128) {
    __shared__ C128Op<D> warp_op[256 / 32];
    if (shared_op) {
      C128Op<D>& op = warp_op[threadIdx.x >> 5];
      c128_prologue<C, K>(ops, op);
      const OpKind kind = op.k;
      bool pairs = a.df != 0;
      if (pairs && kind.arith)
        pairs = op.pairs_ok && pairs_in_range<C, UNROLL * NR>(&reg[0][0]);
      if (pairs || !kind.arith)
        apply_c128_df<C, UNROLL * NR, K, RB0, RB1>(&reg[0][0], op.e, kind);
      else
        apply_c128<C, UNROLL * NR, K, RB0, RB1>(&reg[0][0], op.raw, kind);
    }
  }
#pragma unroll
  for (int u = 0; u < UNROLL; ++u) {
    const uint64_t g = first + (uint64_t)u * blockDim.x;
    if (g >= a.total_units) break;
    if (!shared_op) {
      const C* mp = ops + state[u] * a.op_stride;
#pragma unroll
      for (int j = 0; j < D * D; ++j) m[j] = __ldg(mp + j);
      apply_regs<C, NR, K, RB0, RB1>(reg[u], m);
    } else if constexpr (!kC128) {
      apply_regs<C, NR, K, RB0, RB1>(reg[u], m);
    }
    C* dst = out + obase[u];
#pragma unroll
    for (int c = 0; c < NCH; ++c) {
      int64_t off = 0;
      if (NH > 0 && (c & 1)) off += a.hstride[0];
      if (NH > 1 && (c & 2)) off += a.hstride[1];
      store_chunk<V>(dst + off, &reg[u][c * V]);
    }
  }
}

// complex128 with one operator shared by every state: a persistent kernel
// in warp steps.  A warp step covers one block of 128 amplitudes: its
// "inner" index bits are the gate's targets and the lowest other bits (7
// in all), so the block is made of contiguous runs of at least 32
// amplitudes (512 bytes).  Lanes copy the block lane-contiguously into the
// warp's shared-memory slot with 16-byte cp.async copies, two steps ahead;
// each lane then takes its two pairs (one qubit) or its quad (two qubits)
// out of the slot, applies the gate in registers, puts the results back,
// and the warp stores the block lane-contiguously.  The pair arithmetic
// needs over 100 registers, which leaves no room to hold loads in flight in
// registers; through shared memory each SM keeps 64 KB of loads in flight
// (two blocks of eight warps, two steps of 2 KB ahead) while its warps
// compute.  Lanes never share a pair, so each lane writes back only what
// it read.  Warp steps cover disjoint amplitudes, so in-place updates are
// safe.
constexpr int C128_STAGES = 3;    // slots per warp: two in flight, one in use
constexpr int C128_THREADS = 256;
constexpr int C128_BLOCK = 128;   // amplitudes per warp step

struct StreamArgs {
  uint64_t total_steps;  // num_states << (n - 7)
  int log_steps;         // n - 7
  int df;                // double-float pairs (1) or FP64 (0)
  int64_t in_stride;     // amplitudes between input states (0 = broadcast)
  int n;
  int inner[7];          // inner bit positions, ascending: 0 .. low - 1,
  int low;               // then the targets above that run (hpos)
  int nhigh;
  int hpos[2];
  int b0, b1;            // inner index of the first / second target
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s),
               "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait1() {
  asm volatile("cp.async.wait_group 1;\n" ::: "memory");
}

template <int K>
__global__ void __launch_bounds__(C128_THREADS, 2)
    dense_c128_stream_kernel(const double2* in, double2* out,
                             const double2* ops, StreamArgs a) {
  using C = double2;
  constexpr int D = 1 << K;
  extern __shared__ __align__(16) double2 slots[];  // [warp][stage][128]
  __shared__ uint32_t loc_off[C128_BLOCK];  // inner index -> offset
  __shared__ C128Op<D> warp_op[C128_THREADS / 32];

  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  for (int j = t; j < C128_BLOCK; j += C128_THREADS) {
    uint32_t off = 0;
#pragma unroll
    for (int q = 0; q < 7; ++q)
      if ((j >> q) & 1) off |= 1u << a.inner[q];
    loc_off[j] = off;
  }
  __syncthreads();

  C* const slot = slots + warp * (C128_STAGES * C128_BLOCK);
  const uint64_t nw = (uint64_t)gridDim.x * (C128_THREADS / 32);
  const uint64_t smask = (uint64_t(1) << a.log_steps) - 1;

  // amplitude offset of warp step ws's block (inner bits zero)
  auto block_base = [&](uint64_t ws, uint64_t& st) {
    st = ws >> a.log_steps;
    uint64_t x = (ws & smask) << a.low;
#pragma unroll
    for (int j = 0; j < 2; ++j)
      if (j < a.nhigh) x = insert_zero(x, a.hpos[j]);
    return x;
  };
  auto issue = [&](uint64_t ws, int stage) {
    if (ws < a.total_steps) {
      uint64_t st;
      const uint64_t x = block_base(ws, st);
      const C* src = in + st * a.in_stride + x;
#pragma unroll
      for (int i = 0; i < C128_BLOCK / 32; ++i) {
        const int j = lane + 32 * i;
        cp_async16(&slot[stage * C128_BLOCK + j], src + loc_off[j]);
      }
    }
    cp_async_commit();
  };

  // the lane's amplitudes inside the block, in matrix order
  int idx[4];
  if constexpr (K == 1) {
    const int m = 1 << a.b0;
    idx[0] = (int)insert_zero((uint64_t)lane, a.b0);
    idx[1] = idx[0] | m;
    idx[2] = (int)insert_zero((uint64_t)lane + 32, a.b0);
    idx[3] = idx[2] | m;
  } else {
    const int lo = min(a.b0, a.b1), hi = max(a.b0, a.b1);
    const int base = (int)insert_zero(insert_zero((uint64_t)lane, lo), hi);
    idx[0] = base;
    idx[1] = base | (1 << a.b1);
    idx[2] = base | (1 << a.b0);
    idx[3] = base | (1 << a.b0) | (1 << a.b1);
  }
  constexpr int RB0 = K == 1 ? 0 : 1, RB1 = 0;

  uint64_t ws = (uint64_t)blockIdx.x * (C128_THREADS / 32) + warp;
  issue(ws, 0);
  issue(ws + nw, 1);
  C128Op<D>& op = warp_op[warp];
  c128_prologue<C, K>(ops, op);
  const OpKind kind = op.k;
  const bool pairs_mode = a.df != 0 && op.pairs_ok;

  for (int k = 0; ws < a.total_steps; ++k, ws += nw) {
    C* const S = slot + (k % C128_STAGES) * C128_BLOCK;
    cp_async_wait1();
    __syncwarp();  // every lane's copies of this step have landed, and
                   // every lane is done with the slot reused below
    issue(ws + 2 * nw, (k + 2) % C128_STAGES);
    C r[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) r[j] = S[idx[j]];

    bool pairs = pairs_mode;
    if (pairs && kind.arith) pairs = pairs_in_range<C, 4>(r);
    if (pairs || !kind.arith)
      apply_c128_df<C, 4, K, RB0, RB1>(r, op.e, kind);
    else
      apply_c128<C, 4, K, RB0, RB1>(r, op.raw, kind);

#pragma unroll
    for (int j = 0; j < 4; ++j) S[idx[j]] = r[j];
    __syncwarp();
    uint64_t st;
    const uint64_t x = block_base(ws, st);
    C* dst = out + (st << a.n) + x;
#pragma unroll
    for (int i = 0; i < C128_BLOCK / 32; ++i) {
      const int j = lane + 32 * i;
      __stcs(dst + loc_off[j], S[j]);
    }
  }
}

// Any k <= GBSV_MAX_DENSE_QUBITS: one thread per output amplitude,
// out[i] = sum_b M[row(i), b] * in[base(i) + offs[b]].  Used for k = 0,
// complex128 with k >= 5 and the complex64 cases dense_wide_kernel leaves
// (per-state operators on states of fewer than one tile of groups).
struct GenericArgs {
  uint64_t total;  // num_states << n
  int n;
  int k;
  int64_t in_stride;
  int64_t op_stride;
  uint64_t tmask;       // bits of the target positions
  int pos[GBSV_MAX_DENSE_QUBITS];  // position of matrix bit (k-1-j)
  int df;               // complex128: double-float pairs (1) or FP64 (0)
};

template <typename R>
__global__ void __launch_bounds__(256)
    dense_generic_kernel(const Cx<R>* in, Cx<R>* out, const Cx<R>* ops,
                         GenericArgs a) {
  using C = Cx<R>;
  extern __shared__ uint64_t offs[];
  const int D = 1 << a.k;
  for (int b = threadIdx.x; b < D; b += blockDim.x) {
    uint64_t o = 0;
    for (int j = 0; j < a.k; ++j)
      if ((b >> (a.k - 1 - j)) & 1) o |= uint64_t(1) << a.pos[j];
    offs[b] = o;
  }
  __syncthreads();
  const uint64_t nmask = (uint64_t(1) << a.n) - 1;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
       i < a.total; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t s = i >> a.n;
    const uint64_t loc = i & nmask;
    int row = 0;
    for (int j = 0; j < a.k; ++j)
      row |= (int)((loc >> a.pos[j]) & 1) << (a.k - 1 - j);
    const uint64_t base = loc & ~a.tmask;
    const C* src = in + s * a.in_stride + base;
    const C* mrow = ops + s * a.op_stride + (int64_t)row * D;
    C acc = czero<C>();
    for (int b = 0; b < D; ++b) acc = cmad(__ldg(mrow + b), src[offs[b]], acc);
    out[i] = acc;
  }
}

// k = 3..5 target qubits: one thread per group of 2^k amplitudes (two
// groups when one matrix serves all states and both fit in 256 bytes of
// registers).  complex64 5-qubit operators, and 4-qubit ones with a target
// among the three lowest bits, go to dense_wide_kernel instead
// (wide_applies); this kernel remains their in-place fallback.  The thread reads its group once (consecutive threads take consecutive groups,
// so every load instruction of a warp is contiguous when bit 0 is not a
// target), multiplies by the matrix (in shared memory when one matrix
// serves all states) and writes the group; in place is safe.
template <typename R, int K>
__global__ void __launch_bounds__(128)
    dense_group_kernel(const Cx<R>* in, Cx<R>* out, const Cx<R>* ops,
                       GenericArgs a) {
  using C = Cx<R>;
  constexpr int D = 1 << K;
  __shared__ __align__(16) C msm[D * D];
  __shared__ uint64_t offs[D];
  __shared__ int spos[K];
  const int tid = threadIdx.x;
  if (tid < D) {
    uint64_t o = 0;
    for (int j = 0; j < K; ++j)
      if ((tid >> (K - 1 - j)) & 1) o |= uint64_t(1) << a.pos[j];
    offs[tid] = o;
  }
  if (tid == 0) {  // target positions ascending, for the zero insertion
    int p[K];
    for (int j = 0; j < K; ++j) p[j] = a.pos[j];
    for (int i = 1; i < K; ++i)
      for (int j = i; j > 0 && p[j - 1] > p[j]; --j) {
        const int t = p[j];
        p[j] = p[j - 1];
        p[j - 1] = t;
      }
    for (int j = 0; j < K; ++j) spos[j] = p[j];
  }
  const bool shared_op = a.op_stride == 0;
  // complex128 in pairs: the entries as exact triples, and whether all of
  // them lie in the pair range (block-uniform)
  constexpr bool kC128 = sizeof(R) == 8;
  __shared__ DEC msd[kC128 ? D * D : 1];
  bool bad = false;
  if (shared_op)
    for (int i = tid; i < D * D; i += blockDim.x) {
      const C mv = ops[i];
      msm[i] = mv;
      if constexpr (kC128) {
        msd[i] = df_entry2(mv.x, mv.y);
        bad |= max(df_hiword(mv.x) & 0x7ff00000u,
                   df_hiword(mv.y) & 0x7ff00000u) >= ((DF_EMAX + 1) << 20);
      }
    }
  bad = __syncthreads_or(bad);
  const int n = a.n;
  const uint64_t gps = uint64_t(1) << (n - K);  // groups per state
  const uint64_t total = (a.total >> n) * gps;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  if constexpr (kC128) {
    // one group per thread: the amplitudes split into pairs, each output
    // a compensated dot product (df_rowD); a thread whose amplitudes leave
    // the pair range runs the FP64 rows
    if (shared_op && a.df && !bad) {
      for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + tid; g < total;
           g += stride) {
        const uint64_t s = g / gps;
        uint64_t base = g % gps;
#pragma unroll
        for (int j = 0; j < K; ++j) base = insert_zero(base, spos[j]);
        const C* src = in + s * a.in_stride + base;
        C* dst = out + (s << n) + base;
        C x[D];
#pragma unroll
        for (int b = 0; b < D; ++b) x[b] = src[offs[b]];
        if (pairs_in_range<C, D>(x)) {
          DC xs[D];
#pragma unroll
          for (int b = 0; b < D; ++b) xs[b] = df_split2(x[b].x, x[b].y);
#pragma unroll 2
          for (int r = 0; r < D; ++r) {
            const DC y = df_rowD<D>(msd + r * D, xs);
            C o;
            o.x = df_join(y.re);
            o.y = df_join(y.im);
            dst[offs[r]] = o;
          }
        } else {
#pragma unroll 2
          for (int r = 0; r < D; ++r) {
            C acc = czero<C>();
#pragma unroll
            for (int b = 0; b < D; ++b) acc = cmad(msm[r * D + b], x[b], acc);
            dst[offs[r]] = acc;
          }
        }
      }
      return;
    }
  }
  auto group_base = [&](uint64_t g, const C** src, C** dst) {
    const uint64_t s = g / gps;
    uint64_t base = g % gps;
#pragma unroll
    for (int j = 0; j < K; ++j) base = insert_zero(base, spos[j]);
    *src = in + s * a.in_stride + base;
    *dst = out + (s << n) + base;
  };
  // two groups per thread where their amplitudes fit in registers: every
  // matrix element read from shared memory feeds both
  constexpr bool kPair = 2 * D * sizeof(C) <= 256;
  if constexpr (kPair) {
    if (shared_op) {
      for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + tid; g < total;
           g += 2 * stride) {
        const uint64_t g1 = g + stride;
        const bool two = g1 < total;
        const C *src0, *src1;
        C *dst0, *dst1;
        group_base(g, &src0, &dst0);
        group_base(two ? g1 : g, &src1, &dst1);
        C x0[D], x1[D];
#pragma unroll
        for (int b = 0; b < D; ++b) {
          x0[b] = src0[offs[b]];
          x1[b] = src1[offs[b]];
        }
#pragma unroll 2
        for (int r = 0; r < D; ++r) {
          C acc0 = czero<C>(), acc1 = czero<C>();
#pragma unroll
          for (int b = 0; b < D; ++b) {
            const C mv = msm[r * D + b];
            acc0 = cmad(mv, x0[b], acc0);
            acc1 = cmad(mv, x1[b], acc1);
          }
          dst0[offs[r]] = acc0;
          if (two) dst1[offs[r]] = acc1;
        }
      }
      return;
    }
  }
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + tid; g < total;
       g += stride) {
    const uint64_t s = g / gps;
    uint64_t base = g % gps;
#pragma unroll
    for (int j = 0; j < K; ++j) base = insert_zero(base, spos[j]);
    const C* src = in + s * a.in_stride + base;
    C* dst = out + (s << n) + base;
    C x[D];
#pragma unroll
    for (int b = 0; b < D; ++b) x[b] = src[offs[b]];
    const C* m = shared_op ? msm : ops + s * a.op_stride;
#pragma unroll 4
    for (int r = 0; r < D; ++r) {
      C acc = czero<C>();
#pragma unroll
      for (int b = 0; b < D; ++b) acc = cmad(m[r * D + b], x[b], acc);
      dst[offs[r]] = acc;
    }
  }
}

// ------------------------------------------------------------ dispatch --
template <typename R, int V, int K, int NH, int RB0, int RB1>
static int launch_chunk(const void* in, void* out, const void* ops,
                        const DenseArgs& a, cudaStream_t st) {
  constexpr int NR = (1 << NH) * V;
  constexpr int TARGET = sizeof(R) == 4 ? 16 : 4;
  constexpr int UNROLL = NR >= TARGET ? 1 : TARGET / NR;
  const uint64_t per_block = (uint64_t)UNROLL * 256;
  const uint64_t blocks = (a.total_units + per_block - 1) / per_block;
  if (blocks > 0x7fffffffull)
    return set_error(GBSV_ERR_UNSUPPORTED, "grid too large (%llu blocks)",
                     (unsigned long long)blocks);
  dense_chunk_kernel<R, V, K, NH, RB0, RB1><<<(unsigned)blocks, 256, 0, st>>>(
      static_cast<const Cx<R>*>(in), static_cast<Cx<R>*>(out),
      static_cast<const Cx<R>*>(ops), a);
  return after_launch("dense_chunk_kernel");
}

// complex128, shared operator, n >= 7: the warp-step streaming kernel.
static int launch_c128_stream(const void* in, void* out, int n,
                              int64_t num_states, int64_t in_stride,
                              const void* ops, const int* pos, int k,
                              cudaStream_t st) {
  StreamArgs a{};
  a.n = n;
  a.log_steps = n - 7;
  a.total_steps = (uint64_t)num_states << a.log_steps;
  a.in_stride = in_stride;
  a.df = c128_arith() == GBSV_C128_PAIRS;
  // inner bits: the targets and the lowest other bits, 7 in all
  uint64_t inner_mask = 0;
  for (int j = 0; j < k; ++j) inner_mask |= uint64_t(1) << pos[j];
  for (int b = 0; __builtin_popcountll(inner_mask) < 7; ++b)
    inner_mask |= uint64_t(1) << b;
  int q = 0;
  for (int b = 0; b < n; ++b)
    if ((inner_mask >> b) & 1) {
      if (b == pos[0]) a.b0 = q;
      if (k == 2 && b == pos[1]) a.b1 = q;
      a.inner[q++] = b;
    }
  while (a.low < 7 && a.inner[a.low] == a.low) ++a.low;
  a.nhigh = 7 - a.low;  // at most the two targets
  for (int j = 0; j < a.nhigh; ++j) a.hpos[j] = a.inner[a.low + j];
  constexpr size_t smem = (size_t)(C128_THREADS / 32) * C128_STAGES *
                          C128_BLOCK * sizeof(double2);
  const void* fn = k == 1 ? (const void*)dense_c128_stream_kernel<1>
                          : (const void*)dense_c128_stream_kernel<2>;
  // the shared-memory opt-in, once per device and kernel (a race only
  // repeats it)
  static std::atomic<uint64_t> attr_set[2];
  int dev = 0;
  cudaGetDevice(&dev);
  const uint64_t bit = uint64_t(1) << (dev & 63);
  if (!(attr_set[k - 1].load(std::memory_order_relaxed) & bit)) {
    const cudaError_t e = cudaFuncSetAttribute(
        fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
      return set_error(GBSV_ERR_CUDA, "dense_c128_stream_kernel: %s",
                       cudaGetErrorString(e));
    attr_set[k - 1].fetch_or(bit, std::memory_order_relaxed);
  }
  const uint64_t warps = C128_THREADS / 32;
  uint64_t blocks = (a.total_steps + warps - 1) / warps;
  const uint64_t cap = (uint64_t)sm_count() * 2;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  const double2* i2 = static_cast<const double2*>(in);
  double2* o2 = static_cast<double2*>(out);
  const double2* m2 = static_cast<const double2*>(ops);
  if (k == 1)
    dense_c128_stream_kernel<1>
        <<<(unsigned)blocks, C128_THREADS, smem, st>>>(i2, o2, m2, a);
  else
    dense_c128_stream_kernel<2>
        <<<(unsigned)blocks, C128_THREADS, smem, st>>>(i2, o2, m2, a);
  return after_launch("dense_c128_stream_kernel");
}

// Select the template instance for (V, K, NH, RB0, RB1).
template <typename R>
static int dispatch_chunk(int V, int K, int NH, int rb0, int rb1,
                          const void* in, void* out, const void* ops,
                          const DenseArgs& a, cudaStream_t st) {
#define GBSV_CASE(v, k, nh, r0, r1)                                   \
  if (V == v && K == k && NH == nh && rb0 == r0 && (k == 1 || rb1 == r1)) \
    return launch_chunk<R, v, k, nh, r0, r1>(in, out, ops, a, st);
  // scalar fallback: every target is "high"
  GBSV_CASE(1, 1, 1, 0, 0)
  GBSV_CASE(1, 2, 2, 0, 1)
  if constexpr (sizeof(R) == 4) {
    GBSV_CASE(4, 1, 1, 2, 0)
    GBSV_CASE(4, 1, 0, 0, 0)
    GBSV_CASE(4, 1, 0, 1, 0)
    GBSV_CASE(4, 2, 2, 2, 3)
    GBSV_CASE(4, 2, 1, 2, 0)
    GBSV_CASE(4, 2, 1, 2, 1)
    GBSV_CASE(4, 2, 1, 0, 2)
    GBSV_CASE(4, 2, 1, 1, 2)
    GBSV_CASE(4, 2, 0, 0, 1)
    GBSV_CASE(4, 2, 0, 1, 0)
  } else {
    GBSV_CASE(2, 1, 1, 1, 0)
    GBSV_CASE(2, 1, 0, 0, 0)
    GBSV_CASE(2, 2, 2, 1, 2)
    GBSV_CASE(2, 2, 1, 1, 0)
    GBSV_CASE(2, 2, 1, 0, 1)
  }
#undef GBSV_CASE
  return set_error(GBSV_ERR_UNSUPPORTED,
                   "no dense kernel for V=%d K=%d NH=%d rb=(%d,%d)", V, K, NH,
                   rb0, rb1);
}

// k in {1, 2}: plan chunk width, high/low targets and register bits.
static int apply_small(const void* in, void* out, int dtype, int n,
                       int64_t num_states, int64_t in_stride, const void* ops,
                       int64_t op_stride, const int* pos, int k,
                       cudaStream_t st) {
  const int amp = dtype_bytes(dtype);
  if (dtype == GBSV_C128 && op_stride == 0 && n >= 7 &&
      (uintptr_t)in % 16 == 0 && (uintptr_t)out % 16 == 0)
    return launch_c128_stream(in, out, n, num_states, in_stride, ops, pos, k,
                              st);
  const int vfull = dtype == GBSV_C64 ? 4 : 2;
  const int log_vfull = dtype == GBSV_C64 ? 2 : 1;
  int nh_full = 0;
  for (int j = 0; j < k; ++j) nh_full += pos[j] >= log_vfull;
  const bool aligned = ((uintptr_t)in % 16 == 0) && ((uintptr_t)out % 16 == 0) &&
                       ((in_stride * amp) % 16 == 0);
  const bool fits = n >= log_vfull + nh_full;
  const int V = (aligned && fits) ? vfull : 1;
  const int log_v = V == 1 ? 0 : log_vfull;

  DenseArgs a{};
  a.n = n;
  a.in_stride = in_stride;
  a.op_stride = op_stride;
  a.log_v = log_v;
  int rb[2] = {0, 0};
  int nh = 0;
  int hpos[2] = {0, 0};
  for (int j = 0; j < k; ++j) {
    if (pos[j] >= log_v) {
      rb[j] = log_v + nh;
      a.hstride[nh] = int64_t(1) << pos[j];
      hpos[nh] = pos[j];
      ++nh;
    } else {
      rb[j] = pos[j];
    }
  }
  a.nins = nh;
  if (nh == 2 && hpos[0] > hpos[1]) std::swap(hpos[0], hpos[1]);
  for (int j = 0; j < nh; ++j) a.ins_pos[j] = hpos[j];
  a.log_units = n - log_v - nh;
  a.total_units = (uint64_t)num_states << a.log_units;
  a.df = c128_arith() == GBSV_C128_PAIRS;
  if (dtype == GBSV_C64)
    return dispatch_chunk<float>(V, k, nh, rb[0], rb[1], in, out, ops, a, st);
  return dispatch_chunk<double>(V, k, nh, rb[0], rb[1], in, out, ops, a, st);
}

// ------------------------------------------------ wide operators (c64) ----
// k = 4..12 target qubits, complex64 (k = 4, 5 where the group kernel is
// slower, see wide_applies): a CTA holds a "tile" of BN = 2^(13-k) groups
// (all 2^k amplitudes of each, 8192 amplitudes = 64 KB) in shared memory and
// computes the D x BN output tile as a complex matrix product, the operator
// streamed through shared memory in chunks of BK columns (k <= 6 keeps the
// whole operator resident).  Each thread accumulates TM x TN = 32 outputs
// in registers; per k-step it reads TM operator entries (at most two thread
// rows per warp: broadcasts) and TN/2 16-byte amplitude pairs.  Tile rows
// are XOR-swizzled by 16-byte pairs (row & 15) so that copies of low-target
// tiles spread over the banks; k = 4..8 walk rows in unrolled blocks of 16,
// where the swizzle is a constant of each step and every shared load has an
// immediate offset (the FP32 pipe is then the bound, not integer address
// work).  Amplitudes are copied in by cp.async in input-address order; the
// outputs are stored straight from registers when a thread's column pairs
// are adjacent in memory (target bit 0 free), else staged through shared
// memory and written in the same address order (coalesced either way).
// Every output sums over the operator's columns in order with the fused
// multiply-adds of dense_generic_kernel, so both kernels give the same
// bits.  A tile is read completely before any of it is written, and tiles
// are disjoint, so in place is safe.
template <int K>
struct WideCfg {
  static constexpr int D = 1 << K;
  static constexpr int LBN = 13 - K;               // log2 groups per tile
  static constexpr int BN = 1 << LBN;
  static constexpr int BK = (4096 >> K) < D ? (4096 >> K) : D;  // chunk
  static constexpr int TN = K <= 6 ? 8 : (K == 12 ? 2 : 4);
  static constexpr int TM = 32 / TN;
  static constexpr int NTC = BN / TN;              // thread columns
  static constexpr int NTR = 256 / NTC;            // thread rows
  static constexpr int LDM = BK + 1;               // padded chunk row
  static constexpr int SWM = (BN / 2 < 16 ? BN / 2 : 16) - 1;
  static constexpr size_t SMEM = (size_t)(D * BN + D * LDM) * 8;
  static_assert(NTR * TM == D && NTC * TN == BN && D * BN == 8192, "");
};

struct WideArgs {
  uint64_t groups;  // num_states << (n - k)
  int n;
  int lgps;         // log2 groups per state (n - k)
  int vec;          // output column pairs adjacent and 16-byte aligned
  int nspos;
  int64_t in_stride;
  int64_t op_stride;
  int spos[GBSV_MAX_DENSE_QUBITS];     // target positions, ascending
  int64_t boff[GBSV_MAX_DENSE_QUBITS]; // address offset of matrix bit m
  int64_t cout[9];   // output address offset of tile column bit q
  // the 13 bits of a tile element index (row b, column c), lowest input
  // address first: input address offset and shared index (b * BN + c)
  int64_t ein[13];
  int64_t eout[13];  // output address offset of the same bits
  int32_t eix[13];
  int64_t rj[16];    // offs(2 * NTR * (i >> 1) + (i & 1)), i < TM
  int64_t cj[8];     // output offset of column 2 * NTC * (j >> 1) + (j & 1)
};

template <int K>
__global__ void __launch_bounds__(256, K <= 10 ? 2 : 1)
    dense_wide_kernel(const float2* in, float2* out, const float2* ops,
                      WideArgs a) {
  using W = WideCfg<K>;
  constexpr int D = W::D, BN = W::BN, BK = W::BK, TM = W::TM, TN = W::TN,
                NTC = W::NTC, NTR = W::NTR, LDM = W::LDM, SWM = W::SWM;
  constexpr bool kResident = BK == D;
  extern __shared__ __align__(16) float2 wsm[];
  float2* xs = wsm;           // [D][BN] the tile, columns XOR-swizzled
  float2* ms = wsm + D * BN;  // [D][LDM] columns kc .. kc + BK - 1
  __shared__ int64_t it_in[32], it_out[32];
  __shared__ int32_t it_ix[32];
  const int tid = threadIdx.x;
  if (tid < 32) {  // element bits 8..12 come from the copy iteration
    int64_t g = 0, o = 0;
    int32_t x = 0;
    for (int j = 0; j < 5; ++j)
      if ((tid >> j) & 1) {
        g += a.ein[8 + j];
        o += a.eout[8 + j];
        x += a.eix[8 + j];
      }
    it_in[tid] = g;
    it_out[tid] = o;
    it_ix[tid] = x;
  }
  int64_t t_in = 0, t_out = 0;  // element bits 0..7 come from the thread
  int32_t t_ix = 0;
  for (int j = 0; j < 8; ++j)
    if ((tid >> j) & 1) {
      t_in += a.ein[j];
      t_out += a.eout[j];
      t_ix += a.eix[j];
    }
  const int tcol = tid % NTC, trow = tid / NTC;
  int64_t r_t = 0, c_t = 0;  // offsets of row 2*trow and column 2*tcol
  for (int m = 0; m < K; ++m)
    if (((2 * trow) >> m) & 1) r_t += a.boff[m];
  for (int q = 0; q < W::LBN; ++q)
    if (((2 * tcol) >> q) & 1) c_t += a.cout[q];
  __syncthreads();

  auto load_mat = [&](const float2* mat, int kc) {
#pragma unroll
    for (int i = 0; i < D * BK / 256; ++i) {
      const int e = tid + 256 * i;
      const int r = e / BK, kk = e % BK;
      cp_async8(ms + r * LDM + kk, mat + (int64_t)r * D + kc + kk);
    }
  };

  const uint64_t ntiles = (a.groups + BN - 1) >> W::LBN;
  const uint64_t gmask = (uint64_t(1) << a.lgps) - 1;
  int64_t loaded = -1;
  for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const uint64_t g0 = t << W::LBN;
    const uint64_t s0 = g0 >> a.lgps;
    uint64_t gin = g0 & gmask;
    for (int j = 0; j < a.nspos; ++j) gin = insert_zero(gin, a.spos[j]);
    const float2* src = in + (int64_t)s0 * a.in_stride + gin;
    float2* dst = out + (s0 << a.n) + gin;
    const uint64_t left = a.groups - g0;
    const int cv = left < (uint64_t)BN ? (int)left : BN;
    const float2* mat = ops + (a.op_stride ? (int64_t)s0 * a.op_stride : 0);
#pragma unroll 8
    for (int i = 0; i < 32; ++i) {
      const int32_t x = t_ix + it_ix[i];
      const int b = x >> W::LBN, c = x & (BN - 1);
      if (c < cv)
        cp_async8(xs + b * BN + (c ^ ((b & SWM) << 1)),
                  src + t_in + it_in[i]);
    }
    if constexpr (kResident) {
      const int64_t id = a.op_stride ? (int64_t)s0 : 0;
      if (id != loaded) {  // block-uniform
        load_mat(mat, 0);
        loaded = id;
      }
    } else {
      load_mat(mat, 0);
    }
    cp_async_wait_all();
    __syncthreads();

    float2 acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) acc[i][j] = make_float2(0.f, 0.f);
    for (int kc = 0; kc < D; kc += BK) {
      if (!kResident && kc) {
        __syncthreads();  // the previous chunk is no longer read
        load_mat(mat, kc);
        cp_async_wait_all();
        __syncthreads();
      }
      if constexpr (BK >= 16 && SWM == 15) {
        // blocks of 16 rows: the swizzle of row kc + k16 + u is 2u, a
        // constant of the unrolled step
        for (int k16 = 0; k16 < BK; k16 += 16) {
          const float2* xblk = xs + (kc + k16) * BN;
          const float2* mblk = ms + (2 * trow) * LDM + k16;
#pragma unroll
          for (int u = 0; u < 16; ++u) {
            float2 av[TM], xv[TN];
#pragma unroll
            for (int i = 0; i < TM; ++i)
              av[i] = mblk[(2 * NTR * (i >> 1) + (i & 1)) * LDM + u];
            const float2* xrow = xblk + u * BN;
            const int c0 = (2 * tcol) ^ (2 * u);
#pragma unroll
            for (int j = 0; j < TN / 2; ++j) {
              const float4 v = *reinterpret_cast<const float4*>(
                  xrow + (c0 ^ (2 * NTC * j)));
              xv[2 * j] = make_float2(v.x, v.y);
              xv[2 * j + 1] = make_float2(v.z, v.w);
            }
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
              for (int j = 0; j < TN; ++j)
                acc[i][j] = cmad(av[i], xv[j], acc[i][j]);
          }
        }
      } else {
#pragma unroll 2
        for (int kk = 0; kk < BK; ++kk) {
          const int b = kc + kk;
          float2 av[TM], xv[TN];
#pragma unroll
          for (int i = 0; i < TM; ++i)
            av[i] = ms[(2 * trow + 2 * NTR * (i >> 1) + (i & 1)) * LDM + kk];
          const float2* xrow = xs + b * BN;
          const int sw = (b & SWM) << 1;
#pragma unroll
          for (int j = 0; j < TN / 2; ++j) {
            const float4 v = *reinterpret_cast<const float4*>(
                xrow + ((2 * tcol + 2 * NTC * j) ^ sw));
            xv[2 * j] = make_float2(v.x, v.y);
            xv[2 * j + 1] = make_float2(v.z, v.w);
          }
#pragma unroll
          for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TN; ++j) acc[i][j] = cmad(av[i], xv[j], acc[i][j]);
        }
      }
    }

    if (!a.vec) {
      // outputs through shared memory, then out in input-address order
      __syncthreads();  // the tile is no longer read
#pragma unroll
      for (int i = 0; i < TM; ++i) {
        const int row = 2 * trow + 2 * NTR * (i >> 1) + (i & 1);
        float2* srow = xs + row * BN;
        const int sw = (row & SWM) << 1;
#pragma unroll
        for (int j = 0; j < TN / 2; ++j)
          *reinterpret_cast<float4*>(srow + ((2 * tcol + 2 * NTC * j) ^ sw)) =
              make_float4(acc[i][2 * j].x, acc[i][2 * j].y,
                          acc[i][2 * j + 1].x, acc[i][2 * j + 1].y);
      }
      __syncthreads();
#pragma unroll 8
      for (int i = 0; i < 32; ++i) {
        const int32_t x = t_ix + it_ix[i];
        const int b = x >> W::LBN, c = x & (BN - 1);
        if (c < cv)
          __stcs(dst + t_out + it_out[i], xs[b * BN + (c ^ ((b & SWM) << 1))]);
      }
      __syncthreads();  // the tile is no longer read
      continue;
    }
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      float2* drow = dst + r_t + a.rj[i] + c_t;
#pragma unroll
      for (int j = 0; j < TN / 2; ++j) {
        const int c = 2 * tcol + 2 * NTC * j;
        if (c >= cv) continue;
        float2* p = drow + a.cj[2 * j];
        if (a.vec) {
          __stcs(reinterpret_cast<float4*>(p),
                 make_float4(acc[i][2 * j].x, acc[i][2 * j].y,
                             acc[i][2 * j + 1].x, acc[i][2 * j + 1].y));
        } else {
          __stcs(p, acc[i][2 * j]);
          if (c + 1 < cv) __stcs(drow + a.cj[2 * j + 1], acc[i][2 * j + 1]);
        }
      }
    }
    __syncthreads();  // the tile and operator are no longer read
  }
}

// Fills WideArgs for dense_wide_kernel<K> and launches it.
template <int K>
static int launch_wide(const float2* in, float2* out, const float2* ops,
                       int n, int64_t num_states, int64_t in_stride,
                       int64_t op_stride, const int* pos, cudaStream_t st) {
  using W = WideCfg<K>;
  WideArgs a{};
  a.n = n;
  a.lgps = n - K;
  a.groups = (uint64_t)num_states << a.lgps;
  a.in_stride = in_stride;
  a.op_stride = op_stride;
  a.nspos = K;
  uint64_t tmask = 0;
  for (int j = 0; j < K; ++j) {
    a.spos[j] = pos[j];
    tmask |= uint64_t(1) << pos[j];
  }
  std::sort(a.spos, a.spos + K);
  for (int m = 0; m < K; ++m) a.boff[m] = int64_t(1) << pos[K - 1 - m];
  // tile column bit q: a group bit inside the state (the q-th position that
  // is not a target) or a state bit
  int64_t cin[9] = {0};
  int p = 0;
  for (int q = 0; q < W::LBN; ++q) {
    if (q < a.lgps) {
      while ((tmask >> p) & 1) ++p;
      cin[q] = a.cout[q] = int64_t(1) << p;
      ++p;
    } else {
      cin[q] = in_stride << (q - a.lgps);
      a.cout[q] = int64_t(1) << (n + q - a.lgps);
    }
  }
  // element bits sorted by input address (broadcast bits, offset 0, last)
  int64_t key[13];
  int ne = 0;
  for (int m = 0; m < K; ++m) {
    a.ein[ne] = a.boff[m];
    a.eout[ne] = a.boff[m];
    a.eix[ne++] = W::BN << m;
  }
  for (int q = 0; q < W::LBN; ++q) {
    a.ein[ne] = cin[q];
    a.eout[ne] = a.cout[q];
    a.eix[ne++] = 1 << q;
  }
  for (int j = 0; j < 13; ++j) key[j] = a.ein[j] ? a.ein[j] : INT64_MAX;
  for (int i = 1; i < 13; ++i)
    for (int j = i; j > 0 && key[j - 1] > key[j]; --j) {
      std::swap(key[j - 1], key[j]);
      std::swap(a.ein[j - 1], a.ein[j]);
      std::swap(a.eout[j - 1], a.eout[j]);
      std::swap(a.eix[j - 1], a.eix[j]);
    }
  for (int i = 0; i < W::TM; ++i) {
    const int r = 2 * W::NTR * (i >> 1) + (i & 1);
    int64_t o = 0;
    for (int m = 0; m < K; ++m)
      if ((r >> m) & 1) o += a.boff[m];
    a.rj[i] = o;
  }
  for (int j = 0; j < W::TN; ++j) {
    const int c = 2 * W::NTC * (j >> 1) + (j & 1);
    int64_t o = 0;
    for (int q = 0; q < W::LBN; ++q)
      if ((c >> q) & 1) o += a.cout[q];
    a.cj[j] = o;
  }
  a.vec = a.cout[0] == 1 && n >= 1 &&
          reinterpret_cast<uintptr_t>(out) % 16 == 0;

  // the shared-memory opt-in and the occupancy, once per device
  static std::atomic<int> per_sm_of[64];
  int dev = 0;
  cudaGetDevice(&dev);
  std::atomic<int>& per_sm = per_sm_of[dev & 63];
  int bps = per_sm.load(std::memory_order_relaxed);
  if (bps == 0) {
    cudaError_t e = cudaFuncSetAttribute(
        dense_wide_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
        (int)W::SMEM);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &bps, dense_wide_kernel<K>, 256, W::SMEM);
    if (e != cudaSuccess || bps < 1)
      return set_error(GBSV_ERR_CUDA, "dense_wide_kernel<%d> setup: %s", K,
                       cudaGetErrorString(e));
    per_sm.store(bps, std::memory_order_relaxed);
  }
  const uint64_t ntiles = (a.groups + W::BN - 1) >> W::LBN;
  uint64_t grid = (uint64_t)sm_count() * bps;
  if (grid > ntiles) grid = ntiles;
  dense_wide_kernel<K><<<(unsigned)grid, 256, W::SMEM, st>>>(in, out, ops, a);
  return after_launch("dense_wide_kernel");
}

// Whether dense_wide_kernel takes this operator: complex64, 4 <= k <= 12,
// one operator or a tile inside one state, and in place only over
// contiguous states.  Below 6 qubits the group kernel is the alternative:
// the tile kernel takes every 5-qubit operator (the group kernel's 32
// amplitudes per thread leave it at half the tile kernel's rate) and
// 4-qubit operators with a target among the three lowest bits (groups of
// contiguous amplitudes, where consecutive threads of the group kernel
// read lines 128 bytes or more apart).
static bool wide_applies(int dtype, int n, int k, int64_t num_states,
                         int64_t in_stride, int64_t op_stride,
                         bool in_place, const int* pos) {
  if (dtype != GBSV_C64 || k < 4 || k > 12 || n < k) return false;
  if (k == 4) {
    int lowest = 64;
    for (int j = 0; j < k; ++j) lowest = pos[j] < lowest ? pos[j] : lowest;
    if (lowest >= 3) return false;
  }
  const int lbn = 13 - k;
  if (op_stride != 0 && n - k < lbn) return false;
  if (in_place && num_states > 1 && in_stride != (int64_t(1) << n))
    return false;
  return true;
}

static int apply_wide(const void* in, void* out, int n, int64_t num_states,
                      int64_t in_stride, const void* ops, int64_t op_stride,
                      const int* pos, int k, cudaStream_t st) {
  const float2* i = static_cast<const float2*>(in);
  float2* o = static_cast<float2*>(out);
  const float2* m = static_cast<const float2*>(ops);
  switch (k) {
    case 4: return launch_wide<4>(i, o, m, n, num_states, in_stride, op_stride, pos, st);
    case 5: return launch_wide<5>(i, o, m, n, num_states, in_stride, op_stride, pos, st);
    case 6: return launch_wide<6>(i, o, m, n, num_states, in_stride, op_stride, pos, st);
    case 7: return launch_wide<7>(i, o, m, n, num_states, in_stride, op_stride, pos, st);
    case 8: return launch_wide<8>(i, o, m, n, num_states, in_stride, op_stride, pos, st);
    case 9: return launch_wide<9>(i, o, m, n, num_states, in_stride, op_stride, pos, st);
    case 10: return launch_wide<10>(i, o, m, n, num_states, in_stride, op_stride, pos, st);
    case 11: return launch_wide<11>(i, o, m, n, num_states, in_stride, op_stride, pos, st);
    default: return launch_wide<12>(i, o, m, n, num_states, in_stride, op_stride, pos, st);
  }
}

static int apply_generic(const void* in, void* out, int dtype, int n,
                         int64_t num_states, int64_t in_stride,
                         const void* ops, int64_t op_stride, const int* pos,
                         int k, cudaStream_t st) {
  if (wide_applies(dtype, n, k, num_states, in_stride, op_stride, in == out,
                   pos))
    return apply_wide(in, out, n, num_states, in_stride, ops, op_stride, pos,
                      k, st);
  GenericArgs a{};
  a.total = (uint64_t)num_states << n;
  a.n = n;
  a.k = k;
  a.df = c128_arith() == GBSV_C128_PAIRS;
  a.in_stride = in_stride;
  a.op_stride = op_stride;
  for (int j = 0; j < k; ++j) {
    a.pos[j] = pos[j];
    a.tmask |= uint64_t(1) << pos[j];
  }
  const int kmax_group = dtype == GBSV_C64 ? 5 : 4;
  const bool group = k >= 3 && k <= kmax_group && n >= k;
  // the one-output-per-thread kernel reads other threads' inputs
  if (!group && k >= 1 && in == out)
    return set_error(GBSV_ERR_UNSUPPORTED,
                     "a %d-qubit operator cannot be applied in place", k);
  if (group) {
    uint64_t groups = a.total >> k;
    uint64_t gb = (groups + 127) / 128;
    const uint64_t gcap = (uint64_t)sm_count() * 32;
    if (gb > gcap) gb = gcap;
    if (gb < 1) gb = 1;
#define GBSV_GROUP(R, KK)                                                  \
  dense_group_kernel<R, KK><<<(unsigned)gb, 128, 0, st>>>(                \
      static_cast<const Cx<R>*>(in), static_cast<Cx<R>*>(out),             \
      static_cast<const Cx<R>*>(ops), a)
    if (dtype == GBSV_C64) {
      if (k == 3) GBSV_GROUP(float, 3);
      else if (k == 4) GBSV_GROUP(float, 4);
      else GBSV_GROUP(float, 5);
    } else {
      if (k == 3) GBSV_GROUP(double, 3);
      else GBSV_GROUP(double, 4);
    }
#undef GBSV_GROUP
    return after_launch("dense_group_kernel");
  }
  const size_t smem = sizeof(uint64_t) << k;
  uint64_t blocks = (a.total + 255) / 256;
  const uint64_t cap = (uint64_t)sm_count() * 16;
  if (blocks > cap) blocks = cap;
  if (dtype == GBSV_C64)
    dense_generic_kernel<float><<<(unsigned)blocks, 256, smem, st>>>(
        static_cast<const float2*>(in), static_cast<float2*>(out),
        static_cast<const float2*>(ops), a);
  else
    dense_generic_kernel<double><<<(unsigned)blocks, 256, smem, st>>>(
        static_cast<const double2*>(in), static_cast<double2*>(out),
        static_cast<const double2*>(ops), a);
  return after_launch("dense_generic_kernel");
}

static int check_apply_args(const void* in, void* out, int dtype, int n,
                            int64_t num_states, int64_t in_stride,
                            const void* ops, int64_t op_stride) {
  if (dtype != GBSV_C64 && dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "state dtype %d is not complex",
                     dtype);
  if (n < 0 || n > 62)
    return set_error(GBSV_ERR_INVALID_ARG, "num_qubits %d out of range", n);
  if (num_states < 0 || in_stride < 0 || op_stride < 0)
    return set_error(GBSV_ERR_INVALID_ARG, "negative size or stride");
  if (num_states > 0 && (!in || !out || !ops))
    return set_error(GBSV_ERR_INVALID_ARG, "null pointer");
  return GBSV_OK;
}

}  // namespace gbsv

using namespace gbsv;

extern "C" int gbsv_apply_operator(const void* state_in, void* state_out,
                                   int dtype, int num_qubits,
                                   int64_t num_states, int64_t in_stride,
                                   const void* ops, int64_t op_stride,
                                   const int32_t* qubits, int num_targets,
                                   void* stream) {
  int rc = check_apply_args(state_in, state_out, dtype, num_qubits,
                            num_states, in_stride, ops, op_stride);
  if (rc) return rc;
  const int k = num_targets;
  if (k < 0 || k > num_qubits)
    return set_error(GBSV_ERR_INVALID_ARG,
                     "cannot apply a %d-qubit operator to %d qubits", k,
                     num_qubits);
  if (k > GBSV_MAX_DENSE_QUBITS)
    return set_error(GBSV_ERR_UNSUPPORTED,
                     "operators on more than %d qubits are not supported",
                     GBSV_MAX_DENSE_QUBITS);
  if (k > 0 && !qubits)
    return set_error(GBSV_ERR_INVALID_ARG, "null qubit list");
  int pos[GBSV_MAX_DENSE_QUBITS];
  uint64_t seen = 0;
  for (int j = 0; j < k; ++j) {
    const int q = qubits[j];
    if (q < 0 || q >= num_qubits)
      return set_error(GBSV_ERR_INVALID_ARG, "qubit %d out of range [0, %d)",
                       q, num_qubits);
    if ((seen >> q) & 1)
      return set_error(GBSV_ERR_INVALID_ARG, "qubit %d repeated", q);
    seen |= uint64_t(1) << q;
    pos[j] = num_qubits - 1 - q;
  }
  if (num_states == 0) return GBSV_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (k == 1 || k == 2)
    return apply_small(state_in, state_out, dtype, num_qubits, num_states,
                       in_stride, ops, op_stride, pos, k, st);
  return apply_generic(state_in, state_out, dtype, num_qubits, num_states,
                       in_stride, ops, op_stride, pos, k, st);
}

extern "C" int gbsv_apply_all_qubits(const void* state_in, void* state_out,
                                     int dtype, int num_qubits,
                                     int64_t num_states, int64_t in_stride,
                                     const void* ops, int64_t op_stride,
                                     int64_t op_qubit_stride, void* stream) {
  int rc = check_apply_args(state_in, state_out, dtype, num_qubits,
                            num_states, in_stride, ops, op_stride);
  if (rc) return rc;
  if (num_qubits < 1)
    return set_error(GBSV_ERR_INVALID_ARG,
                     "apply_all_qubits needs at least one qubit");
  if (op_qubit_stride < 0)
    return set_error(GBSV_ERR_INVALID_ARG, "negative operator qubit stride");
  if (num_states == 0) return GBSV_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int amp = dtype_bytes(dtype);
  const int64_t N = int64_t(1) << num_qubits;
  for (int q = 0; q < num_qubits; ++q) {
    const void* src = q == 0 ? state_in : state_out;
    const int64_t stride = q == 0 ? in_stride : N;
    const void* op =
        static_cast<const char*>(ops) + (int64_t)q * op_qubit_stride * amp;
    int pos = num_qubits - 1 - q;
    rc = apply_small(src, state_out, dtype, num_qubits, num_states, stride, op,
                     op_stride, &pos, 1, st);
    if (rc) return rc;
  }
  return GBSV_OK;
}

// ------------------------------------------------------------ apply_phase --
namespace gbsv {

struct PhaseArgs {
  uint64_t total;
  int ndim;
  int64_t shape[GBSV_MAX_DIMS];
  int64_t sa[GBSV_MAX_DIMS];
  int64_t sb[GBSV_MAX_DIMS];
  int df;  // double angles: double-float pairs (1) or FP64 (0)
};

// out = (cos t - i sin t) * psi.
template <typename RA, typename RS, typename RO>
__device__ __forceinline__ Cx<RO> phase_one(RA t, Cx<RS> v, int df) {
  // The phase factor is formed in the angle's precision, as torch forms
  // exp(-1j * angles) in complex(angles.dtype); the product is then taken
  // in the promoted output precision.
  if constexpr (sizeof(RA) == 8) {
    // double angles in pairs (df_sincos) when the angle is within 2^20 and
    // the amplitude within the pair range; FP64 otherwise
    uint32_t mx = 0;
    if constexpr (sizeof(RS) == 8)
      mx = max(df_hiword(v.x) & 0x7ff00000u, df_hiword(v.y) & 0x7ff00000u);
    const bool ok = df && (df_hiword(t) & 0x7ff00000u) <= ((1023u + 19) << 20) &&
                    (sizeof(RS) == 4 ||
                     (mx < ((DF_EMAX + 1) << 20) &&
                      (mx == 0 || mx >= (DF_EMIN << 20))));
    if (ok) {
      const DSC sc = df_sincos(t);
      DC a;
      if constexpr (sizeof(RS) == 8) {
        a = df_split2(v.x, v.y);
      } else {
        a.re = DF{(float)v.x, 0.f};
        a.im = DF{(float)v.y, 0.f};
      }
      const DF re = df_sum2(df_prod2(sc.c, a.re), df_prod2(sc.s, a.im));
      const DF im = df_sum2(df_prod2(sc.c, a.im), df_neg(df_prod2(sc.s, a.re)));
      Cx<RO> o;
      o.x = df_join(re);
      o.y = df_join(im);
      return o;
    }
  }
  RA sa, ca;
  sincos(t, &sa, &ca);
  const RO s = (RO)sa, c = (RO)ca;
  const RO x = (RO)v.x, y = (RO)v.y;
  Cx<RO> o;
  o.x = c * x + s * y;
  o.y = c * y - s * x;
  return o;
}

template <typename RA, typename RS, typename RO, int NDIM>
__global__ void __launch_bounds__(256)
    phase_kernel(const RA* ang, const Cx<RS>* psi, Cx<RO>* out, PhaseArgs a) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if constexpr (NDIM == 1) {
    // four elements per thread, all loads issued before the sincos work
    const int64_t s0 = a.sa[0], s1 = a.sb[0];
    for (; i + 3 * stride < a.total; i += 4 * stride) {
      RA t[4];
      Cx<RS> v[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        t[k] = ang[(int64_t)(i + k * stride) * s0];
        v[k] = psi[(int64_t)(i + k * stride) * s1];
      }
#pragma unroll
      for (int k = 0; k < 4; ++k)
        out[i + k * stride] = phase_one<RA, RS, RO>(t[k], v[k], a.df);
    }
  }
  for (; i < a.total; i += stride) {
    int64_t oa = 0, ob = 0;
    if constexpr (NDIM == 1) {
      oa = (int64_t)i * a.sa[0];
      ob = (int64_t)i * a.sb[0];
    } else {
      uint64_t r = i;
      for (int d = a.ndim - 1; d >= 0; --d) {
        const uint64_t sz = (uint64_t)a.shape[d];
        const uint64_t idx = r % sz;
        r /= sz;
        oa += (int64_t)idx * a.sa[d];
        ob += (int64_t)idx * a.sb[d];
      }
    }
    out[i] = phase_one<RA, RS, RO>(ang[oa], psi[ob], a.df);
  }
}

template <typename RA, typename RS, typename RO>
static int launch_phase(const void* ang, const void* psi, void* out,
                        const PhaseArgs& a, cudaStream_t st) {
  uint64_t blocks = (a.total + 255) / 256;
  const uint64_t cap = (uint64_t)sm_count() * 32;
  if (blocks > cap) blocks = cap;
  if (a.ndim == 1)
    phase_kernel<RA, RS, RO, 1><<<(unsigned)blocks, 256, 0, st>>>(
        static_cast<const RA*>(ang), static_cast<const Cx<RS>*>(psi),
        static_cast<Cx<RO>*>(out), a);
  else
    phase_kernel<RA, RS, RO, 0><<<(unsigned)blocks, 256, 0, st>>>(
        static_cast<const RA*>(ang), static_cast<const Cx<RS>*>(psi),
        static_cast<Cx<RO>*>(out), a);
  return after_launch("phase_kernel");
}

}  // namespace gbsv

extern "C" int gbsv_apply_phase(const void* angles, int angle_dtype,
                                const void* state, int state_dtype, void* out,
                                int out_dtype, const gbsv_bcast_t* bc,
                                void* stream) {
  if (!bc || bc->ndim < 1 || bc->ndim > GBSV_MAX_DIMS)
    return set_error(GBSV_ERR_INVALID_ARG, "bad broadcast descriptor");
  if (angle_dtype != GBSV_F32 && angle_dtype != GBSV_F64)
    return set_error(GBSV_ERR_INVALID_ARG, "angles must be float32/float64");
  if (state_dtype != GBSV_C64 && state_dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "state must be complex");
  const int want = (angle_dtype == GBSV_F64 || state_dtype == GBSV_C128)
                       ? GBSV_C128
                       : GBSV_C64;
  if (out_dtype != want)
    return set_error(GBSV_ERR_INVALID_ARG,
                     "output dtype %d is not the promoted type %d", out_dtype,
                     want);
  PhaseArgs a{};
  a.df = c128_arith() == GBSV_C128_PAIRS;
  a.ndim = bc->ndim;
  uint64_t total = 1;
  for (int d = 0; d < bc->ndim; ++d) {
    if (bc->shape[d] < 0)
      return set_error(GBSV_ERR_INVALID_ARG, "negative extent");
    a.shape[d] = bc->shape[d];
    a.sa[d] = bc->stride_a[d];
    a.sb[d] = bc->stride_b[d];
    total *= (uint64_t)bc->shape[d];
  }
  a.total = total;
  if (total == 0) return GBSV_OK;
  if (!angles || !state || !out)
    return set_error(GBSV_ERR_INVALID_ARG, "null pointer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (angle_dtype == GBSV_F32 && state_dtype == GBSV_C64)
    return launch_phase<float, float, float>(angles, state, out, a, st);
  if (angle_dtype == GBSV_F64 && state_dtype == GBSV_C64)
    return launch_phase<double, float, double>(angles, state, out, a, st);
  if (angle_dtype == GBSV_F32 && state_dtype == GBSV_C128)
    return launch_phase<float, double, double>(angles, state, out, a, st);
  return launch_phase<double, double, double>(angles, state, out, a, st);
}
