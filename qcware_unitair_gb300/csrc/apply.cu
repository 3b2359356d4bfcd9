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
#include <stdio.h>

#include <algorithm>

#include "common.cuh"

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

// complex128: GB300 issues FP64 at a small fraction of its FP32 rate, so a
// gate's FP64 work, not HBM, bounded the complex128 path.  The matrix's
// kind (permutation, diagonal, anti-diagonal, real, real diagonal with
// imaginary off-diagonal, controlled 2x2, general) is found once per thread
// and each kind runs its own loop with only the FP64 operations it needs.
// The kind is the same for a whole warp when the operator is shared, and
// the loops are too large to be turned into selects, so no FP64 work is
// issued for the other kinds.  Roundings are those of cmul / cmad.
constexpr int EC_ZERO = 0, EC_ONE = 1, EC_REAL = 2, EC_IMAG = 3,
              EC_FULL = 4;

// From the bit patterns (integer compares: an FP64 compare costs an FP64
// issue slot; +0 and -0 are both zero)
template <typename C>
__device__ __forceinline__ int entry_class(const C& m) {
  const unsigned long long xb = __double_as_longlong(m.x);
  const unsigned long long yb = __double_as_longlong(m.y);
  const bool xz = (xb << 1) == 0, yz = (yb << 1) == 0;
  if (yz) return xz ? EC_ZERO : (xb == 0x3FF0000000000000ull ? EC_ONE : EC_REAL);
  return xz ? EC_IMAG : EC_FULL;
}

// r[i] *= m for the registers i with (i & MASK) == PAT
template <typename C, int NR, int MASK, int PAT>
__device__ __forceinline__ void scale_sel(C* r, const C& m, int cls) {
  switch (cls) {
    case EC_ONE:
      return;
    case EC_ZERO:
#pragma unroll
      for (int i = 0; i < NR; ++i)
        if ((i & MASK) == PAT) r[i].x = r[i].y = 0;
      return;
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
    default:
#pragma unroll
      for (int i = 0; i < NR; ++i)
        if ((i & MASK) == PAT) r[i] = cmul(m, r[i]);
      return;
  }
}

constexpr int K1_PERM = 0, K1_DIAG = 1, K1_ANTI = 2, K1_REAL = 3,
              K1_RX = 4, K1_FULL = 5;

__device__ __forceinline__ int kind_2x2(int c0, int c1, int c2, int c3) {
  if (c1 == EC_ZERO && c2 == EC_ZERO) return K1_DIAG;
  if (c0 == EC_ZERO && c3 == EC_ZERO)
    return c1 == EC_ONE && c2 == EC_ONE ? K1_PERM : K1_ANTI;
  const bool re = c0 <= EC_REAL && c1 <= EC_REAL && c2 <= EC_REAL &&
                  c3 <= EC_REAL;
  if (re) return K1_REAL;
  if (c0 <= EC_REAL && c3 <= EC_REAL && c1 == EC_IMAG && c2 == EC_IMAG)
    return K1_RX;
  return K1_FULL;
}

// The 2x2 (m0 m1; m2 m3) on register bit T, for the registers i with
// (i & CM) == CV (a control pattern; 0, 0 for none).
template <typename C, int NR, int T, int CM, int CV>
__device__ __forceinline__ void apply_2x2(C* r, const C& m0, const C& m1,
                                          const C& m2, const C& m3, int kind,
                                          int c0, int c3) {
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
      scale_sel<C, NR, B | CM, CV>(r, m0, c0);
      scale_sel<C, NR, B | CM, B | CV>(r, m3, c3);
      return;
    case K1_ANTI:
#pragma unroll
      for (int i = 0; i < NR; ++i) {
        if ((i & B) || (i & CM) != CV) continue;
        const C a0 = r[i], a1 = r[i | B];
        r[i] = cmul(m1, a1);
        r[i | B] = cmul(m2, a0);
      }
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

// Precomputed structure of a complex128 operator (see apply_c128).
struct OpKind {
  int kind;     // K1_* for 2x2; for 4x4: 0 general, 1 permutation,
                // 2 diagonal, 3 controlled 2x2
  int sub;      // 4x4 controlled: K1_* of the 2x2 block
  int c[4];     // classes of the four diagonal (or block) entries
  int perm;     // 4x4 permutation: source column of row j in bits 2j..2j+1
};

template <typename C, int K>
__device__ __forceinline__ OpKind classify_op(const C* m) {
  OpKind k{};
  if constexpr (K == 1) {
    const int c0 = entry_class(m[0]), c1 = entry_class(m[1]),
              c2 = entry_class(m[2]), c3 = entry_class(m[3]);
    k.kind = kind_2x2(c0, c1, c2, c3);
    k.c[0] = c0;
    k.c[3] = c3;
    return k;
  } else {
    int cl[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) cl[j] = entry_class(m[j]);
    bool diag = true, perm = true, ctrl = true;
    int pm = 0;
#pragma unroll
    for (int row = 0; row < 4; ++row) {
      int ones = 0, nz = 0, col = 0;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = cl[4 * row + j];
        if (c != EC_ZERO) {
          ++nz;
          col = j;
          if (c == EC_ONE) ++ones;
          if (j != row) diag = false;
          // controlled: identity on rows 0, 1; rows 2, 3 inside cols 2, 3
          if (row < 2 ? (j != row || c != EC_ONE) : j < 2) ctrl = false;
        } else if (row < 2 && j == row) {
          ctrl = false;
        }
      }
      if (!(nz == 1 && ones == 1)) perm = false;
      pm |= col << (2 * row);
    }
    if (perm) {
      k.kind = 1;
      k.perm = pm;
    } else if (diag) {
      k.kind = 2;
#pragma unroll
      for (int j = 0; j < 4; ++j) k.c[j] = cl[5 * j];
    } else if (ctrl) {
      k.kind = 3;
      k.sub = kind_2x2(cl[10], cl[11], cl[14], cl[15]);
      k.c[0] = cl[10];
      k.c[3] = cl[15];
    } else {
      k.kind = 0;
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

// Matrix index bit 1 (K = 2: the first target) is register bit RB0, bit 0
// register bit RB1.
template <typename C, int NR, int K, int RB0, int RB1>
__device__ __forceinline__ void apply_c128(C* r, const C* m,
                                           const OpKind& k) {
  if constexpr (K == 1) {
    apply_2x2<C, NR, RB0, 0, 0>(r, m[0], m[1], m[2], m[3], k.kind, k.c[0],
                                k.c[3]);
  } else {
    constexpr int M0 = 1 << RB0, M1 = 1 << RB1;
    switch (k.kind) {
      case 1:  // permutation: row j takes column perm_j
#pragma unroll
        for (int i = 0; i < NR; ++i) {
          if (i & (M0 | M1)) continue;
          const int idx[4] = {i, i | M1, i | M0, i | M0 | M1};
          C v[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) v[j] = r[idx[j]];
#pragma unroll
          for (int j = 0; j < 4; ++j)
            r[idx[j]] = pick4(v, (k.perm >> (2 * j)) & 3);
        }
        return;
      case 2:  // diagonal
        scale_sel<C, NR, M0 | M1, 0>(r, m[0], k.c[0]);
        scale_sel<C, NR, M0 | M1, M1>(r, m[5], k.c[1]);
        scale_sel<C, NR, M0 | M1, M0>(r, m[10], k.c[2]);
        scale_sel<C, NR, M0 | M1, M0 | M1>(r, m[15], k.c[3]);
        return;
      case 3:  // controlled: the lower-right 2x2 where bit RB0 is set
        apply_2x2<C, NR, RB1, M0, M0>(r, m[10], m[11], m[14], m[15], k.sub,
                                      k.c[0], k.c[3]);
        return;
      default:
        apply_regs<C, NR, K, RB0, RB1>(r, m);
        return;
    }
  }
}

// NH high targets (chunks per unit = 2^NH); RB0 / RB1 are the register-index
// bits of the first / second target in matrix order.
template <typename R, int V, int K, int NH, int RB0, int RB1>
__global__ void __launch_bounds__(256, 2)
    dense_chunk_kernel(const Cx<R>* in, Cx<R>* out, const Cx<R>* ops,
                       DenseArgs a) {
  using C = Cx<R>;
  constexpr int NCH = 1 << NH;
  constexpr int NR = NCH * V;
  constexpr int D = 1 << K;
  constexpr int TARGET = sizeof(R) == 4 ? 16 : 8;  // amplitudes per thread
  constexpr int UNROLL = NR >= TARGET ? 1 : TARGET / NR;

  C m[D * D];
  OpKind kind{};  // complex128: the operator's structure
  constexpr bool kClassed = sizeof(R) == 8;
  const bool shared_op = a.op_stride == 0;
  if (shared_op) {
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

  // complex128 with a shared operator: classified while the state loads
  // are in flight, then one structured pass over every unit's registers
  // (the target bits index within each unit's NR block; registers of units
  // past the end are computed and not stored)
  if constexpr (kClassed) {
    if (shared_op) {
      kind = classify_op<C, K>(m);
      apply_c128<C, UNROLL * NR, K, RB0, RB1>(&reg[0][0], m, kind);
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
    } else if constexpr (!kClassed) {
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

// Any k <= GBSV_MAX_DENSE_QUBITS: one thread per output amplitude,
// out[i] = sum_b M[row(i), b] * in[base(i) + offs[b]].  Used for k = 0 and
// k >= 3, where no configuration of the engine is bandwidth-critical.
struct GenericArgs {
  uint64_t total;  // num_states << n
  int n;
  int k;
  int64_t in_stride;
  int64_t op_stride;
  uint64_t tmask;       // bits of the target positions
  int pos[GBSV_MAX_DENSE_QUBITS];  // position of matrix bit (k-1-j)
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
// registers).  The thread reads its group once (consecutive threads take consecutive groups,
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
  if (shared_op)
    for (int i = tid; i < D * D; i += blockDim.x) msm[i] = ops[i];
  __syncthreads();
  const int n = a.n;
  const uint64_t gps = uint64_t(1) << (n - K);  // groups per state
  const uint64_t total = (a.total >> n) * gps;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
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
  constexpr int TARGET = sizeof(R) == 4 ? 16 : 8;
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
  if (dtype == GBSV_C64)
    return dispatch_chunk<float>(V, k, nh, rb[0], rb[1], in, out, ops, a, st);
  return dispatch_chunk<double>(V, k, nh, rb[0], rb[1], in, out, ops, a, st);
}

static int apply_generic(const void* in, void* out, int dtype, int n,
                         int64_t num_states, int64_t in_stride,
                         const void* ops, int64_t op_stride, const int* pos,
                         int k, cudaStream_t st) {
  GenericArgs a{};
  a.total = (uint64_t)num_states << n;
  a.n = n;
  a.k = k;
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
};

// out = (cos t - i sin t) * psi.
template <typename RA, typename RS, typename RO>
__device__ __forceinline__ Cx<RO> phase_one(RA t, Cx<RS> v) {
  // The phase factor is formed in the angle's precision, as torch forms
  // exp(-1j * angles) in complex(angles.dtype); the product is then taken
  // in the promoted output precision.
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
        out[i + k * stride] = phase_one<RA, RS, RO>(t[k], v[k]);
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
    out[i] = phase_one<RA, RS, RO>(ang[oa], psi[ob]);
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
