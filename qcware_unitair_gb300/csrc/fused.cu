// Fused gate stages: one HBM pass applies a run of gates.
//
// A stage picks m "tile bits": the c lowest amplitude-index bits (so a tile
// is made of 2^(m-c) runs of 2^c contiguous amplitudes, >= 128 bytes) plus
// m - c arbitrary higher bits.  Every assignment of the other n - m bits
// names one tile of 2^m amplitudes.  A CTA copies its tile into shared
// memory (16-byte cp.async), applies every gate of the stage there, and
// writes the tile back, so the stage costs one read and one write of the
// state however many gates it holds.  A gate can join a stage when
//   * its non-diagonal targets are tile bits (dense 1- and 2-qubit gates),
//   * its controls outside the tile become a per-tile condition, and
//   * diagonal gates may sit anywhere: on tile bits they scale amplitudes,
//     on bits outside the tile they are one complex factor per tile.
// The host planner (fusion.py) builds the stages; whole states of up to m
// qubits are a single tile, so a whole circuit on them is one launch.
//
// Shared memory holds the tile with a 16-byte-unit XOR swizzle
// (unit u = l >> 1 is stored at u ^ ((u >> 3) & 7)) so pair updates on any
// tile bit stay within the 2-wavefront minimum per warp.
#include "common.cuh"

namespace gbsv {

constexpr int FG_DENSE1 = 0;  // 2x2 on local bit b0
constexpr int FG_DENSE2 = 1;  // 4x4 on local bits b0 (matrix MSB), b1
constexpr int FG_DIAG = 2;    // diagonal on 1-2 qubits, local or global
constexpr int FG_MAX_TILE_BITS = 14;


struct StageArgs {
  int n, m, c;
  int64_t num_states;
  int64_t in_stride;          // amplitudes between input states (0 = bcast)
  int hpos[FG_MAX_TILE_BITS];  // global position of local bit c + j
  int spos[FG_MAX_TILE_BITS];  // all m tile positions, ascending
  const FusedGate* gates;
  int num_gates;
};

__device__ __forceinline__ int swz(int l) {
  const int u = l >> 1;
  return ((u ^ ((u >> 3) & 7)) << 1) | (l & 1);
}


// A stage's gates are copied into shared memory in chunks (records plus this
// CTA's matrix values), so applying a gate never waits on global memory.
constexpr int GCHUNK = 32;

template <typename C>
struct SGate {
  int32_t kind, nq, b0, b1;
  uint64_t cmask, cval;
  C m[16];
};

template <typename C>
__device__ __forceinline__ void load_gate_chunk(SGate<C>* sg,
                                                const FusedGate* gates,
                                                const C* pool, uint64_t s,
                                                int first, int count) {
  for (int idx = threadIdx.x; idx < count * 17; idx += blockDim.x) {
    const int gi = idx / 17, slot = idx % 17;
    const FusedGate& g = gates[first + gi];
    if (slot == 0) {
      sg[gi].kind = g.kind;
      sg[gi].nq = g.nq;
      sg[gi].b0 = g.b0;
      sg[gi].b1 = g.b1;
      sg[gi].cmask = g.cmask;
      sg[gi].cval = g.cval;
    } else {
      // kinds 7 (a 4x4 permutation) and 8 (register diagonal) are the
      // register-blocked FG_PERM2 / FG_RDIAG declared below
      const int nvals = (g.kind == FG_DENSE2 || g.kind == 7) ? 16
                        : (g.kind == FG_DIAG || g.kind == 8) ? (1 << g.nq)
                                                             : 4;
      if (slot - 1 < nvals)
        sg[gi].m[slot - 1] =
            pool[g.mat + (int64_t)s * g.mat_bstride + (slot - 1)];
    }
  }
}

// Apply gates[0 .. num_gates) to the tile S (2^m amplitudes, swizzled for
// complex64) of state s whose base index is `base`; gates on bits outside
// the tile become per-tile factors accumulated into tscale.
template <typename R>
__device__ __forceinline__ void run_gates_smem(Cx<R>* S, int M, uint64_t base,
                                               uint64_t s,
                                               const FusedGate* gates,
                                               int num_gates,
                                               const Cx<R>* pool,
                                               Cx<R>& tscale, bool& scaled) {
  using C = Cx<R>;
  constexpr int PER = 16 / sizeof(C);
  const int T = blockDim.x;
  const int tid = threadIdx.x;
  __shared__ SGate<C> sg[GCHUNK];
  for (int c0 = 0; c0 < num_gates; c0 += GCHUNK) {
    const int cnt = min(GCHUNK, num_gates - c0);
    if (c0 > 0) __syncthreads();
    load_gate_chunk<C>(sg, gates, pool, s, c0, cnt);
    __syncthreads();
    for (int gi = 0; gi < cnt; ++gi) {
      const SGate<C>& g = sg[gi];
      if ((base & g.cmask) != g.cval) continue;  // uniform across the CTA
      int gidx = 0, lb0 = -1, lb1 = -1;
      if (g.kind == FG_DIAG) {
        // index bits of qubits outside the tile come from the tile base
        for (int q = 0; q < g.nq; ++q) {
          const int b = q == 0 ? g.b0 : g.b1;
          if (b < 0)
            gidx |= (int)((base >> (-1 - b)) & 1) << (g.nq - 1 - q);
          else if (q == 0)
            lb0 = b;
          else
            lb1 = b;
        }
        if (lb0 < 0 && lb1 < 0) {
          tscale = cmul(tscale, g.m[gidx]);
          scaled = true;
          continue;  // a per-tile factor: no shared-memory pass
        }
      }
      if (g.kind == FG_DENSE1) {
        const C m0 = g.m[0], m1 = g.m[1], m2 = g.m[2], m3 = g.m[3];
        const int b = g.b0;
        for (int j = tid; j < (M >> 1); j += T) {
          const int i0 = (int)insert_zero((uint64_t)j, b);
          const int i1 = i0 | (1 << b);
          const int p0 = PER == 2 ? swz(i0) : i0;
          const int p1 = PER == 2 ? swz(i1) : i1;
          const C x0 = S[p0], x1 = S[p1];
          S[p0] = cmad(m1, x1, cmul(m0, x0));
          S[p1] = cmad(m3, x1, cmul(m2, x0));
        }
      } else if (g.kind == FG_DENSE2) {
        const int hi = g.b0 > g.b1 ? g.b0 : g.b1;
        const int lo = g.b0 > g.b1 ? g.b1 : g.b0;
        const int M0 = 1 << g.b0, M1 = 1 << g.b1;
        const volatile C* vm = g.m;
        for (int j = tid; j < (M >> 2); j += T) {
          const int i = (int)insert_zero(insert_zero((uint64_t)j, lo), hi);
          int p[4] = {i, i | M1, i | M0, i | M0 | M1};
          C v[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            if (PER == 2) p[k] = swz(p[k]);
            v[k] = S[p[k]];
          }
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            C e[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              e[k].x = vm[4 * r + k].x;
              e[k].y = vm[4 * r + k].y;
            }
            C acc = cmul(e[0], v[0]);
            acc = cmad(e[1], v[1], acc);
            acc = cmad(e[2], v[2], acc);
            acc = cmad(e[3], v[3], acc);
            S[p[r]] = acc;
          }
        }
      } else {  // FG_DIAG with at least one tile qubit
        const C d0 = g.m[0], d1 = g.m[1];
        const C d2 = g.nq == 2 ? g.m[2] : d0, d3 = g.nq == 2 ? g.m[3] : d1;
        for (int l = tid; l < M; l += T) {
          int idx = gidx;
          if (lb0 >= 0) idx |= ((l >> lb0) & 1) << (g.nq - 1);
          if (lb1 >= 0) idx |= ((l >> lb1) & 1);
          const C f = idx == 0 ? d0 : idx == 1 ? d1 : idx == 2 ? d2 : d3;
          const int pl = PER == 2 ? swz(l) : l;
          S[pl] = cmul(f, S[pl]);
        }
      }
      __syncthreads();
    }
  }

}

template <typename R>
__global__ void __launch_bounds__(512, 2)
    fused_stage_kernel(const Cx<R>* in, Cx<R>* out, const Cx<R>* pool,
                       StageArgs a) {
  using C = Cx<R>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* S = reinterpret_cast<C*>(smem_raw);
  const int T = blockDim.x;
  const int tid = threadIdx.x;
  const int M = 1 << a.m;
  const int run = 1 << a.c;
  const uint64_t tiles_per_state = uint64_t(1) << (a.n - a.m);
  const uint64_t s = blockIdx.x / tiles_per_state;
  uint64_t base = blockIdx.x % tiles_per_state;
  for (int j = 0; j < a.m; ++j) base = insert_zero(base, a.spos[j]);

  const C* src = in + s * a.in_stride + base;
  C* dst = out + (s << a.n) + base;

  // ---- load: 16-byte pieces; a piece never crosses a run --------------
  constexpr int PER = 16 / sizeof(C);  // amplitudes per 16-byte piece
  for (int l = tid * PER; l < M; l += T * PER) {
    const int r = l >> a.c;
    uint64_t off = (uint64_t)(l & (run - 1));
    for (int j = 0; j < a.m - a.c; ++j)
      if ((r >> j) & 1) off += uint64_t(1) << a.hpos[j];
    if constexpr (PER == 2)
      cp_async16<R>(&S[swz(l)], src + off);
    else
      cp_async16<R>(&S[l], src + off);
  }
  cp_async_wait_all();
  __syncthreads();

  C tscale;
  tscale.x = 1;
  tscale.y = 0;
  bool scaled = false;

  run_gates_smem<R>(S, M, base, s, a.gates, a.num_gates, pool, tscale,
                    scaled);

  // ---- store --------------------------------------------------------
  for (int l = tid * PER; l < M; l += T * PER) {
    const int r = l >> a.c;
    uint64_t off = (uint64_t)(l & (run - 1));
    for (int j = 0; j < a.m - a.c; ++j)
      if ((r >> j) & 1) off += uint64_t(1) << a.hpos[j];
    const int pl = PER == 2 ? swz(l) : l;
    C v0 = S[pl];
    if (scaled) v0 = cmul(tscale, v0);
    if constexpr (PER == 2) {
      C v1 = S[pl + 1];
      if (scaled) v1 = cmul(tscale, v1);
      __stcs(reinterpret_cast<float4*>(dst + off),
             make_float4(v0.x, v0.y, v1.x, v1.y));
    } else {
      __stcs(dst + off, v0);
    }
  }
}

}  // namespace gbsv

using namespace gbsv;

extern "C" int gbsv_fused_max_tile_qubits(int dtype) {
  return dtype == GBSV_C64 ? 14 : 13;
}

extern "C" int gbsv_run_stage(const void* state_in, void* state_out, int dtype,
                              int num_qubits, int64_t num_states,
                              int64_t in_stride, int tile_qubits,
                              int contiguous_qubits,
                              const int32_t* tile_positions,
                              const void* gates, int num_gates,
                              const void* pool, void* stream) {
  if (dtype != GBSV_C64 && dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "state dtype must be complex");
  const int n = num_qubits, m = tile_qubits, c = contiguous_qubits;
  const int mmax = gbsv_fused_max_tile_qubits(dtype);
  const int cmin = dtype == GBSV_C64 ? 1 : 0;  // a 16-byte piece per run
  if (n < 1 || n > 62 || m < 1 || m > mmax || m > n || c < cmin || c > m)
    return set_error(GBSV_ERR_INVALID_ARG,
                     "bad stage shape n=%d m=%d c=%d (max m %d)", n, m, c,
                     mmax);
  if (num_states < 0 || in_stride < 0 || num_gates < 0)
    return set_error(GBSV_ERR_INVALID_ARG, "negative size");
  if (num_states == 0) return GBSV_OK;
  if (!state_in || !state_out || !tile_positions ||
      (num_gates > 0 && (!gates || !pool)))
    return set_error(GBSV_ERR_INVALID_ARG, "null pointer");
  const int amp = dtype_bytes(dtype);
  if ((uintptr_t)state_in % 16 || (uintptr_t)state_out % 16 ||
      (in_stride * amp) % 16)
    return set_error(GBSV_ERR_INVALID_ARG, "states must be 16-byte aligned");
  StageArgs a{};
  a.n = n;
  a.m = m;
  a.c = c;
  a.num_states = num_states;
  a.in_stride = in_stride;
  a.gates = static_cast<const FusedGate*>(gates);
  a.num_gates = num_gates;
  uint64_t seen = 0;
  for (int j = 0; j < m; ++j) {
    const int p = tile_positions[j];
    if (p < 0 || p >= n || ((seen >> p) & 1))
      return set_error(GBSV_ERR_INVALID_ARG, "bad tile position %d", p);
    if (j < c && p != j)
      return set_error(GBSV_ERR_INVALID_ARG,
                       "tile positions must start with 0..c-1");
    seen |= uint64_t(1) << p;
    if (j >= c) a.hpos[j - c] = p;
    a.spos[j] = p;
  }
  for (int i = 1; i < m; ++i)
    for (int j = i; j > 0 && a.spos[j - 1] > a.spos[j]; --j) {
      const int t = a.spos[j];
      a.spos[j] = a.spos[j - 1];
      a.spos[j - 1] = t;
    }
  const uint64_t blocks = (uint64_t)num_states << (n - m);
  if (blocks > 0x7fffffffull)
    return set_error(GBSV_ERR_UNSUPPORTED, "too many tiles");
  const size_t smem = (size_t)amp << m;
  int threads = (1 << m) / 4;
  if (threads > 512) threads = 512;
  if (threads < 32) threads = 32;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == GBSV_C64) {
    static bool attr_set = false;
    if (!attr_set) {
      cudaFuncSetAttribute(fused_stage_kernel<float>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(sizeof(float2) << mmax));
      attr_set = true;
    }
    fused_stage_kernel<float><<<(unsigned)blocks, threads, smem, st>>>(
        static_cast<const float2*>(state_in), static_cast<float2*>(state_out),
        static_cast<const float2*>(pool), a);
  } else {
    static bool attr_set = false;
    if (!attr_set) {
      cudaFuncSetAttribute(fused_stage_kernel<double>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(sizeof(double2) << mmax));
      attr_set = true;
    }
    fused_stage_kernel<double><<<(unsigned)blocks, threads, smem, st>>>(
        static_cast<const double2*>(state_in),
        static_cast<double2*>(state_out), static_cast<const double2*>(pool),
        a);
  }
  return after_launch("fused_stage_kernel");
}

// ---------------------------------------------------------------------------
// Register-blocked stages.  Same tiles and HBM traffic as above, but each of
// the 2^(m-RB) threads holds 2^RB amplitudes of the tile in registers.  A
// "layout" names RB tile bits that index a thread's registers; the other
// m - RB tile bits are the thread index.  Within a layout
//   * dense gates on register bits run in registers,
//   * diagonal gates need no particular layout (each register knows its
//     full tile index),
//   * a control on a thread bit is a per-thread condition,
// so shared memory is read and written once per layout instead of once per
// gate.  The host planner groups a stage's gates into layouts.
namespace gbsv {

constexpr int FG_CDENSE1 = 3;  // 2x2 on register bit b0 if tile bit b1 is 1
constexpr int FG_REAL1 = 4;    // real 2x2 on register bit b0 (H, RY)
constexpr int FG_ANTI1 = 5;    // [[0, a], [b, 0]] on register bit b0 (X, Y);
                               //   nq == 1 marks a == b == 1 (a pure swap)
constexpr int FG_CANTI1 = 6;   // FG_ANTI1 where tile bit b1 is 1 (CNOT)
constexpr int FG_PERM2 = 7;    // 4x4 permutation on register bits b0, b1;
                               //   nq packs the source of each output row
constexpr int FG_RDIAG = 8;    // diagonal on nq qubits, each encoded as a
                               //   register bit (0..RB-1), RB + thread tile
                               //   bit, or -1 - position outside the tile
constexpr int LAYOUT_MAX_RB = 5;

struct Layout {
  int32_t rb[LAYOUT_MAX_RB];  // tile bits of register-index bits 0..RB-1
  int32_t first_gate;
  int32_t num_gates;
  int32_t pad_;
};

struct Stage2Args {
  int n, m, c;
  int64_t in_stride;
  int hpos[FG_MAX_TILE_BITS];
  int spos[FG_MAX_TILE_BITS];
  const FusedGate* gates;
  const Layout* layouts;
  int num_layouts;
};

template <typename C, int NR, int K>
__device__ __forceinline__ void reg_apply1(C* v, const C& m0, const C& m1,
                                           const C& m2, const C& m3) {
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if ((i >> K) & 1) continue;
    const C x0 = v[i], x1 = v[i | (1 << K)];
    v[i] = cmad(m1, x1, cmul(m0, x0));
    v[i | (1 << K)] = cmad(m3, x1, cmul(m2, x0));
  }
}

// mm points to shared memory and is read volatile at each use, so the 16
// matrix entries never occupy registers.
template <typename C, int NR, int K0, int K1>
__device__ __forceinline__ void reg_apply2(C* v, const volatile C* mm) {
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if ((i >> K0) & 1 || (i >> K1) & 1) continue;
    const int idx[4] = {i, i | (1 << K1), i | (1 << K0),
                        i | (1 << K0) | (1 << K1)};
    C x[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) x[k] = v[idx[k]];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      C e[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        e[k].x = mm[4 * r + k].x;
        e[k].y = mm[4 * r + k].y;
      }
      C acc = cmul(e[0], x[0]);
      acc = cmad(e[1], x[1], acc);
      acc = cmad(e[2], x[2], acc);
      acc = cmad(e[3], x[3], acc);
      v[idx[r]] = acc;
    }
  }
}

template <typename C, int NR, int K>
__device__ __forceinline__ void reg_real1(C* v, float a00, float a01,
                                          float a10, float a11) {
  using R = decltype(C().x);
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if ((i >> K) & 1) continue;
    const C x0 = v[i], x1 = v[i | (1 << K)];
    C y0, y1;
    y0.x = (R)a00 * x0.x + (R)a01 * x1.x;
    y0.y = (R)a00 * x0.y + (R)a01 * x1.y;
    y1.x = (R)a10 * x0.x + (R)a11 * x1.x;
    y1.y = (R)a10 * x0.y + (R)a11 * x1.y;
    v[i] = y0;
    v[i | (1 << K)] = y1;
  }
}

template <typename C, int NR, int K>
__device__ __forceinline__ void reg_real1d(C* v, double a00, double a01,
                                           double a10, double a11) {
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if ((i >> K) & 1) continue;
    const C x0 = v[i], x1 = v[i | (1 << K)];
    C y0, y1;
    y0.x = a00 * x0.x + a01 * x1.x;
    y0.y = a00 * x0.y + a01 * x1.y;
    y1.x = a10 * x0.x + a11 * x1.x;
    y1.y = a10 * x0.y + a11 * x1.y;
    v[i] = y0;
    v[i | (1 << K)] = y1;
  }
}

// [[0, a], [b, 0]]: out0 = a x1, out1 = b x0 (a plain swap when unit)
template <typename C, int NR, int K>
__device__ __forceinline__ void reg_anti1(C* v, bool unit, const C& a,
                                          const C& b) {
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if ((i >> K) & 1) continue;
    const C x0 = v[i], x1 = v[i | (1 << K)];
    if (unit) {
      v[i] = x1;
      v[i | (1 << K)] = x0;
    } else {
      v[i] = cmul(a, x1);
      v[i | (1 << K)] = cmul(b, x0);
    }
  }
}

// diagonal (f0, f1) on register bit K; f0 == 1 skips half the registers
template <typename C, int NR, int K>
__device__ __forceinline__ void reg_diag1(C* v, const C& f0, const C& f1) {
  const bool one0 = f0.x == 1 && f0.y == 0;
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if ((i >> K) & 1)
      v[i] = cmul(f1, v[i]);
    else if (!one0)
      v[i] = cmul(f0, v[i]);
  }
}

template <typename C, int NR, int K0, int K1>
__device__ __forceinline__ void reg_diag2(C* v, const C* d) {
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    const int idx = (((i >> K0) & 1) << 1) | ((i >> K1) & 1);
    const C f = d[idx];
    if (!(f.x == 1 && f.y == 0)) v[i] = cmul(f, v[i]);
  }
}

// out[row r] = x[src(r)] on the quad of register bits (K0 = matrix MSB)
template <typename C, int NR, int K0, int K1>
__device__ __forceinline__ void reg_perm2(C* v, int code) {
  const int s0 = code & 3, s1 = (code >> 2) & 3, s2 = (code >> 4) & 3,
            s3 = (code >> 6) & 3;
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if ((i >> K0) & 1 || (i >> K1) & 1) continue;
    const int idx[4] = {i, i | (1 << K1), i | (1 << K0),
                        i | (1 << K0) | (1 << K1)};
    const C x0 = v[idx[0]], x1 = v[idx[1]], x2 = v[idx[2]], x3 = v[idx[3]];
    auto pick = [&](int q) {
      return q == 0 ? x0 : q == 1 ? x1 : q == 2 ? x2 : x3;
    };
    v[idx[0]] = pick(s0);
    v[idx[1]] = pick(s1);
    v[idx[2]] = pick(s2);
    v[idx[3]] = pick(s3);
  }
}

#define GBSV_SWITCH_K(k, NR, CALL)                 \
  switch (k) {                                     \
    case 0: { constexpr int K = 0; CALL; } break;  \
    case 1: { constexpr int K = 1; CALL; } break;  \
    case 2: { constexpr int K = 2; CALL; } break;  \
    default:                                       \
      if constexpr (NR >= 16) {                    \
        constexpr int K = 3;                       \
        CALL;                                      \
      }                                            \
      break;                                       \
  }

#define GBSV_SWITCH_K2(k0, k1, NR, CALL)                                 \
  do {                                                                   \
    if (k0 == 0 && k1 == 1) { constexpr int K0 = 0, K1 = 1; CALL; }      \
    else if (k0 == 1 && k1 == 0) { constexpr int K0 = 1, K1 = 0; CALL; } \
    else if (k0 == 0 && k1 == 2) { constexpr int K0 = 0, K1 = 2; CALL; } \
    else if (k0 == 2 && k1 == 0) { constexpr int K0 = 2, K1 = 0; CALL; } \
    else if (k0 == 1 && k1 == 2) { constexpr int K0 = 1, K1 = 2; CALL; } \
    else if (k0 == 2 && k1 == 1) { constexpr int K0 = 2, K1 = 1; CALL; } \
    else if constexpr (NR >= 16) {                                       \
      if (k0 == 0 && k1 == 3) { constexpr int K0 = 0, K1 = 3; CALL; }    \
      else if (k0 == 3 && k1 == 0) { constexpr int K0 = 3, K1 = 0; CALL; } \
      else if (k0 == 1 && k1 == 3) { constexpr int K0 = 1, K1 = 3; CALL; } \
      else if (k0 == 3 && k1 == 1) { constexpr int K0 = 3, K1 = 1; CALL; } \
      else if (k0 == 2 && k1 == 3) { constexpr int K0 = 2, K1 = 3; CALL; } \
      else if (k0 == 3 && k1 == 2) { constexpr int K0 = 3, K1 = 2; CALL; } \
    }                                                                    \
  } while (0)

template <typename C, int NR>
__device__ __forceinline__ void reg_dense1(C* v, int k, const C* mm) {
  const C m0 = mm[0], m1 = mm[1], m2 = mm[2], m3 = mm[3];
  switch (k) {
    case 0: reg_apply1<C, NR, 0>(v, m0, m1, m2, m3); break;
    case 1: reg_apply1<C, NR, 1>(v, m0, m1, m2, m3); break;
    case 2: reg_apply1<C, NR, 2>(v, m0, m1, m2, m3); break;
    default:
      if constexpr (NR >= 16) reg_apply1<C, NR, 3>(v, m0, m1, m2, m3);
      break;
  }
}

template <typename C, int NR>
__device__ __forceinline__ void reg_dense2(C* v, int k0, int k1,
                                           const volatile C* mm) {
#define GBSV_R2(a, b)                                  \
  if (k0 == a && k1 == b) {                            \
    reg_apply2<C, NR, a, b>(v, mm);                    \
    return;                                            \
  }
  GBSV_R2(0, 1) GBSV_R2(1, 0) GBSV_R2(0, 2) GBSV_R2(2, 0) GBSV_R2(1, 2)
  GBSV_R2(2, 1)
  if constexpr (NR >= 16) {
    GBSV_R2(0, 3) GBSV_R2(3, 0) GBSV_R2(1, 3) GBSV_R2(3, 1) GBSV_R2(2, 3)
    GBSV_R2(3, 2)
  }
#undef GBSV_R2
}

template <typename R, int RB>
__global__ void __launch_bounds__(512, sizeof(R) == 4 ? 2 : 1)
    fused_reg_kernel(const Cx<R>* in, Cx<R>* out, const Cx<R>* pool,
                     Stage2Args a) {
  using C = Cx<R>;
  constexpr int NR = 1 << RB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* S = reinterpret_cast<C*>(smem_raw);
  __shared__ SGate<C> sg[GCHUNK];
  const int T = blockDim.x;
  const int tid = threadIdx.x;
  const int M = 1 << a.m;
  const int run = 1 << a.c;
  const uint64_t tiles_per_state = uint64_t(1) << (a.n - a.m);
  const uint64_t s = blockIdx.x / tiles_per_state;
  uint64_t base = blockIdx.x % tiles_per_state;
  for (int j = 0; j < a.m; ++j) base = insert_zero(base, a.spos[j]);
  const C* src = in + s * a.in_stride + base;
  C* dst = out + (s << a.n) + base;
  constexpr int PER = 16 / sizeof(C);
  for (int l = tid * PER; l < M; l += T * PER) {
    const int r = l >> a.c;
    uint64_t off = (uint64_t)(l & (run - 1));
    for (int j = 0; j < a.m - a.c; ++j)
      if ((r >> j) & 1) off += uint64_t(1) << a.hpos[j];
    cp_async16<R>(&S[PER == 2 ? swz(l) : l], src + off);
  }
  cp_async_wait_all();
  __syncthreads();

  C tscale;
  tscale.x = 1;
  tscale.y = 0;
  C v[NR];
  for (int li = 0; li < a.num_layouts; ++li) {
    const Layout L = a.layouts[li];
    int rbmask = 0;
#pragma unroll
    for (int k = 0; k < RB; ++k) rbmask |= 1 << L.rb[k];
    // thread index bits fill the non-register tile bits in order
    int tb = 0;
    {
      int t = tid;
      for (int bit = 0; bit < a.m; ++bit) {
        if ((rbmask >> bit) & 1) continue;
        tb |= (t & 1) << bit;
        t >>= 1;
      }
    }
    // tile index of register i: tb | sum of po[k] over the set bits k of i
    int po[RB];
#pragma unroll
    for (int k = 0; k < RB; ++k) po[k] = 1 << L.rb[k];
    auto off = [&](int i) {
      int o = tb;
#pragma unroll
      for (int k = 0; k < RB; ++k)
        if ((i >> k) & 1) o |= po[k];
      return o;
    };
#pragma unroll
    for (int i = 0; i < NR; ++i) v[i] = S[PER == 2 ? swz(off(i)) : off(i)];

    for (int c0 = 0; c0 < L.num_gates; c0 += GCHUNK) {
      const int cnt = min(GCHUNK, L.num_gates - c0);
      __syncthreads();  // the previous chunk is no longer being read
      load_gate_chunk<C>(sg, a.gates, pool, s, L.first_gate + c0, cnt);
      __syncthreads();
      for (int gi = 0; gi < cnt; ++gi) {
        const SGate<C>& g = sg[gi];
        if ((base & g.cmask) != g.cval) continue;
        if (g.kind == FG_REAL1) {
          if constexpr (sizeof(R) == 4) {
            const float a00 = g.m[0].x, a01 = g.m[1].x, a10 = g.m[2].x,
                        a11 = g.m[3].x;
            GBSV_SWITCH_K(g.b0, NR,
                          (reg_real1<C, NR, K>(v, a00, a01, a10, a11)));
          } else {
            const double a00 = g.m[0].x, a01 = g.m[1].x, a10 = g.m[2].x,
                         a11 = g.m[3].x;
            GBSV_SWITCH_K(g.b0, NR,
                          (reg_real1d<C, NR, K>(v, a00, a01, a10, a11)));
          }
        } else if (g.kind == FG_ANTI1 ||
                   (g.kind == FG_CANTI1 && ((tb >> g.b1) & 1))) {
          const bool unit = g.nq == 1;
          const C aa = g.m[1], bb = g.m[2];
          GBSV_SWITCH_K(g.b0, NR, (reg_anti1<C, NR, K>(v, unit, aa, bb)));
        } else if (g.kind == FG_CANTI1) {
          // control bit is 0 for this thread: nothing to do
        } else if (g.kind == FG_PERM2) {
          const int code = g.nq;
          GBSV_SWITCH_K2(g.b0, g.b1, NR, (reg_perm2<C, NR, K0, K1>(v, code)));
        } else if (g.kind == FG_RDIAG) {
          // split the qubits into register bits and fixed (thread/global)
          int fixed = 0, kr0 = -1, kr1 = -1, sh0 = 0, sh1 = 0;
          for (int q = 0; q < g.nq; ++q) {
            const int b = q == 0 ? g.b0 : g.b1;
            const int shift = g.nq - 1 - q;
            if (b < 0) {
              fixed |= (int)((base >> (-1 - b)) & 1) << shift;
            } else if (b >= RB) {
              fixed |= ((tb >> (b - RB)) & 1) << shift;
            } else if (kr0 < 0) {
              kr0 = b;
              sh0 = shift;
            } else {
              kr1 = b;
              sh1 = shift;
            }
          }
          if (kr0 < 0) {
            const C f = g.m[fixed];
            if (!(f.x == 1 && f.y == 0)) {
#pragma unroll
              for (int i = 0; i < NR; ++i) v[i] = cmul(f, v[i]);
            }
          } else if (kr1 < 0) {
            const C f0 = g.m[fixed], f1 = g.m[fixed | (1 << sh0)];
            GBSV_SWITCH_K(kr0, NR, (reg_diag1<C, NR, K>(v, f0, f1)));
          } else {
            // both qubits in registers: matrix order is (q0, q1) = (kr0, kr1)
            const C* d = g.m;
            GBSV_SWITCH_K2(kr0, kr1, NR, (reg_diag2<C, NR, K0, K1>(v, d)));
          }
        } else if (g.kind == FG_DENSE1) {
          reg_dense1<C, NR>(v, g.b0, g.m);
        } else if (g.kind == FG_CDENSE1) {
          if ((tb >> g.b1) & 1) reg_dense1<C, NR>(v, g.b0, g.m);
        } else if (g.kind == FG_DENSE2) {
          reg_dense2<C, NR>(v, g.b0, g.b1, g.m);
        } else {  // FG_DIAG
          int gidx = 0, lb0 = -1, lb1 = -1;
          for (int q = 0; q < g.nq; ++q) {
            const int b = q == 0 ? g.b0 : g.b1;
            if (b < 0)
              gidx |= (int)((base >> (-1 - b)) & 1) << (g.nq - 1 - q);
            else if (q == 0)
              lb0 = b;
            else
              lb1 = b;
          }
          if (lb0 < 0 && lb1 < 0) {
            tscale = cmul(tscale, g.m[gidx]);
            continue;
          }
          const C d0 = g.m[0], d1 = g.m[1];
          const C d2 = g.nq == 2 ? g.m[2] : d0;
          const C d3 = g.nq == 2 ? g.m[3] : d1;
#pragma unroll
          for (int i = 0; i < NR; ++i) {
            int idx = gidx;
            if (lb0 >= 0) idx |= ((off(i) >> lb0) & 1) << (g.nq - 1);
            if (lb1 >= 0) idx |= ((off(i) >> lb1) & 1);
            const C f = idx == 0 ? d0 : idx == 1 ? d1 : idx == 2 ? d2 : d3;
            v[i] = cmul(f, v[i]);
          }
        }
      }
    }
#pragma unroll
    for (int i = 0; i < NR; ++i) S[PER == 2 ? swz(off(i)) : off(i)] = v[i];
    __syncthreads();
  }

  const bool scaled = tscale.x != 1 || tscale.y != 0;
  for (int l = tid * PER; l < M; l += T * PER) {
    const int r = l >> a.c;
    uint64_t off = (uint64_t)(l & (run - 1));
    for (int j = 0; j < a.m - a.c; ++j)
      if ((r >> j) & 1) off += uint64_t(1) << a.hpos[j];
    const int pl = PER == 2 ? swz(l) : l;
    C v0 = S[pl];
    if (scaled) v0 = cmul(tscale, v0);
    if constexpr (PER == 2) {
      C v1 = S[pl + 1];
      if (scaled) v1 = cmul(tscale, v1);
      __stcs(reinterpret_cast<float4*>(dst + off),
             make_float4(v0.x, v0.y, v1.x, v1.y));
    } else {
      __stcs(dst + off, v0);
    }
  }
}

}  // namespace gbsv

extern "C" int gbsv_fused_register_bits(int dtype) {
  return dtype == GBSV_C64 ? 4 : 3;
}

extern "C" int gbsv_run_stage_layouts(
    const void* state_in, void* state_out, int dtype, int num_qubits,
    int64_t num_states, int64_t in_stride, int tile_qubits,
    int contiguous_qubits, const int32_t* tile_positions, const void* gates,
    const void* layouts, int num_layouts, const void* pool, void* stream) {
  if (dtype != GBSV_C64 && dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "state dtype must be complex");
  const int n = num_qubits, m = tile_qubits, c = contiguous_qubits;
  const int rb = gbsv_fused_register_bits(dtype);
  const int mmax = gbsv_fused_max_tile_qubits(dtype);
  const int cmin = dtype == GBSV_C64 ? 1 : 0;
  if (n < 1 || n > 62 || m < rb || m > mmax || m > n || c < cmin || c > m)
    return set_error(GBSV_ERR_INVALID_ARG,
                     "bad layout stage n=%d m=%d c=%d", n, m, c);
  if (num_states < 0 || in_stride < 0 || num_layouts < 0)
    return set_error(GBSV_ERR_INVALID_ARG, "negative size");
  if (num_states == 0) return GBSV_OK;
  if (!state_in || !state_out || !tile_positions ||
      (num_layouts > 0 && (!layouts || !gates || !pool)))
    return set_error(GBSV_ERR_INVALID_ARG, "null pointer");
  const int amp = dtype_bytes(dtype);
  if ((uintptr_t)state_in % 16 || (uintptr_t)state_out % 16 ||
      (in_stride * amp) % 16)
    return set_error(GBSV_ERR_INVALID_ARG, "states must be 16-byte aligned");
  Stage2Args a{};
  a.n = n;
  a.m = m;
  a.c = c;
  a.in_stride = in_stride;
  a.gates = static_cast<const FusedGate*>(gates);
  a.layouts = static_cast<const Layout*>(layouts);
  a.num_layouts = num_layouts;
  uint64_t seen = 0;
  for (int j = 0; j < m; ++j) {
    const int p = tile_positions[j];
    if (p < 0 || p >= n || ((seen >> p) & 1) || (j < c && p != j))
      return set_error(GBSV_ERR_INVALID_ARG, "bad tile position %d", p);
    seen |= uint64_t(1) << p;
    if (j >= c) a.hpos[j - c] = p;
    a.spos[j] = p;
  }
  for (int i = 1; i < m; ++i)
    for (int j = i; j > 0 && a.spos[j - 1] > a.spos[j]; --j) {
      const int t = a.spos[j];
      a.spos[j] = a.spos[j - 1];
      a.spos[j - 1] = t;
    }
  const uint64_t blocks = (uint64_t)num_states << (n - m);
  if (blocks > 0x7fffffffull)
    return set_error(GBSV_ERR_UNSUPPORTED, "too many tiles");
  const int threads = 1 << (m - rb);
  if (threads > 512)
    return set_error(GBSV_ERR_UNSUPPORTED, "tile too large for one CTA");
  const size_t smem = (size_t)amp << m;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == GBSV_C64) {
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(fused_reg_kernel<float, 4>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(sizeof(float2) << mmax));
      attr = true;
    }
    fused_reg_kernel<float, 4><<<(unsigned)blocks, threads, smem, st>>>(
        static_cast<const float2*>(state_in), static_cast<float2*>(state_out),
        static_cast<const float2*>(pool), a);
  } else {
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(fused_reg_kernel<double, 3>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(sizeof(double2) << mmax));
      attr = true;
    }
    fused_reg_kernel<double, 3><<<(unsigned)blocks, threads, smem, st>>>(
        static_cast<const double2*>(state_in),
        static_cast<double2*>(state_out), static_cast<const double2*>(pool),
        a);
  }
  return after_launch("fused_reg_kernel");
}

// ---------------------------------------------------------------------------
// Many programs in one launch: CTA i owns one whole state of 2^n <= 2^14
// amplitudes (a single tile) at states[i] and runs its own gate list
// gates[first[i] .. first[i] + count[i]) on it in shared memory.  Requests
// with different circuits but the same qubit count share one launch.
namespace gbsv {

template <typename R>
__global__ void __launch_bounds__(512, 2)
    multi_program_kernel(int n, const unsigned long long* states,
                         const int32_t* first, const int32_t* count,
                         const FusedGate* gates, const Cx<R>* pool) {
  using C = Cx<R>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* S = reinterpret_cast<C*>(smem_raw);
  const int M = 1 << n;
  const int T = blockDim.x;
  const int tid = threadIdx.x;
  C* st = reinterpret_cast<C*>(states[blockIdx.x]);
  constexpr int PER = 16 / sizeof(C);
  for (int l = tid * PER; l < M; l += T * PER)
    cp_async16<R>(&S[PER == 2 ? swz(l) : l], st + l);
  cp_async_wait_all();
  __syncthreads();
  C tscale;
  tscale.x = 1;
  tscale.y = 0;
  bool scaled = false;
  run_gates_smem<R>(S, M, 0, 0, gates + first[blockIdx.x], count[blockIdx.x],
                    pool, tscale, scaled);
  for (int l = tid * PER; l < M; l += T * PER) {
    const int pl = PER == 2 ? swz(l) : l;
    C v0 = S[pl];
    if (scaled) v0 = cmul(tscale, v0);
    if constexpr (PER == 2) {
      C v1 = S[pl + 1];
      if (scaled) v1 = cmul(tscale, v1);
      __stcs(reinterpret_cast<float4*>(st + l),
             make_float4(v0.x, v0.y, v1.x, v1.y));
    } else {
      __stcs(st + l, v0);
    }
  }
}

}  // namespace gbsv

extern "C" int gbsv_run_programs(int dtype, int num_qubits, int num_ctas,
                                 const void* state_ptrs,
                                 const void* gate_first,
                                 const void* gate_count, const void* gates,
                                 const void* pool, void* stream) {
  if (dtype != GBSV_C64 && dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "state dtype must be complex");
  const int mmax = gbsv_fused_max_tile_qubits(dtype);
  const int nmin = dtype == GBSV_C64 ? 1 : 0;
  if (num_qubits < nmin || num_qubits > mmax || num_ctas < 0)
    return set_error(GBSV_ERR_INVALID_ARG,
                     "run_programs needs %d <= qubits <= %d (got %d)", nmin,
                     mmax, num_qubits);
  if (num_ctas == 0) return GBSV_OK;
  if (!state_ptrs || !gate_first || !gate_count || !gates || !pool)
    return set_error(GBSV_ERR_INVALID_ARG, "null pointer");
  const int amp = dtype_bytes(dtype);
  const size_t smem = (size_t)amp << num_qubits;
  int threads = (1 << num_qubits) / 4;
  if (threads > 512) threads = 512;
  if (threads < 32) threads = 32;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == GBSV_C64) {
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(multi_program_kernel<float>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(sizeof(float2) << mmax));
      attr = true;
    }
    multi_program_kernel<float><<<num_ctas, threads, smem, st>>>(
        num_qubits, static_cast<const unsigned long long*>(state_ptrs),
        static_cast<const int32_t*>(gate_first),
        static_cast<const int32_t*>(gate_count),
        static_cast<const FusedGate*>(gates),
        static_cast<const float2*>(pool));
  } else {
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(multi_program_kernel<double>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(sizeof(double2) << mmax));
      attr = true;
    }
    multi_program_kernel<double><<<num_ctas, threads, smem, st>>>(
        num_qubits, static_cast<const unsigned long long*>(state_ptrs),
        static_cast<const int32_t*>(gate_first),
        static_cast<const int32_t*>(gate_count),
        static_cast<const FusedGate*>(gates),
        static_cast<const double2*>(pool));
  }
  return after_launch("multi_program_kernel");
}
