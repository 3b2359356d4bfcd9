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
#include "dfloat.cuh"

#include <algorithm>

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
// the T = 2^(m-RB) threads holds 2^RB amplitudes of the tile in registers.  A
// "layout" names RB tile bits that index a thread's registers; the other
// m - RB tile bits are the thread index.  Within a layout
//   * dense gates on register bits run in registers,
//   * diagonal gates need no particular layout (each register knows its
//     full tile index); a factor that depends only on thread or outside bits
//     is one scalar per thread, applied once when the layout ends (it
//     commutes with everything a thread does to its own registers),
//   * a control on a thread bit is a per-thread condition,
// so shared memory is read and written once per layout instead of once per
// gate.  The host planner groups a stage's gates into layouts.
//
// The kernel is persistent: CTA b walks a contiguous range of tiles and,
// when two tiles fit in shared memory, prefetches tile t+1 (cp.async) into
// the second buffer while it computes tile t.  A stage's gate records are
// decoded once per CTA into flat operations in shared memory (matrix values
// again when the state changes, for gates with one matrix per state), so a
// gate costs one uniform jump-table dispatch plus its arithmetic.
//
// Shared-memory addresses use an XOR-linear swizzle (complex64: bits 1-3 of
// the amplitude index ^= bits 4-6, bit 0 stays so that 16-byte pieces stay
// whole for the tile copies; complex128: bits 0-2 ^= bits 3-5).
// Because it is linear and a thread's offset bits are disjoint from its
// register bits, address(register i) = swz(thread offset) ^ swz(register
// offset i), both read from per-layout tables.
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
  int nbuf;                // tile buffers in shared memory (1 or 2)
  int64_t num_states;
  int df;                  // complex128 in double-float pairs
};

constexpr int TS_MAXG = 96;   // decoded gates resident per CTA
constexpr int TS_MAXL = 16;   // layouts resident per CTA
constexpr int TS_MAXM = 512;  // matrix values resident per CTA
constexpr int TS_CHUNK = 32;  // gates per chunk when a stage is not resident

// Flat operation codes: + K (register bit, < 5) or + P (ordered pair of
// register bits, pair_index, < 20).  Codes below TOP_DIAG1 are dense and
// carry a thread condition (x) and a tile condition (a, b).
constexpr int TOP_DENSE1 = 0;
constexpr int TOP_REAL1 = 5;
constexpr int TOP_SWAP1 = 10;
constexpr int TOP_ANTI1 = 15;
constexpr int TOP_DENSE2 = 20;
constexpr int TOP_PERM2 = 40;
constexpr int TOP_SWAP2 = 60;   // SWAP of two register bits
constexpr int TOP_CX2 = 80;     // CNOT, control P's first bit
constexpr int TOP_DIAG1 = 100;
constexpr int TOP_DIAG2 = 105;
constexpr int TOP_SCALAR = 125;
constexpr int TOP_NOP = 126;

__device__ __forceinline__ int pair_index(int k0, int k1) {
  return k0 * 4 + (k1 < k0 ? k1 : k1 - 1);
}

struct __align__(16) TOp {
  int16_t op;
  int16_t code;   // PERM2: source rows; DIAG1: index bit of the register qubit
  int16_t moff;   // first matrix value in the CTA's value array
  int16_t nq;
  int32_t x, y;   // dense: thread condition (tile-bit mask, 0 = none);
                  // diagonal: tile-bit masks of thread qubits q0 / q1
  uint64_t a, b;  // dense: tile condition (cmask, cval);
                  // diagonal: outside-bit masks of q0 / q1
};

struct TLayout {
  int32_t first, count;
  int32_t nscal;               // leading operations that are thread scalars
  int32_t spo[LAYOUT_MAX_RB];  // swizzled tile offsets of the register bits
  int32_t spw[LAYOUT_MAX_RB];  // the same for the write-back (relabelled)
  int32_t cw;                  // write-back offset of flipped register bits
  uint16_t lo_s[32], hi_s[16]; // swizzled offsets of thread bits 0-4 / 5-8
  uint16_t lo_r[32], hi_r[16]; // the same, plain
};

template <typename R>
__device__ __forceinline__ int swz_amp(int a) {
  if constexpr (sizeof(R) == 4)
    return a ^ (((a >> 4) & 7) << 1);
  else
    return a ^ ((a >> 3) & 7);
}

__device__ __forceinline__ int fg_nvals(int kind, int nq) {
  return (kind == FG_DENSE2 || kind == FG_PERM2) ? 16
         : (kind == FG_DIAG || kind == FG_RDIAG) ? (1 << nq)
                                                 : 4;
}

// Decode one record into a flat operation.  For FG_DIAG records (tile bits
// rather than register / thread encodings) `rb` gives the layout's register
// bits.
template <int RB>
__device__ TOp ts_decode(const FusedGate& g, int moff, const int32_t* rb) {
  TOp o;
  o.op = TOP_NOP;
  o.code = 0;
  o.moff = (int16_t)moff;
  o.nq = (int16_t)g.nq;
  o.x = o.y = 0;
  o.a = o.b = 0;
  const int kind = g.kind;
  if (kind == FG_RDIAG || kind == FG_DIAG) {
    const int nq = g.nq;
    int kreg[2] = {-1, -1};
    for (int j = 0; j < nq && j < 2; ++j) {
      int b = j == 0 ? g.b0 : g.b1;
      if (kind == FG_DIAG && b >= 0) {  // tile bit: register or thread?
        int k = -1;
        for (int r = 0; r < RB; ++r)
          if (rb[r] == b) k = r;
        b = k >= 0 ? k : RB + b;
      }
      if (b < 0) {
        const uint64_t mk = uint64_t(1) << (-1 - b);
        if (j == 0) o.a = mk; else o.b = mk;
      } else if (b >= RB) {
        const int mk = 1 << (b - RB);
        if (j == 0) o.x = mk; else o.y = mk;
      } else {
        kreg[j] = b;
      }
    }
    if (kreg[0] >= 0 && kreg[1] >= 0) {
      o.op = (int16_t)(TOP_DIAG2 + pair_index(kreg[0], kreg[1]));
    } else if (kreg[0] >= 0) {
      o.op = (int16_t)(TOP_DIAG1 + kreg[0]);
      o.code = (int16_t)(nq == 2 ? 2 : 1);
    } else if (kreg[1] >= 0) {
      o.op = (int16_t)(TOP_DIAG1 + kreg[1]);
      o.code = 1;
    } else {
      o.op = TOP_SCALAR;
    }
    return o;
  }
  o.a = g.cmask;
  o.b = g.cval;
  switch (kind) {
    case FG_DENSE1: o.op = (int16_t)(TOP_DENSE1 + g.b0); break;
    case FG_REAL1: o.op = (int16_t)(TOP_REAL1 + g.b0); break;
    case FG_ANTI1:
      o.op = (int16_t)((g.nq == 1 ? TOP_SWAP1 : TOP_ANTI1) + g.b0);
      break;
    case FG_CDENSE1:
      o.op = (int16_t)(TOP_DENSE1 + g.b0);
      o.x = 1 << g.b1;
      break;
    case FG_CANTI1:
      o.op = (int16_t)((g.nq == 1 ? TOP_SWAP1 : TOP_ANTI1) + g.b0);
      o.x = 1 << g.b1;
      break;
    case FG_DENSE2: o.op = (int16_t)(TOP_DENSE2 + pair_index(g.b0, g.b1)); break;
    case FG_PERM2:
      // rows in (b0, b1) order: SWAP = sources (0, 2, 1, 3); CNOT with
      // control b0 = (0, 1, 3, 2); CNOT with control b1 = (0, 3, 2, 1)
      if (g.nq == 0xd8) {
        o.op = (int16_t)(TOP_SWAP2 + pair_index(g.b0, g.b1));
      } else if (g.nq == 0xb4) {
        o.op = (int16_t)(TOP_CX2 + pair_index(g.b0, g.b1));
      } else if (g.nq == 0x6c) {
        o.op = (int16_t)(TOP_CX2 + pair_index(g.b1, g.b0));
      } else {
        o.op = (int16_t)(TOP_PERM2 + pair_index(g.b0, g.b1));
        o.code = (int16_t)g.nq;
      }
      break;
    default: break;
  }
  return o;
}

// Value permutations applied when a gate's matrix values are copied in.
constexpr int VP_REV4 = 4;      // 2x2 conjugated by X: entries reversed
constexpr int VP_XOR4X4 = 8;    // 4x4 conjugated by X on bits F (low 2)
constexpr int VP_XORDIAG = 16;  // diagonal values indexed by i ^ F

// Rewrite a decoded operation on logical register bits onto physical bits
// of the relabelling (perm, flip); X and SWAP only update the relabelling.
// Returns whether an operation remains to run; vm receives the value
// permutation its matrix needs.
template <int RB>
__device__ bool ts_relabel(TOp& o, int* perm, int& flip, int8_t& vm) {
  const int op = o.op;
  const bool cond = o.x != 0 || o.a != 0;
  auto pair_of = [](int p, int& k0, int& k1) {
    k0 = p >> 2;
    const int j = p & 3;
    k1 = j < k0 ? j : j + 1;
  };
  if (op < TOP_DENSE2) {  // one register bit
    const int fam = op / 5, k = op - 5 * fam;
    const int pk = perm[k];
    const bool fl = (flip >> pk) & 1;
    if (fam == TOP_SWAP1 / 5 && !cond) {  // X: complement the bit
      flip ^= 1 << pk;
      return false;
    }
    o.op = (int16_t)(5 * fam + pk);
    if (fl && fam != TOP_SWAP1 / 5) vm = VP_REV4;
    return true;
  }
  if (op < TOP_DIAG1) {  // two register bits
    const int base = op < TOP_PERM2 ? TOP_DENSE2
                     : op < TOP_SWAP2 ? TOP_PERM2
                     : op < TOP_CX2 ? TOP_SWAP2
                                    : TOP_CX2;
    int k0, k1;
    pair_of(op - base, k0, k1);
    const int p0 = perm[k0], p1 = perm[k1];
    const int F = (((flip >> p0) & 1) << 1) | ((flip >> p1) & 1);
    if (base == TOP_SWAP2 && !cond) {
      perm[k0] = p1;
      perm[k1] = p0;
      return false;
    }
    o.op = (int16_t)(base + pair_index(p0, p1));
    if (base == TOP_CX2) {
      // control complemented: flip the target everywhere as well
      if (F & 2) flip ^= 1 << p1;
    } else if (base == TOP_DENSE2 && F) {
      vm = (int8_t)(VP_XOR4X4 | F);
    } else if (base == TOP_PERM2 && F) {
      int code = 0;
      for (int r = 0; r < 4; ++r)
        code |= (((o.code >> (2 * (r ^ F))) & 3) ^ F) << (2 * r);
      o.code = (int16_t)code;
    }
    return true;
  }
  if (op < TOP_DIAG2) {  // diagonal with one register bit
    const int pk = perm[op - TOP_DIAG1];
    o.op = (int16_t)(TOP_DIAG1 + pk);
    if ((flip >> pk) & 1) vm = (int8_t)(VP_XORDIAG | o.code);
    return true;
  }
  if (op < TOP_SCALAR) {  // diagonal on two register bits
    int k0, k1;
    pair_of(op - TOP_DIAG2, k0, k1);
    const int p0 = perm[k0], p1 = perm[k1];
    const int F = (((flip >> p0) & 1) << 1) | ((flip >> p1) & 1);
    o.op = (int16_t)(TOP_DIAG2 + pair_index(p0, p1));
    if (F) vm = (int8_t)(VP_XORDIAG | F);
    return true;
  }
  return op != TOP_NOP;
}

// ----------------------------------------------------- register kernels --
// The operations are written once over a value type V (the registers) and
// an entry type E (the matrix values): V = E = float2 / double2 for
// complex64 and FP64 complex128, V = DC (double-float pairs) and E = DEC
// (exact float triples) for complex128 in pairs.  These overloads are the
// arithmetic they share.
template <typename C>
__device__ __forceinline__ C op_row2(const C& m0, const C& x0, const C& m1,
                                     const C& x1) {
  return cmad(m1, x1, cmul(m0, x0));
}
template <typename C>
__device__ __forceinline__ C op_row2_real(const C& m0, const C& x0,
                                          const C& m1, const C& x1) {
  C y;
  y.x = fma(m0.x, x0.x, m1.x * x1.x);
  y.y = fma(m0.x, x0.y, m1.x * x1.y);
  return y;
}
template <typename C>
__device__ __forceinline__ C op_mul(const C& m, const C& x) {
  return cmul(m, x);
}
template <typename C>
__device__ __forceinline__ C op_row4(const C* m, const C* x) {
  C acc = czero<C>();
  for (int k = 0; k < 4; ++k) acc = cmad(m[k], x[k], acc);
  return acc;
}
template <typename C>
__device__ __forceinline__ bool is_one(const C& f) {
  return f.x == 1 && f.y == 0;
}
// thread scalar *= entry
template <typename C>
__device__ __forceinline__ C op_scal(const C& ts, const C& m) {
  return cmul(ts, m);
}
// value *= thread scalar
template <typename C>
__device__ __forceinline__ C op_by_scal(const C& ts, const C& x) {
  return cmul(ts, x);
}

__device__ __forceinline__ DC op_row2(const DEC& m0, const DC& x0,
                                      const DEC& m1, const DC& x1) {
  return df_row2<false>(m0, x0, m1, x1);
}
__device__ __forceinline__ DC op_row2_real(const DEC& m0, const DC& x0,
                                           const DEC& m1, const DC& x1) {
  return df_row2_real<false>(m0.re, x0, m1.re, x1);
}
__device__ __forceinline__ DC op_mul(const DEC& m, const DC& x) {
  return df_cmul<false>(m, x);
}
__device__ __forceinline__ DC op_row4(const DEC* m, const DC* x) {
  return df_row4<false>(m, x);
}
// 1 + 0i up to the last 5 bits of the real part (|x - 1| < 2^-48) and an
// imaginary part below 2^-149: skipping such a factor costs less than the
// pairs' own rounding
__device__ __forceinline__ bool is_one(const DEC& f) {
  return f.re.hi == 1.f && f.re.mid == 0.f && f.im.hi == 0.f;
}
__device__ __forceinline__ DC op_scal(const DC& ts, const DEC& m) {
  return df_cmul<false>(m, ts);
}
// a pair as an exact triple (its low word in the middle)
__device__ __forceinline__ DEC df_as_entry(const DC& x) {
  DEC e;
  e.re = DE{x.re.hi, x.re.lo, 0.f};
  e.im = DE{x.im.hi, x.im.lo, 0.f};
  return e;
}
__device__ __forceinline__ DC op_by_scal(const DC& ts, const DC& x) {
  return df_cmul<false>(df_as_entry(ts), x);
}
__device__ __forceinline__ bool is_one(const DC& f) {
  return f.re.hi == 1.f && f.re.lo == 0.f && f.im.hi == 0.f &&
         f.im.lo == 0.f;
}

template <typename V, typename E, int NR, int K>
__device__ __forceinline__ void ts_dense1(V* v, const E* mm) {
  const E m0 = mm[0], m1 = mm[1], m2 = mm[2], m3 = mm[3];
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if ((i >> K) & 1) continue;
    const V x0 = v[i], x1 = v[i | (1 << K)];
    v[i] = op_row2(m0, x0, m1, x1);
    v[i | (1 << K)] = op_row2(m2, x0, m3, x1);
  }
}

template <typename V, typename E, int NR, int K>
__device__ __forceinline__ void ts_real1(V* v, const E* mm) {
  const E m0 = mm[0], m1 = mm[1], m2 = mm[2], m3 = mm[3];
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if ((i >> K) & 1) continue;
    const V x0 = v[i], x1 = v[i | (1 << K)];
    const V y0 = op_row2_real(m0, x0, m1, x1);
    const V y1 = op_row2_real(m2, x0, m3, x1);
    v[i] = y0;
    v[i | (1 << K)] = y1;
  }
}

template <typename V, int NR, int K>
__device__ __forceinline__ void ts_swap1(V* v) {
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if ((i >> K) & 1) continue;
    const V t = v[i];
    v[i] = v[i | (1 << K)];
    v[i | (1 << K)] = t;
  }
}

template <typename V, typename E, int NR, int K>
__device__ __forceinline__ void ts_anti1(V* v, const E* mm) {
  const E a = mm[1], b = mm[2];
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if ((i >> K) & 1) continue;
    const V x0 = v[i], x1 = v[i | (1 << K)];
    v[i] = op_mul(a, x1);
    v[i | (1 << K)] = op_mul(b, x0);
  }
}

// X on register bit KT where register bit KC is 1
template <typename V, int NR, int KC, int KT>
__device__ __forceinline__ void ts_cx2(V* v) {
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if (!((i >> KC) & 1) || (i >> KT) & 1) continue;
    const V t = v[i];
    v[i] = v[i | (1 << KT)];
    v[i | (1 << KT)] = t;
  }
}

template <typename C>
__device__ __forceinline__ C sel4(const C* pm, int i) {
  const C lo = (i & 1) ? pm[1] : pm[0];
  const C hi = (i & 1) ? pm[3] : pm[2];
  return (i & 2) ? hi : lo;
}
// triples stay in shared memory: an indexed load, not 18 selects
__device__ __forceinline__ DEC sel4(const DEC* pm, int i) { return pm[i]; }

// 4x4 (dense, or a permutation given by code) on register bits k0 (matrix
// MSB) and k1 known only at run time: the registers go through a local
// copy that is indexed at run time, so the register array itself is only
// ever indexed by constants.
template <typename V, typename E, int NR>
__device__ __noinline__ void ts_generic2_mem(V* t, int k0, int k1,
                                             bool dense, int code,
                                             const E* mm) {
  const int b0 = 1 << k0, b1 = 1 << k1;
  for (int i = 0; i < NR; ++i) {
    if (i & (b0 | b1)) continue;
    const int idx[4] = {i, i | b1, i | b0, i | b0 | b1};
    V x[4];
    for (int k = 0; k < 4; ++k) x[k] = t[idx[k]];
    for (int r = 0; r < 4; ++r) {
      if (dense) {
        E row[4];
        for (int k = 0; k < 4; ++k) row[k] = mm[4 * r + k];
        t[idx[r]] = op_row4(row, x);
      } else {
        t[idx[r]] = x[(code >> (2 * r)) & 3];
      }
    }
  }
}

template <typename V, typename E, int NR>
__device__ __forceinline__ void ts_generic2(V* v, int k0, int k1, bool dense,
                                            int code, const E* mm) {
  V t[NR];
#pragma unroll
  for (int i = 0; i < NR; ++i) t[i] = v[i];
  ts_generic2_mem<V, E, NR>(t, k0, k1, dense, code, mm);
#pragma unroll
  for (int i = 0; i < NR; ++i) v[i] = t[i];
}

// diagonal on register bits k0 (index MSB), k1 known at run time
template <typename V, typename E, int NR>
__device__ __forceinline__ void ts_diag2_any(V* v, int k0, int k1,
                                             const E* d) {
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    const int idx = (((i >> k0) & 1) << 1) | ((i >> k1) & 1);
    const E f = sel4(d, idx);
    if (!is_one(f)) v[i] = op_mul(f, v[i]);
  }
}

// diag(f0, f1) on register bit K
template <typename V, typename E, int NR, int K>
__device__ __forceinline__ void ts_diag1(V* v, const E& f0, const E& f1) {
  const bool one0 = is_one(f0), one1 = is_one(f1);
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if ((i >> K) & 1) {
      if (!one1) v[i] = op_mul(f1, v[i]);
    } else if (!one0) {
      v[i] = op_mul(f0, v[i]);
    }
  }
}

#define TS_K(BASE, KK, ...)                   \
  case BASE + KK: {                           \
    constexpr int K = KK;                     \
    if constexpr (K < RB) { __VA_ARGS__; }    \
  } break;
#define TS_KS(BASE, ...)                                            \
  TS_K(BASE, 0, __VA_ARGS__) TS_K(BASE, 1, __VA_ARGS__)             \
  TS_K(BASE, 2, __VA_ARGS__) TS_K(BASE, 3, __VA_ARGS__)             \
  TS_K(BASE, 4, __VA_ARGS__)
#define TS_P(BASE, A, J, ...)                                   \
  case BASE + A * 4 + J: {                                      \
    constexpr int K0 = A, K1 = J < A ? J : J + 1;               \
    if constexpr (K0 < RB && K1 < RB) { __VA_ARGS__; }          \
  } break;
#define TS_P4(BASE, A, ...)                                             \
  TS_P(BASE, A, 0, __VA_ARGS__) TS_P(BASE, A, 1, __VA_ARGS__)           \
  TS_P(BASE, A, 2, __VA_ARGS__) TS_P(BASE, A, 3, __VA_ARGS__)
#define TS_PS(BASE, ...)                                                \
  TS_P4(BASE, 0, __VA_ARGS__) TS_P4(BASE, 1, __VA_ARGS__)               \
  TS_P4(BASE, 2, __VA_ARGS__) TS_P4(BASE, 3, __VA_ARGS__)               \
  TS_P4(BASE, 4, __VA_ARGS__)

// An operation (two 16-byte loads) and its first four matrix values.
__device__ __forceinline__ TOp ts_load_op(const TOp* p) {
  const uint4 w0 = reinterpret_cast<const uint4*>(p)[0];
  const uint4 w1 = reinterpret_cast<const uint4*>(p)[1];
  TOp o;
  o.op = (int16_t)(w0.x & 0xffff);
  o.code = (int16_t)(w0.x >> 16);
  o.moff = (int16_t)(w0.y & 0xffff);
  o.nq = (int16_t)(w0.y >> 16);
  o.x = (int32_t)w0.z;
  o.y = (int32_t)w0.w;
  o.a = (uint64_t)w1.x | ((uint64_t)w1.y << 32);
  o.b = (uint64_t)w1.z | ((uint64_t)w1.w << 32);
  return o;
}

template <typename C>
__device__ __forceinline__ void ts_load_vals(C* pm, const C* src) {
  if constexpr (sizeof(C) == 8) {  // moff is even: two 16-byte loads
    const float4 a = reinterpret_cast<const float4*>(src)[0];
    const float4 b = reinterpret_cast<const float4*>(src)[1];
    pm[0] = make_float2(a.x, a.y);
    pm[1] = make_float2(a.z, a.w);
    pm[2] = make_float2(b.x, b.y);
    pm[3] = make_float2(b.z, b.w);
  } else {
#pragma unroll
    for (int j = 0; j < 4; ++j) pm[j] = src[j];
  }
}

// Apply one decoded operation to a thread's registers.
template <typename V, typename E, int RB>
__device__ __forceinline__ void ts_apply(V* v, const TOp& o, const E* pm,
                                         const E* mats, int tb,
                                         uint64_t base, V& ts) {
  constexpr int NR = 1 << RB;
  const int op = o.op;
  const E* mm = pm;
  if (op < TOP_DIAG1) {
    if ((tb & o.x) != o.x || (base & o.a) != o.b) return;
  }
  int fixed = 0;
  if (op >= TOP_DIAG1) {
    const int hb = o.nq == 2 ? 2 : 1;
    if ((tb & o.x) | ((base & o.a) != 0)) fixed |= hb;
    if ((tb & o.y) | ((base & o.b) != 0)) fixed |= 1;
  }
  // two-level dispatch: operation family, then register bit(s)
  if (op < TOP_DENSE2) {
    const int fam = op / 5, kk = op - 5 * fam;
    switch (fam) {
      case TOP_DENSE1 / 5:
        switch (kk) { TS_KS(0, (ts_dense1<V, E, NR, K>(v, mm))) }
        break;
      case TOP_REAL1 / 5:
        switch (kk) { TS_KS(0, (ts_real1<V, E, NR, K>(v, mm))) }
        break;
      case TOP_SWAP1 / 5:
        switch (kk) { TS_KS(0, (ts_swap1<V, NR, K>(v))) }
        break;
      default:
        switch (kk) { TS_KS(0, (ts_anti1<V, E, NR, K>(v, mm))) }
        break;
    }
  } else if (op < TOP_DIAG1) {
    if (op < TOP_CX2) {
      // general 4x4 or permutation (a SWAP left here carries a condition,
      // which planners never produce): rare, not unrolled
      const int p = op < TOP_PERM2   ? op - TOP_DENSE2
                    : op < TOP_SWAP2 ? op - TOP_PERM2
                                     : op - TOP_SWAP2;
      const int k0 = p >> 2, j = p & 3, k1 = j < k0 ? j : j + 1;
      const int code = op < TOP_SWAP2 ? o.code : 0xd8;
      ts_generic2<V, E, NR>(v, k0, k1, op < TOP_PERM2, code, mats + o.moff);
    } else {
      switch (op - TOP_CX2) { TS_PS(0, (ts_cx2<V, NR, K0, K1>(v))) }
    }
  } else if (op < TOP_DIAG2) {
    const E f0 = sel4(pm, fixed), f1 = sel4(pm, fixed | o.code);
    switch (op - TOP_DIAG1) { TS_KS(0, (ts_diag1<V, E, NR, K>(v, f0, f1))) }
  } else if (op < TOP_SCALAR) {
    const int p = op - TOP_DIAG2;
    const int k0 = p >> 2, j = p & 3, k1 = j < k0 ? j : j + 1;
    ts_diag2_any<V, E, NR>(v, k0, k1, pm);
  } else if (op == TOP_SCALAR) {
    ts = op_scal(ts, sel4(pm, fixed));
  }
}

#undef TS_K
#undef TS_KS
#undef TS_P
#undef TS_P4
#undef TS_PS

// Operations [first, end) in order.
template <typename V, typename E, int RB>
__device__ __forceinline__ void ts_run(V* v, const TOp* ops, const E* mats,
                                       int first, int end, int tb,
                                       uint64_t base, V& ts) {
  for (int gi = first; gi < end; ++gi) {
    const TOp o = ts_load_op(&ops[gi]);
    if constexpr (sizeof(E) == sizeof(DEC)) {  // triples: read in place
      ts_apply<V, E, RB>(v, o, mats + o.moff, mats, tb, base, ts);
    } else {
      E pm[4];
      ts_load_vals(pm, mats + o.moff);
      ts_apply<V, E, RB>(v, o, pm, mats, tb, base, ts);
    }
  }
}

// Which tile bit each thread-index bit stands for in a layout.  Shared
// memory is read and written at (thread bits | register bits), swizzled; a
// half-warp's 16 lanes (complex64, 8-byte accesses; a quarter-warp of 8
// lanes for complex128) hit distinct banks exactly when the swizzled
// low-address images of their lane bits are linearly independent over
// GF(2).  So the lowest thread-index bits take, in ascending order, the
// non-register tile bits that raise that rank, then the rest ascending.
// The order is packed 4 bits per thread-index bit (at most 14 - RB <= 11).
__device__ __forceinline__ int ts_order_get(uint64_t ord, int j) {
  return (int)((ord >> (4 * j)) & 15);
}

template <typename R>
__device__ uint64_t ts_thread_bit_order(int rbmask, int m) {
  constexpr int BANK_BITS = sizeof(R) == 4 ? 4 : 3;
  // image of tile bit b in the low BANK_BITS address bits after swz_amp
  auto image = [](int b) {
    const int a = swz_amp<R>(1 << b);
    return a & ((1 << BANK_BITS) - 1);
  };
  int lead[BANK_BITS];  // basis vector whose highest set bit is h, or 0
  for (int h = 0; h < BANK_BITS; ++h) lead[h] = 0;
  int nb = 0;
  uint64_t ord = 0;
  int taken = 0, j = 0;
  for (int b = 0; b < m && nb < BANK_BITS; ++b) {
    if ((rbmask >> b) & 1) continue;
    int v = image(b);
    bool added = false;
    for (int h = BANK_BITS - 1; h >= 0 && v; --h) {
      if (!((v >> h) & 1)) continue;
      if (lead[h] == 0) {
        lead[h] = v;
        added = true;
        break;
      }
      v ^= lead[h];
    }
    if (!added) continue;
    ++nb;
    ord |= (uint64_t)b << (4 * j++);
    taken |= 1 << b;
  }
  for (int b = 0; b < m; ++b)
    if (!((rbmask >> b) & 1) && !((taken >> b) & 1))
      ord |= (uint64_t)b << (4 * j++);
  return ord;
}

// Offset (in amplitudes, within the state) of tile amplitude l: the low c
// bits are contiguous, bit c + j of l lands on global position hpos[j].
__device__ __forceinline__ uint64_t ts_tile_offset(const Stage2Args& a,
                                                   int l) {
  uint64_t off = (uint64_t)(l & ((1 << a.c) - 1));
  const int r = l >> a.c;
  for (int j = 0; j < a.m - a.c; ++j)
    if ((r >> j) & 1) off += uint64_t(1) << a.hpos[j];
  return off;
}

// One CTA's share of a register stage: tiles [cta * T / nctas,
// (cta + 1) * T / nctas) of the stage's T tiles.
template <typename R, int RB>
__device__ __forceinline__ void fused_reg_body(const Cx<R>* in, Cx<R>* out,
                                               const Cx<R>* pool,
                                               const Stage2Args& a,
                                               uint64_t cta, uint64_t nctas) {
  using C = Cx<R>;
  constexpr int NR = 1 << RB;
  constexpr int PER = 16 / sizeof(C);
  constexpr int NIT = NR / PER;  // 16-byte pieces per thread per tile
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* const S0 = reinterpret_cast<C*>(smem_raw);
  __shared__ TOp ops[TS_MAXG];
  __shared__ __align__(16) C mats[TS_MAXM + 4];
  // complex128 in pairs: the values as exact float triples
  constexpr bool kPairs = sizeof(R) == 8;
  __shared__ DEC matsd[kPairs ? TS_MAXM + 4 : 1];
  __shared__ int sh_pairs;
  __shared__ TLayout lay[TS_MAXL];
  __shared__ uint64_t offh[NIT];
  __shared__ int16_t nv[TS_MAXG];   // values per gate, then their offsets
  __shared__ int8_t vp[TS_MAXG];    // value permutation of each gate
  __shared__ int16_t grp[TS_MAXG];  // merged into the run headed by gate grp
  __shared__ int8_t gm[TS_MAXG];    // bit 0: diagonal values, bit 1: head
  __shared__ int sh_total;

  const int T = blockDim.x;
  const int tid = threadIdx.x;
  const int M = 1 << a.m;
  const uint64_t tps = uint64_t(1) << (a.n - a.m);
  const uint64_t num_tiles = (uint64_t)a.num_states * tps;
  const uint64_t t0 = cta * num_tiles / nctas;
  const uint64_t t1 = (cta + 1) * num_tiles / nctas;
  if (t0 >= t1) return;

  // the stage's gates are records [g0, g0 + G) of the program's array
  const int L = a.num_layouts;
  int g0 = 0x7fffffff, g1 = 0;
  for (int li = 0; li < L; ++li) {
    const Layout& ly = a.layouts[li];
    g0 = min(g0, ly.first_gate);
    g1 = max(g1, ly.first_gate + ly.num_gates);
  }
  if (g1 <= g0) g0 = g1 = 0;
  const int G = g1 - g0;
  const FusedGate* const gates = a.gates + g0;
  // resident: every layout and gate (and its values) decoded once
  bool resident = L <= TS_MAXL && G <= TS_MAXG;
  if (resident) {
    for (int gi = tid; gi < G; gi += T) {
      const FusedGate& g = gates[gi];
      // at least 4 values: a single-qubit diagonal that heads a merged
      // run of single-qubit gates holds their 2x2 product
      nv[gi] = (int16_t)max(fg_nvals(g.kind, g.nq), 4);
      vp[gi] = 0;
      grp[gi] = -1;
      gm[gi] = 0;
    }
    __syncthreads();
    if (tid == 0) {
      int s = 0;
      for (int gi = 0; gi < G; ++gi) {
        const int k = (nv[gi] + 1) & ~1;  // even offsets: 16-byte loads
        nv[gi] = (int16_t)s;
        s += k;
      }
      sh_total = s;
    }
    __syncthreads();
    resident = sh_total <= TS_MAXM;
  }
  bool batched = false;
  for (int gi = tid; gi < G; gi += T)
    batched |= gates[gi].mat_bstride != 0;
  batched = __syncthreads_or(batched);

  // per-layout address tables (resident layouts only; otherwise rebuilt
  // per layout below)
  auto build_layout = [&](int li, TLayout& dst, int e) {
    const Layout& ly = a.layouts[li];
    int rbmask = 0;
    for (int k = 0; k < RB; ++k) rbmask |= 1 << ly.rb[k];
    if (e < 48) {
      const int tbits = e < 32 ? e : (e - 32) << 5;
      const uint64_t ord = ts_thread_bit_order<R>(rbmask, a.m);
      int tb = 0, t = tbits;
      for (int j = 0; j < a.m - RB && t; ++j) {
        tb |= (t & 1) << ts_order_get(ord, j);
        t >>= 1;
      }
      if (e < 32) {
        dst.lo_r[e] = (uint16_t)tb;
        dst.lo_s[e] = (uint16_t)swz_amp<R>(tb);
      } else {
        dst.hi_r[e - 32] = (uint16_t)tb;
        dst.hi_s[e - 32] = (uint16_t)swz_amp<R>(tb);
      }
    } else if (e < 48 + RB) {
      dst.spo[e - 48] = swz_amp<R>(1 << ly.rb[e - 48]);
      dst.spw[e - 48] = dst.spo[e - 48];
    } else if (e == 48 + RB) {
      dst.first = ly.first_gate - g0;
      dst.count = ly.num_gates;
      dst.nscal = 0;
      dst.cw = 0;
    }
  };
  constexpr int LE = 48 + RB + 1;  // table entries per layout
  if (L <= TS_MAXL) {
    for (int idx = tid; idx < L * LE; idx += T)
      build_layout(idx / LE, lay[idx / LE], idx % LE);
  }
  for (int it = tid; it < NIT; it += T) offh[it] = ts_tile_offset(a, it * T * PER);
  const uint64_t offt = ts_tile_offset(a, tid * PER);

  // decode the resident gates and load values for state s
  bool has_runs = false;
  auto load_values = [&](uint64_t s) {
    for (int gi = tid; gi < G; gi += T) {
      const FusedGate& g = gates[gi];
      const int k = fg_nvals(g.kind, g.nq);
      const C* src = pool + g.mat + (int64_t)s * g.mat_bstride;
      const int mo = nv[gi];
      const int vm = vp[gi];  // value permutation from relabelling
      if (vm == 0) {
        for (int j = 0; j < k; ++j) mats[mo + j] = src[j];
      } else if (vm == VP_REV4) {
        for (int j = 0; j < 4; ++j) mats[mo + j] = src[3 - j];
      } else if (vm & VP_XOR4X4) {
        const int F = vm & 3;
        for (int j = 0; j < 16; ++j)
          mats[mo + j] = src[4 * ((j >> 2) ^ F) + ((j & 3) ^ F)];
      } else {  // VP_XORDIAG
        const int F = vm & 3;
        for (int j = 0; j < k; ++j) mats[mo + j] = src[j ^ F];
      }
    }
    if (!has_runs) return;
    __syncthreads();
    // merged runs of single-qubit gates: the head holds M_last ... M_first
    auto mat2 = [&](int gi, C* m) {
      const C* x = mats + nv[gi];
      if (gm[gi] & 1) {
        m[0] = x[0];
        m[1] = czero<C>();
        m[2] = czero<C>();
        m[3] = x[1];
      } else {
        for (int e = 0; e < 4; ++e) m[e] = x[e];
      }
    };
    for (int h = tid; h < G; h += T) {
      if (!(gm[h] & 2)) continue;
      C acc[4], g2[4], r[4];
      mat2(h, acc);
      for (int j = h + 1; j < G; ++j) {
        if (grp[j] != h) continue;
        mat2(j, g2);
        r[0] = cmad(g2[1], acc[2], cmul(g2[0], acc[0]));
        r[1] = cmad(g2[1], acc[3], cmul(g2[0], acc[1]));
        r[2] = cmad(g2[3], acc[2], cmul(g2[2], acc[0]));
        r[3] = cmad(g2[3], acc[3], cmul(g2[2], acc[1]));
        for (int e = 0; e < 4; ++e) acc[e] = r[e];
      }
      for (int e = 0; e < 4; ++e) mats[nv[h] + e] = acc[e];
    }
  };
  // complex128: split the resident values into exact triples; pairs are
  // used when every value lies in the pair range (block-uniform)
  auto to_pairs = [&]() {
    if constexpr (kPairs) {
      bool bad = false;
      for (int i = tid; i < sh_total; i += T) {
        const C m = mats[i];
        matsd[i] = df_entry2(m.x, m.y);
        const uint32_t e = max(df_hiword(m.x) & 0x7ff00000u,
                               df_hiword(m.y) & 0x7ff00000u);
        bad |= e >= ((DF_EMAX + 1) << 20);
      }
      bad = __syncthreads_or(bad);
      if (tid == 0) sh_pairs = a.df != 0 && !bad;
      __syncthreads();
    }
  };
  uint64_t loaded_s = t0 / tps;
  if (resident) {
    // One thread per layout walks its gates in order.
    //  * Thread scalars commute with everything a layout does: they move to
    //    the layout's front and run in a short loop of their own.
    //  * X and SWAP on register bits move no data: the layout keeps a
    //    relabelling (logical register bit k lives in physical bit perm[k],
    //    physical bits in `flip` hold complemented values); later
    //    operations are rewritten onto physical bits (matrix values
    //    permuted to match, vp) and the write-back uses the final map.
    __syncthreads();  // layout tables
    for (int li = tid; li < L; li += T) {
      const int f = lay[li].first, cnt = lay[li].count;
      const int32_t* rb = a.layouts[li].rb;
      int ns = 0;
      for (int j = f; j < f + cnt; ++j)
        ns += ts_decode<RB>(gates[j], nv[j], rb).op == TOP_SCALAR;
      int ps = f, po = f + ns;
      int perm[RB];
      for (int k = 0; k < RB; ++k) perm[k] = k;
      int flip = 0;
      // open run of unconditioned single-qubit gates per physical bit:
      // head gate and the position of its operation
      int run_head[RB], run_pos[RB];
      for (int k = 0; k < RB; ++k) run_head[k] = -1;
      for (int j = f; j < f + cnt; ++j) {
        TOp o = ts_decode<RB>(gates[j], nv[j], rb);
        vp[j] = 0;
        grp[j] = -1;
        gm[j] = 0;
        if (o.op == TOP_SCALAR) {
          ops[ps++] = o;
          continue;
        }
        if (!ts_relabel<RB>(o, perm, flip, vp[j])) continue;
        const int op = o.op;
        int b0 = -1, b1 = -1;  // physical register bits the op touches
        bool single = false;   // an unconditioned single-qubit 2x2
        if (op < TOP_DENSE2) {
          b0 = op % 5;
          single = op / 5 != TOP_SWAP1 / 5 && o.x == 0 && o.a == 0;
        } else if (op < TOP_DIAG1) {
          const int pp = (op - TOP_DENSE2) % 20;
          b0 = pp >> 2;
          b1 = (pp & 3) < b0 ? (pp & 3) : (pp & 3) + 1;
        } else if (op < TOP_DIAG2) {
          b0 = op - TOP_DIAG1;
          single = o.nq == 1;
          if (single) gm[j] = 1;
        } else if (op < TOP_SCALAR) {
          const int pp = op - TOP_DIAG2;
          b0 = pp >> 2;
          b1 = (pp & 3) < b0 ? (pp & 3) : (pp & 3) + 1;
        }
        if (single && run_head[b0] >= 0) {  // joins the open run
          grp[j] = (int16_t)run_head[b0];
          gm[run_head[b0]] |= 2;
          ops[run_pos[b0]].op = (int16_t)(TOP_DENSE1 + b0);
          has_runs = true;
          continue;
        }
        if (b0 >= 0) run_head[b0] = -1;
        if (b1 >= 0) run_head[b1] = -1;
        if (single) {
          run_head[b0] = j;
          run_pos[b0] = po;
        }
        ops[po++] = o;
      }
      lay[li].count = po - f;
      lay[li].nscal = ns;
      // physical bit b holds logical bit k with perm[k] == b
      int cw = 0;
      for (int k = 0; k < RB; ++k) {
        lay[li].spw[perm[k]] = lay[li].spo[k];
        if ((flip >> perm[k]) & 1) cw ^= lay[li].spo[k];
      }
      lay[li].cw = cw;
    }
    has_runs = __syncthreads_or(has_runs);
    load_values(loaded_s);
    __syncthreads();
    to_pairs();
  }

  auto tile_base = [&](uint64_t t) {
    uint64_t base = t % tps;
    for (int j = 0; j < a.m; ++j) base = insert_zero(base, a.spos[j]);
    return base;
  };
  auto prefetch = [&](uint64_t t, C* S) {
    const uint64_t s = t / tps;
    const C* src = in + s * a.in_stride + tile_base(t) + offt;
#pragma unroll
    for (int it = 0; it < NIT; ++it) {
      const int l = (tid + it * T) * PER;
      cp_async16<R>(&S[swz_amp<R>(l)], src + offh[it]);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };

  __syncthreads();  // tables, offh
  prefetch(t0, S0);
  C v[NR];
  for (uint64_t t = t0; t < t1; ++t) {
    C* S = S0 + (a.nbuf == 2 ? (int)((t - t0) & 1) * M : 0);
    cp_async_wait_all();
    __syncthreads();
    const uint64_t s = t / tps;
    if (resident && batched && s != loaded_s) {
      load_values(s);
      loaded_s = s;
      __syncthreads();
      to_pairs();
    }
    if (a.nbuf == 2 && t + 1 < t1) prefetch(t + 1, S0 + (int)((t + 1 - t0) & 1) * M);
    const uint64_t base = tile_base(t);
    bool tile_pairs = false;  // complex128: this tile runs in pairs

    for (int li = 0; li < L; ++li) {
      if (L > TS_MAXL) {  // rebuild this layout's tables in slot 0
        for (int idx = tid; idx < LE; idx += T) build_layout(li, lay[0], idx);
        __syncthreads();
      }
      const TLayout& ly = lay[L > TS_MAXL ? 0 : li];
      const int tb = ly.lo_r[tid & 31] | ly.hi_r[tid >> 5];
      const int sb = ly.lo_s[tid & 31] ^ ly.hi_s[tid >> 5];
      int sp[RB];
#pragma unroll
      for (int k = 0; k < RB; ++k) sp[k] = ly.spo[k];
      auto addr = [&](int i) {
        int x = sb;
#pragma unroll
        for (int k = 0; k < RB; ++k)
          if ((i >> k) & 1) x ^= sp[k];
        return x;
      };
      const int first = ly.first, count = ly.count;
      // write-back addresses: the final relabelling of register bits
      int spw[RB];
#pragma unroll
      for (int k = 0; k < RB; ++k) spw[k] = ly.spw[k];
      const int sbw = sb ^ ly.cw;
      auto waddr = [&](int i) {
        int x = sbw;
#pragma unroll
        for (int k = 0; k < RB; ++k)
          if ((i >> k) & 1) x ^= spw[k];
        return x;
      };
      // FP64 / complex64: the layout's operations on v
      auto run_plain = [&]() {
        C ts;
        ts.x = 1;
        ts.y = 0;
        if (resident) {
          const int ns = ly.nscal;
          for (int gi = first; gi < first + ns; ++gi) {
            const TOp o = ts_load_op(&ops[gi]);
            const int hb = o.nq == 2 ? 2 : 1;
            int fixed = ((tb & o.x) | ((base & o.a) != 0)) ? hb : 0;
            if ((tb & o.y) | ((base & o.b) != 0)) fixed |= 1;
            ts = cmul(ts, mats[o.moff + fixed]);
          }
          ts_run<C, C, RB>(v, ops, mats, first + ns, first + count, tb, base,
                           ts);
        } else {
          for (int c0 = 0; c0 < count; c0 += TS_CHUNK) {
            const int cnt = min(TS_CHUNK, count - c0);
            __syncthreads();  // the previous chunk is no longer read
            for (int j = tid; j < cnt; j += T) {
              const FusedGate& g = gates[first + c0 + j];
              ops[j] = ts_decode<RB>(g, 16 * j, a.layouts[li].rb);
              const C* src = pool + g.mat + (int64_t)s * g.mat_bstride;
              const int k = fg_nvals(g.kind, g.nq);
              for (int e = 0; e < k; ++e) mats[16 * j + e] = src[e];
            }
            __syncthreads();
            ts_run<C, C, RB>(v, ops, mats, 0, cnt, tb, base, ts);
          }
        }
        if (!is_one(ts)) {
#pragma unroll
          for (int i = 0; i < NR; ++i) v[i] = cmul(ts, v[i]);
        }
      };

      bool pairs = false;
      if constexpr (kPairs) pairs = resident && sh_pairs;  // block-uniform
      if (pairs) {
        if constexpr (kPairs) {
          // complex128 in pairs: the tile stays in shared memory as float
          // pairs (16 bytes, like a double2) from the first layout's read,
          // which splits, to the last layout's write, which renormalises
          // and joins; in between the pairs are left unnormalised
          float4* const S4 = reinterpret_cast<float4*>(S);
          DC w[NR];
          if (li == 0) {
            uint32_t mx = 0;
#pragma unroll
            for (int i = 0; i < NR; ++i) {
              v[i] = S[addr(i)];
              mx = max(mx, max(df_hiword(v[i].x) & 0x7ff00000u,
                               df_hiword(v[i].y) & 0x7ff00000u));
            }
            const bool ok = mx < ((DF_EMAX + 1) << 20) &&
                             (mx == 0 || mx >= (DF_EMIN << 20));
            tile_pairs = __syncthreads_and(ok);
            if (tile_pairs) {
#pragma unroll
              for (int i = 0; i < NR; ++i) w[i] = df_split2(v[i].x, v[i].y);
            }
          } else if (tile_pairs) {
#pragma unroll
            for (int i = 0; i < NR; ++i) {
              const float4 q = S4[addr(i)];
              w[i].re = DF{q.x, q.y};
              w[i].im = DF{q.z, q.w};
            }
          } else {
#pragma unroll
            for (int i = 0; i < NR; ++i) v[i] = S[addr(i)];
          }
          if (tile_pairs) {
            DC tsd;
            tsd.re = DF{1.f, 0.f};
            tsd.im = DF{0.f, 0.f};
            const int ns = ly.nscal;
            for (int gi = first; gi < first + ns; ++gi) {
              const TOp o = ts_load_op(&ops[gi]);
              const int hb = o.nq == 2 ? 2 : 1;
              int fixed = ((tb & o.x) | ((base & o.a) != 0)) ? hb : 0;
              if ((tb & o.y) | ((base & o.b) != 0)) fixed |= 1;
              tsd = op_scal(tsd, matsd[o.moff + fixed]);
            }
            ts_run<DC, DEC, RB>(w, ops, matsd, first + ns, first + count, tb,
                                base, tsd);
            if (!is_one(tsd)) {
#pragma unroll
              for (int i = 0; i < NR; ++i) w[i] = op_by_scal(tsd, w[i]);
            }
            if (li == L - 1) {
#pragma unroll
              for (int i = 0; i < NR; ++i) {
                C y;
                y.x = df_join(df_norm(w[i].re));
                y.y = df_join(df_norm(w[i].im));
                S[waddr(i)] = y;
              }
            } else {
#pragma unroll
              for (int i = 0; i < NR; ++i)
                S4[waddr(i)] = make_float4(w[i].re.hi, w[i].re.lo,
                                           w[i].im.hi, w[i].im.lo);
            }
          } else {
            run_plain();
#pragma unroll
            for (int i = 0; i < NR; ++i) S[waddr(i)] = v[i];
          }
        }
      } else {
#pragma unroll
        for (int i = 0; i < NR; ++i) v[i] = S[addr(i)];
        run_plain();
#pragma unroll
        for (int i = 0; i < NR; ++i) S[waddr(i)] = v[i];
      }
      __syncthreads();
    }

    C* dst = out + (s << a.n) + base + offt;
#pragma unroll
    for (int it = 0; it < NIT; ++it) {
      const int l = (tid + it * T) * PER;
      const int pl = swz_amp<R>(l);
      if constexpr (PER == 2) {
        const float4 w = *reinterpret_cast<const float4*>(&S[pl]);
        __stcs(reinterpret_cast<float4*>(dst + offh[it]), w);
      } else {
        __stcs(dst + offh[it], S[pl]);
      }
    }
    if (a.nbuf == 1 && t + 1 < t1) {
      __syncthreads();  // the tile buffer is free again
      prefetch(t + 1, S0);
    }
  }
  // drain: no cp.async may be outstanding when the CTA exits
  cp_async_wait_all();
}

template <typename R, int RB>
__global__ void __launch_bounds__(RB >= 5 ? 256 : 512, 1)
    fused_reg_kernel(const Cx<R>* in, Cx<R>* out, const Cx<R>* pool,
                     Stage2Args a) {
  fused_reg_body<R, RB>(in, out, pool, a, blockIdx.x, gridDim.x);
}

// Many register stages in one launch (one stage each of several programs
// with the same tile size): CTAs [cta_first[i], cta_first[i + 1]) run
// stage i.  The descriptors travel in the kernel's parameter block.
constexpr int MULTI_MAX = 48;
template <typename R>
struct MultiStage {
  const Cx<R>* in;
  Cx<R>* out;
  const Cx<R>* pool;
  Stage2Args a;
};
template <typename R>
struct MultiArgs {
  int num;
  int cta_first[MULTI_MAX + 1];
  MultiStage<R> st[MULTI_MAX];
};

template <typename R, int RB>
__global__ void __launch_bounds__(RB >= 5 ? 256 : 512, 1)
    fused_reg_multi_kernel(const __grid_constant__ MultiArgs<R> m) {
  int lo = 0, hi = m.num - 1;  // the last i with cta_first[i] <= blockIdx.x
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (m.cta_first[mid] <= (int)blockIdx.x)
      lo = mid;
    else
      hi = mid - 1;
  }
  const MultiStage<R>& d = m.st[lo];
  fused_reg_body<R, RB>(d.in, d.out, d.pool, d.a,
                        blockIdx.x - m.cta_first[lo],
                        m.cta_first[lo + 1] - m.cta_first[lo]);
}

}  // namespace gbsv

extern "C" int gbsv_fused_register_bits(int dtype) {
  return dtype == GBSV_C64 ? 4 : 3;
}

namespace {
template <typename R, int RB>
int launch_reg_stage(const void* state_in, void* state_out, const void* pool,
                     gbsv::Stage2Args a, int threads, cudaStream_t st) {
  using C = gbsv::Cx<R>;
  auto kern = gbsv::fused_reg_kernel<R, RB>;
  const size_t tile = sizeof(C) << a.m;
  // static shared memory of the kernel (tables, decoded gates, values)
  static int static_smem = -1;
  if (static_smem < 0) {
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, kern) != cudaSuccess)
      return gbsv::after_launch("fused_reg_kernel attributes");
    static_smem = (int)fa.sharedSizeBytes;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         227 * 1024 - static_smem);
  }
  a.nbuf = (2 * tile + (size_t)static_smem <= 227u * 1024u) ? 2 : 1;
  a.df = sizeof(R) == 8 && gbsv::c128_arith() == GBSV_C128_PAIRS;
  const size_t smem = tile * a.nbuf;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
  if (per_sm < 1) per_sm = 1;
  const uint64_t tiles = (uint64_t)a.num_states << (a.n - a.m);
  const uint64_t cap = (uint64_t)per_sm * gbsv::sm_count();
  const unsigned grid = (unsigned)(tiles < cap ? tiles : cap);
  kern<<<grid, threads, smem, st>>>(static_cast<const C*>(state_in),
                                    static_cast<C*>(state_out),
                                    static_cast<const C*>(pool), a);
  return gbsv::after_launch("fused_reg_kernel");
}
}  // namespace

namespace {
template <typename R, int RB>
int launch_reg_multi(const gbsv_multi_stage_t* stages, int num, int n,
                     int m, cudaStream_t st) {
  using C = gbsv::Cx<R>;
  auto kern = gbsv::fused_reg_multi_kernel<R, RB>;
  const size_t tile = sizeof(C) << m;
  static int static_smem = -1;
  if (static_smem < 0) {
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, kern) != cudaSuccess)
      return gbsv::after_launch("fused_reg_multi_kernel attributes");
    static_smem = (int)fa.sharedSizeBytes;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         227 * 1024 - static_smem);
  }
  const int nbuf = (2 * tile + (size_t)static_smem <= 227u * 1024u) ? 2 : 1;
  const size_t smem = tile * nbuf;
  const int threads = 1 << (m - RB);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
  if (per_sm < 1) per_sm = 1;
  const uint64_t cap = (uint64_t)per_sm * gbsv::sm_count();
  for (int first = 0; first < num; first += gbsv::MULTI_MAX) {
    const int cnt = std::min(num - first, gbsv::MULTI_MAX);
    gbsv::MultiArgs<R> ma{};
    ma.num = cnt;
    uint64_t total = 0;
    for (int i = 0; i < cnt; ++i)
      total += (uint64_t)stages[first + i].num_states << (n - m);
    int ctas = 0;
    for (int i = 0; i < cnt; ++i) {
      const gbsv_multi_stage_t& d = stages[first + i];
      gbsv::Stage2Args& a = ma.st[i].a;
      a.n = n;
      a.m = m;
      a.c = d.contiguous_qubits;
      a.in_stride = d.in_stride;
      a.gates = static_cast<const gbsv::FusedGate*>(d.gates);
      a.layouts = static_cast<const gbsv::Layout*>(d.layouts);
      a.num_layouts = d.num_layouts;
      a.num_states = d.num_states;
      a.nbuf = nbuf;
      a.df = sizeof(R) == 8 && gbsv::c128_arith() == GBSV_C128_PAIRS;
      for (int j = 0; j < m; ++j) {
        if (j >= a.c) a.hpos[j - a.c] = d.tile_positions[j];
        a.spos[j] = d.tile_positions[j];
      }
      for (int x = 1; x < m; ++x)
        for (int y = x; y > 0 && a.spos[y - 1] > a.spos[y]; --y) {
          const int t = a.spos[y];
          a.spos[y] = a.spos[y - 1];
          a.spos[y - 1] = t;
        }
      ma.st[i].in = static_cast<const C*>(d.state_in);
      ma.st[i].out = static_cast<C*>(d.state_out);
      ma.st[i].pool = static_cast<const C*>(d.pool);
      // CTAs in proportion to the stage's tiles (at least one each)
      const uint64_t tiles = (uint64_t)d.num_states << (n - m);
      uint64_t k = (cap * tiles + total - 1) / total;
      if (k > tiles) k = tiles;
      if (k < 1) k = 1;
      ma.cta_first[i] = ctas;
      ctas += (int)k;
    }
    ma.cta_first[cnt] = ctas;
    kern<<<ctas, threads, smem, st>>>(ma);
    const int rc = gbsv::after_launch("fused_reg_multi_kernel");
    if (rc) return rc;
  }
  return GBSV_OK;
}
}  // namespace

extern "C" int gbsv_run_stages_multi(int dtype, int num_qubits,
                                     int tile_qubits,
                                     const gbsv_multi_stage_t* stages,
                                     int num_stages, void* stream) {
  using namespace gbsv;
  if (dtype != GBSV_C64 && dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "state dtype must be complex");
  const int n = num_qubits, m = tile_qubits;
  const int rb = gbsv_fused_register_bits(dtype);
  const int mmax = gbsv_fused_max_tile_qubits(dtype);
  if (n < 1 || n > 62 || m < rb || m > mmax || m > n || m - rb > 9)
    return set_error(GBSV_ERR_INVALID_ARG, "bad multi stage n=%d m=%d", n,
                     m);
  if (num_stages < 0) return set_error(GBSV_ERR_INVALID_ARG, "num_stages");
  if (num_stages == 0) return GBSV_OK;
  if (!stages) return set_error(GBSV_ERR_INVALID_ARG, "null pointer");
  const int amp = dtype_bytes(dtype);
  const int cmin = dtype == GBSV_C64 ? 1 : 0;
  for (int i = 0; i < num_stages; ++i) {
    const gbsv_multi_stage_t& d = stages[i];
    if (d.num_states < 1 || d.in_stride < 0 || d.num_layouts < 1 ||
        d.contiguous_qubits < cmin || d.contiguous_qubits > m)
      return set_error(GBSV_ERR_INVALID_ARG, "bad stage %d", i);
    if (!d.state_in || !d.state_out || !d.gates || !d.layouts || !d.pool)
      return set_error(GBSV_ERR_INVALID_ARG, "null pointer in stage %d", i);
    if ((uintptr_t)d.state_in % 16 || (uintptr_t)d.state_out % 16 ||
        (d.in_stride * amp) % 16)
      return set_error(GBSV_ERR_INVALID_ARG,
                       "states must be 16-byte aligned");
    if (((uint64_t)d.num_states << (n - m)) > 0x7fffffffull)
      return set_error(GBSV_ERR_UNSUPPORTED, "too many tiles");
    uint64_t seen = 0;
    for (int j = 0; j < m; ++j) {
      const int p = d.tile_positions[j];
      if (p < 0 || p >= n || ((seen >> p) & 1) ||
          (j < d.contiguous_qubits && p != j))
        return set_error(GBSV_ERR_INVALID_ARG,
                         "bad tile position %d in stage %d", p, i);
      seen |= uint64_t(1) << p;
    }
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == GBSV_C64)
    return launch_reg_multi<float, 4>(stages, num_stages, n, m, st);
  return launch_reg_multi<double, 3>(stages, num_stages, n, m, st);
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
  a.num_states = num_states;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == GBSV_C64)
    return launch_reg_stage<float, 4>(state_in, state_out, pool, a, threads,
                                      st);
  return launch_reg_stage<double, 3>(state_in, state_out, pool, a, threads,
                                     st);
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
  // 16-byte copies: a misaligned state is left untouched (the whole CTA
  // returns before its first barrier)
  if (reinterpret_cast<uintptr_t>(st) % 16) return;
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
