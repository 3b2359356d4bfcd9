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

struct FusedGate {
  int32_t kind;
  int32_t nq;          // FG_DIAG: number of qubits (1 or 2)
  int32_t b0, b1;      // local bit (>= 0) or, for FG_DIAG, -1 - global pos
  uint64_t cmask;      // apply only where (tile base & cmask) == cval
  uint64_t cval;
  int64_t mat;         // complex-element offset into the matrix pool
  int64_t mat_bstride; // per-state stride in the pool (0 = shared)
};

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

template <typename R>
__device__ __forceinline__ void cp_async16(Cx<R>* smem, const Cx<R>* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s),
               "l"(gmem)
               : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
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

  // The current gate's matrix is staged in shared memory (a broadcast read
  // for every thread) so that 4x4 gates do not hold 32 registers.
  __shared__ C gmat[16];
  for (int gi = 0; gi < a.num_gates; ++gi) {
    const FusedGate g = a.gates[gi];
    if ((base & g.cmask) != g.cval) continue;  // uniform across the CTA
    const C* mp = pool + g.mat + (int64_t)s * g.mat_bstride;
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
        tscale = cmul(tscale, mp[gidx]);
        scaled = true;
        continue;  // a per-tile factor: no shared-memory pass
      }
    }
    const int nvals = g.kind == FG_DENSE1 ? 4 : g.kind == FG_DENSE2 ? 16
                                                                    : 1 << g.nq;
    if (tid < nvals) gmat[tid] = mp[tid];
    __syncthreads();
    if (g.kind == FG_DENSE1) {
      const C m0 = gmat[0], m1 = gmat[1], m2 = gmat[2], m3 = gmat[3];
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
      for (int j = tid; j < (M >> 2); j += T) {
        const int i = (int)insert_zero(insert_zero((uint64_t)j, lo), hi);
        int p[4] = {i, i | M1, i | M0, i | M0 | M1};
        C v[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          if (PER == 2) p[k] = swz(p[k]);
          v[k] = S[p[k]];
        }
        // matrix entries are re-read from shared memory each iteration
        // (volatile) instead of being hoisted into 32-64 registers
        const volatile C* vm = gmat;
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
      const C d0 = gmat[0], d1 = gmat[1];
      const C d2 = g.nq == 2 ? gmat[2] : d0, d3 = g.nq == 2 ? gmat[3] : d1;
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
