// Qubit permutations, multi-controlled gates and sampling.
//
// gbsv_permute_qubits  out qubit j <- in qubit perm[j]: one gather pass that
//   replaces unitair's permute_qubits / swap / roll_qubits
//   (src/unitair/simulation/operations.py:506-654), which are torch
//   permute + contiguous copies of the tensor layout.
// gbsv_phase_flip      diagonal sign (-1)^(number of masks whose bits are all
//   set): multi_cz (one mask per control/target pair, operations.py:657-748)
//   and multi_controlled_z (one mask of all qubits, :751-783) in one pass,
//   without unitair's 2^n integer phase tensors.
// gbsv_multi_controlled_x  swap of the target pair where every control is
//   1: the X that unitair builds as H, multi_controlled_z, H (:786-805).
// gbsv_sample          draws indices from |psi|^2: one pass builds sums of
//   amplitude groups and chunks and a prefix over the chunks, then one
//   thread per sample searches the chunks, the chunk's groups and the
//   group's amplitudes; uniforms come from a counter-based hash of (seed,
//   sample), so results do not depend on launch order.  Replaces the Categorical sampling of measure
//   (src/unitair/simulation/measurement.py:9-70).
#include <atomic>

#include "common.cuh"

namespace gbsv {

// A qubit permutation moves every amplitude; done as a tiled transpose so
// that both the reads and the writes are runs of 2^c contiguous amplitudes.
// Tile bits T (input positions): bits 0..c-1 (contiguous reads) plus the
// input bits that land on output bits 0..c-1 (contiguous writes), topped up
// with the lowest other bits to 12 for complex64 (c = 6: both sides move
// runs of at least 512 bytes, which a full qubit reversal needs to reach
// the copy rate) or 11 for complex128 (c = 5), 8 amplitudes per thread so
// the per-tile index work is amortised.  A CTA reads a tile in input
// order into shared memory and writes it back in output order; the other
// bits pick the tile and move as a block.
constexpr int PERM_MAX_TB = 12;
template <typename R>
constexpr int perm_tile_bits() { return sizeof(R) == 4 ? 12 : 11; }

struct PermArgs {
  int n, tb;
  int tin[PERM_MAX_TB];   // input bit of tile-local bit j (j < c: bit j)
  int wl[PERM_MAX_TB];    // output-local bit k: tile-local bit it comes from
  int wp[PERM_MAX_TB];    // output-local bit k: output bit (k < c: bit k)
  int rest_in[64];        // bits outside the tile, ascending
  int rest_out[64];       // ... and where they land
  uint64_t tiles_per_state, total_tiles;
};

// Shared-memory swizzle of tile element l: every group of higher bits is
// XOR-folded onto the bank bits (4 for 8-byte elements, 3 for 16-byte), so
// lanes that walk any single high tile bit still hit distinct banks, on
// the read side and on the write side of the transpose.
template <typename R>
__device__ __forceinline__ int perm_swz(int l) {
  return sizeof(R) == 4 ? (l ^ (((l >> 4) ^ (l >> 8)) & 15))
                        : (l ^ (((l >> 3) ^ (l >> 6) ^ (l >> 9)) & 7));
}

// O: the offset type of tile elements within a state (uint32_t up to 32
// qubits, which keeps the per-thread tables in registers)
template <typename R, typename O>
__global__ void __launch_bounds__(sizeof(R) == 4 ? 512 : 256, 2)
    permute_kernel(const Cx<R>* in, Cx<R>* out, PermArgs a) {
  using C = Cx<R>;
  __shared__ C S[1 << perm_tile_bits<R>()];
  const int M = 1 << a.tb, T = blockDim.x, tid = threadIdx.x;
  const int K = M / T;  // elements per thread per tile, <= 8
  // per-thread offsets of its K tile elements, read and write side
  O roff[8], woff[8];
  int rl[8], wsm[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    roff[k] = woff[k] = 0;
    rl[k] = wsm[k] = 0;
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    if (k >= K) break;
    const int l = tid + k * T;
    O ro = 0, wo = 0;
    int ls = 0;
    for (int j = 0; j < a.tb; ++j) {
      if ((l >> j) & 1) {
        ro |= O(1) << a.tin[j];
        wo |= O(1) << a.wp[j];
        ls |= 1 << a.wl[j];
      }
    }
    roff[k] = ro;
    rl[k] = perm_swz<R>(l);
    woff[k] = wo;
    wsm[k] = perm_swz<R>(ls);
  }
  // tile t's base offsets: bit j of its index within the state goes to
  // input bit rest_in[j] and output bit rest_out[j]; lane l handles bits l
  // and l + 32, an OR over the warp assembles the offsets
  const int lane = tid & 31, nrest = a.n - a.tb;
  const uint64_t in0 = lane < nrest ? uint64_t(1) << a.rest_in[lane] : 0;
  const uint64_t out0 = lane < nrest ? uint64_t(1) << a.rest_out[lane] : 0;
  const uint64_t in1 =
      lane + 32 < nrest ? uint64_t(1) << a.rest_in[lane + 32] : 0;
  const uint64_t out1 =
      lane + 32 < nrest ? uint64_t(1) << a.rest_out[lane + 32] : 0;
  auto bases = [&](uint64_t t, uint64_t* bin, uint64_t* bout) {
    const uint64_t s = t / a.tiles_per_state, r = t % a.tiles_per_state;
    const uint64_t i = (((r >> lane) & 1) ? in0 : 0) |
                       (((r >> (lane + 32)) & 1) ? in1 : 0);
    const uint64_t o = (((r >> lane) & 1) ? out0 : 0) |
                       (((r >> (lane + 32)) & 1) ? out1 : 0);
    *bin = (s << a.n) |
           ((uint64_t)__reduce_or_sync(0xffffffffu, (unsigned)(i >> 32))
            << 32) |
           __reduce_or_sync(0xffffffffu, (unsigned)i);
    *bout = (s << a.n) |
            ((uint64_t)__reduce_or_sync(0xffffffffu, (unsigned)(o >> 32))
             << 32) |
            __reduce_or_sync(0xffffffffu, (unsigned)o);
  };
  uint64_t t = blockIdx.x;
  if (t >= a.total_tiles) return;
  // the next tile's loads are issued before the current tile's stores
  C v[8];
  uint64_t bin, bout;
  bases(t, &bin, &bout);
#pragma unroll
  for (int k = 0; k < 8; ++k)
    if (k < K) v[k] = __ldcs(in + bin + roff[k]);
  for (; t < a.total_tiles; t += gridDim.x) {
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (k < K) S[rl[k]] = v[k];
    __syncthreads();
    C* dst = out + bout;
    const uint64_t nt = t + gridDim.x;
    if (nt < a.total_tiles) {
      bases(nt, &bin, &bout);
#pragma unroll
      for (int k = 0; k < 8; ++k)
        if (k < K) v[k] = __ldcs(in + bin + roff[k]);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (k < K) __stcs(dst + woff[k], S[wsm[k]]);
    __syncthreads();
  }
}

// V consecutive amplitudes per thread (32 bytes for complex64) so that
// every access is a full sector
template <typename R, int V>
__global__ void __launch_bounds__(256)
    phase_flip_kernel(const Cx<R>* in, Cx<R>* out, uint64_t total, int n,
                      const uint64_t* masks, int num_masks) {
  __shared__ uint64_t sm[256];
  for (int k = threadIdx.x; k < num_masks; k += blockDim.x) sm[k] = masks[k];
  __syncthreads();
  const uint64_t nmask = (uint64_t(1) << n) - 1;
  for (uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * V;
       i < total; i += (uint64_t)gridDim.x * blockDim.x * V) {
    Cx<R> v[V];
    load_chunk<V>(in + i, v);
    // the V amplitudes differ only in the low log2(V) index bits: a mask
    // fires for amplitude e when its high part is set in the shared high
    // bits and its low part is a subset of e
    const uint64_t hi = i & nmask;
    unsigned par = 0;  // bit e: parity of amplitude e
    for (int k = 0; k < num_masks; ++k) {
      const uint64_t m = sm[k];
      const unsigned lo = (unsigned)(m & (V - 1));
      if ((hi & (m & ~uint64_t(V - 1))) == (m & ~uint64_t(V - 1))) {
        unsigned sub = 0;  // amplitudes e with lo a subset of e
#pragma unroll
        for (int e = 0; e < V; ++e) sub |= (((unsigned)e & lo) == lo) << e;
        par ^= sub;
      }
    }
#pragma unroll
    for (int e = 0; e < V; ++e)
      if ((par >> e) & 1) {
        v[e].x = -v[e].x;
        v[e].y = -v[e].y;
      }
    store_chunk<V>(out + i, v);
  }
}

template <typename R>
__global__ void __launch_bounds__(256)
    mcx_kernel(const Cx<R>* in, Cx<R>* out, uint64_t pairs, int n, int tpos,
               uint64_t cmask) {
  const uint64_t half = uint64_t(1) << (n - 1);
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
       j < pairs; j += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t s = j / half, r = j % half;
    const uint64_t i0 = (s << n) + insert_zero(r, tpos);
    const uint64_t i1 = i0 + (uint64_t(1) << tpos);
    const Cx<R> a = in[i0], b = in[i1];
    const bool on = ((i0 - (s << n)) & cmask) == cmask;
    out[i0] = on ? b : a;
    out[i1] = on ? a : b;
  }
}

// ---- sampling ----------------------------------------------------------
// complex128 states and states under 256 amplitudes (complex64 states of
// whole 256-amplitude chunks take the finer tables further below).
// Three tables over the state: SUB[i] = sum |psi|^2 over 32-amplitude group
// i (FP32), SUMS[c] over 1024-amplitude chunk c (32 groups, FP64), CDF =
// inclusive prefix of SUMS.  A sample binary-searches CDF for its chunk,
// then scans the chunk's 32 group sums and the chosen group's 32
// amplitudes: 32 + 32 reads instead of up to 1024.  One thread per sample,
// so a warp has 32 independent searches in flight.
constexpr int CHUNK = 1024;
constexpr int GROUP = 32;

// one warp per chunk, lane l sums group l (32 contiguous amplitudes)
template <typename R>
__global__ void __launch_bounds__(256)
    chunk_sum_kernel(const Cx<R>* psi, uint64_t num_chunks, uint64_t dim,
                     double* sums, float* subs) {
  const int lane = threadIdx.x & 31;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t c = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
       c < num_chunks; c += nwarps) {
    const uint64_t base = c * CHUNK + (uint64_t)lane * GROUP;
    Acc<R> acc;
    if (base + GROUP <= dim) {
      constexpr int V = 32 / sizeof(Cx<R>);  // 32-byte pieces
#pragma unroll
      for (int j = 0; j < GROUP; j += V) {
        // cached loads: the lanes read 256 B apart, so both halves of a
        // sector are read by one lane in consecutive loads
        Cx<R> v[V];
        if constexpr (sizeof(R) == 4) {
          const float4 q0 = reinterpret_cast<const float4*>(psi + base + j)[0];
          const float4 q1 = reinterpret_cast<const float4*>(psi + base + j)[1];
          v[0] = make_float2(q0.x, q0.y);
          v[1] = make_float2(q0.z, q0.w);
          v[2] = make_float2(q1.x, q1.y);
          v[3] = make_float2(q1.z, q1.w);
        } else {
#pragma unroll
          for (int e = 0; e < V; ++e) v[e] = psi[base + j + e];
        }
#pragma unroll
        for (int e = 0; e < V; ++e) {
          acc.add_prod(v[e].x, v[e].x);
          acc.add_prod(v[e].y, v[e].y);
        }
      }
    } else {
      for (uint64_t i = base; i < dim && i < base + GROUP; ++i) {
        const Cx<R> v = psi[i];
        acc.add_prod(v.x, v.x);
        acc.add_prod(v.y, v.y);
      }
    }
    double g = acc.value();
    subs[c * GROUP + lane] = (float)g;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) g += __shfl_xor_sync(0xffffffffu, g, o);
    if (lane == 0) sums[c] = g;
  }
}

// Block-wide exclusive scan of one double per thread (blockDim.x <= 1024);
// returns the thread's exclusive prefix, *total the block's sum.
__device__ __forceinline__ double block_exclusive_scan(double v,
                                                       double* total) {
  __shared__ double wsum[33];  // warp offsets, then the block total
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    double x = lane < nw ? wsum[lane] : 0.0;
    double xi = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double t = __shfl_up_sync(0xffffffffu, xi, o);
      if (lane >= o) xi += t;
    }
    if (lane < nw) wsum[lane] = xi - x;  // exclusive warp offsets
    if (lane == nw - 1) wsum[32] = xi;   // block total
  }
  __syncthreads();
  const double r = wsum[w] + incl - v;
  *total = wsum[32];
  __syncthreads();
  return r;
}

// Scan in three steps: per-block totals of seg-chunk segments, an exclusive
// scan of the totals (one block), then each block's inclusive scan.
__global__ void __launch_bounds__(1024)
    scan_totals_kernel(const double* sums, uint64_t num_chunks, uint64_t seg,
                       double* tot) {
  const uint64_t lo = (uint64_t)blockIdx.x * seg;
  const uint64_t per = seg / blockDim.x;
  double acc = 0.0;
  for (uint64_t k = 0; k < per; ++k) {
    const uint64_t i = lo + threadIdx.x * per + k;
    if (i < num_chunks) acc += sums[i];
  }
  double total;
  block_exclusive_scan(acc, &total);
  if (threadIdx.x == 0) tot[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024)
    scan_offsets_kernel(double* tot, int num_blocks) {
  const double v = threadIdx.x < num_blocks ? tot[threadIdx.x] : 0.0;
  double total;
  const double ex = block_exclusive_scan(v, &total);
  if (threadIdx.x < num_blocks) tot[threadIdx.x] = ex;
}

__global__ void __launch_bounds__(1024)
    scan_blocks_kernel(const double* sums, uint64_t num_chunks, uint64_t seg,
                       const double* offsets, double* cdf) {
  const uint64_t lo = (uint64_t)blockIdx.x * seg;
  const uint64_t per = seg / blockDim.x;
  const uint64_t first = lo + threadIdx.x * per;
  double acc = 0.0;
  for (uint64_t k = 0; k < per; ++k)
    if (first + k < num_chunks) acc += sums[first + k];
  double total;
  double run = offsets[blockIdx.x] + block_exclusive_scan(acc, &total);
  for (uint64_t k = 0; k < per; ++k)
    if (first + k < num_chunks) {
      run += sums[first + k];
      cdf[first + k] = run;
    }
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  // splitmix64 finalizer (Steele, Lea, Flood 2014)
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// Picks, from a run of non-negative values v[0..k), the first k with
// v[k] > 0 and (inclusive prefix) > rem; without one, the last v[k] > 0
// (rounding can leave rem just above the run's own sum).  *excl_out = the
// exclusive prefix of the pick.
struct Pick {
  float excl = 0.f, pick_excl = 0.f, last_excl = 0.f;
  int pick = -1, last = -1;
  __device__ __forceinline__ void add(float v, int k, float rem) {
    const float incl = excl + v;
    if (v > 0.f) {
      if (pick < 0 && incl > rem) {
        pick = k;
        pick_excl = excl;
      }
      last = k;
      last_excl = excl;
    }
    excl = incl;
  }
  __device__ __forceinline__ int result(float* excl_out) const {
    if (pick >= 0) {
      *excl_out = pick_excl;
      return pick;
    }
    *excl_out = last_excl;
    return last;
  }
};

template <typename R>
__global__ void __launch_bounds__(256)
    sample_kernel(const Cx<R>* psi, const double* cdf, const float* subs,
                  uint64_t num_chunks, uint64_t dim, uint64_t num_samples,
                  uint64_t seed, int64_t* out) {
  const double total = cdf[num_chunks - 1];
  // every stride-th CDF value in shared memory: the first levels of the
  // search stay on chip
  constexpr int COARSE = 2048;
  __shared__ double coarse[COARSE];
  const uint64_t stride = (num_chunks + COARSE - 1) / COARSE;
  const int ncoarse = (int)((num_chunks + stride - 1) / stride);
  for (int i = threadIdx.x; i < ncoarse; i += blockDim.x) {
    uint64_t e = (uint64_t)(i + 1) * stride;
    if (e > num_chunks) e = num_chunks;
    coarse[i] = cdf[e - 1];
  }
  __syncthreads();
  const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t sidx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
       sidx < num_samples; sidx += nthreads) {
    const uint64_t h = mix64(seed ^ mix64(sidx));
    const double u = (double)(h >> 11) * (1.0 / 9007199254740992.0) * total;
    // first chunk whose inclusive prefix exceeds u: coarse block, then
    // within it
    int clo = 0, chi = ncoarse - 1;
    while (clo < chi) {
      const int mid = (clo + chi) >> 1;
      if (coarse[mid] > u) chi = mid; else clo = mid + 1;
    }
    uint64_t lo = (uint64_t)clo * stride;
    uint64_t hi = (uint64_t)(clo + 1) * stride;
    if (hi > num_chunks) hi = num_chunks;
    hi -= 1;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if (cdf[mid] > u) hi = mid; else lo = mid + 1;
    }
    const double run = lo ? cdf[lo - 1] : 0.0;
    // the rest of u inside the chunk; FP32 from here (a chunk's share only)
    float rem = (float)(u - run);
    // the chunk's 32 group sums: 128 contiguous bytes
    Pick gp;
    {
      const float4* sv = reinterpret_cast<const float4*>(subs + lo * GROUP);
      float4 q[GROUP / 4];
#pragma unroll
      for (int k = 0; k < GROUP / 4; ++k) q[k] = sv[k];
#pragma unroll
      for (int k = 0; k < GROUP / 4; ++k) {
        gp.add(q[k].x, 4 * k, rem);
        gp.add(q[k].y, 4 * k + 1, rem);
        gp.add(q[k].z, 4 * k + 2, rem);
        gp.add(q[k].w, 4 * k + 3, rem);
      }
    }
    float gex;
    int grp = gp.result(&gex);
    if (grp < 0) grp = 0;
    rem -= gex;
    const uint64_t gbase = lo * CHUNK + (uint64_t)grp * GROUP;
    Pick ap;
    if (gbase + GROUP <= dim) {
      // the group's amplitudes in 128-byte batches of 16-byte loads
      constexpr int PER = 16 / (int)sizeof(Cx<R>);  // amplitudes per load
      constexpr int BATCH = 8;                       // loads per batch
      const uint4* av = reinterpret_cast<const uint4*>(psi + gbase);
#pragma unroll
      for (int b = 0; b < GROUP / (PER * BATCH); ++b) {
        uint4 q[BATCH];
#pragma unroll
        for (int k = 0; k < BATCH; ++k) q[k] = av[b * BATCH + k];
#pragma unroll
        for (int k = 0; k < BATCH; ++k) {
          const Cx<R>* c = reinterpret_cast<const Cx<R>*>(&q[k]);
#pragma unroll
          for (int e = 0; e < PER; ++e)
            ap.add((float)((R)c[e].x * c[e].x + (R)c[e].y * c[e].y),
                   (b * BATCH + k) * PER + e, rem);
        }
      }
    } else {
      for (int k = 0; gbase + k < dim && k < GROUP; ++k) {
        const Cx<R> c = psi[gbase + k];
        ap.add((float)((R)c.x * c.x + (R)c.y * c.y), k, rem);
      }
    }
    float aex;
    const int a = ap.result(&aex);
    out[sidx] = (int64_t)gbase + (a < 0 ? 0 : a);
  }
}

// ---- sampling, complex64 states of whole 256-amplitude chunks ---------
// Finer tables so that a sample reads less at random: 16-amplitude groups
// (SUB2, FP32) inside 256-amplitude chunks, so a sample reads 64 bytes of
// group sums and 128 bytes of amplitudes (half of the 1024 / 32 layout;
// fewer bytes read at random per sample).  The table pass scans as it
// goes: each warp owns a contiguous segment of chunks and writes their
// segment-local inclusive prefix LCDF (FP64) and its total; one small
// kernel turns the totals into segment offsets.  The chunk CDF is
// 8 bytes per 256 amplitudes (32 MB at 30 qubits), L2-resident for the
// searches.
constexpr int SCHUNK = 256;
constexpr int SGROUP = 16;
constexpr int SGROUPS = SCHUNK / SGROUP;
// segments of the chunk table; the sample kernel keeps their offsets in
// shared memory ((segments + 1) doubles within 48 KB)
constexpr int STABLE_MAX_SEGS = 6016;

// Warp w of the grid owns the contiguous segment of chunks [w * per,
// (w + 1) * per) (per is a multiple of 4) and walks it in quads, keeping
// the running prefix as it goes, so the segment's local prefix LCDF needs
// no second pass.  Lane l loads float4 j * 32 + l of the quad, j < 16 (8 KB
// in flight per warp): amplitudes 64 j + 2 l and + 1, so after a 3-step
// butterfly lanes 8 q .. 8 q + 7 hold group 4 (j & 3) + q of chunk j / 4.
__global__ void __launch_bounds__(256)
    sample_table_c64_kernel(const float4* psi, uint64_t nchunks,
                            uint64_t per, double* lcdf, float* subs,
                            double* tot) {
  const int lane = threadIdx.x & 31;
  const uint64_t seg = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t first = seg * per;
  if (first >= nchunks) return;
  const uint64_t end = first + per < nchunks ? first + per : nchunks;
  double run = 0.0;  // lane 0: the segment's prefix so far
  for (uint64_t c4 = first; c4 < end; c4 += 4) {
    const float4* src = psi + c4 * (SCHUNK / 2);
    const int nq = end - c4 < 4 ? (int)(end - c4) : 4;  // chunks here
    float4 q[16];
#pragma unroll
    for (int j = 0; j < 16; ++j)
      q[j] = j / 4 < nq ? src[j * 32 + lane] : make_float4(0, 0, 0, 0);
    float g[16];
#pragma unroll
    for (int j = 0; j < 16; ++j)
      g[j] = fmaf(q[j].x, q[j].x,
                  fmaf(q[j].y, q[j].y, fmaf(q[j].z, q[j].z, q[j].w * q[j].w)));
#pragma unroll
    for (int o = 1; o < 8; o <<= 1)
#pragma unroll
      for (int j = 0; j < 16; ++j)
        g[j] += __shfl_xor_sync(0xffffffffu, g[j], o);
    const int grp = lane >> 3;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (k >= nq) break;
      const uint64_t c = c4 + k;
      if ((lane & 7) == 0) {
#pragma unroll
        for (int j = 0; j < 4; ++j)
          subs[c * SGROUPS + 4 * j + grp] = g[4 * k + j];
      }
      // the chunk sum: its 16 FP32 group sums added with error-free
      // TwoSum (lanes 0, 8, 16, 24 hold four each), so the chunk CDF and
      // the group sums agree
      float hi = 0.f, lo = 0.f;
      if ((lane & 7) == 0) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float x = g[4 * k + j];
          const float t = hi + x;
          const float bp = t - hi;
          lo += (hi - (t - bp)) + (x - bp);
          hi = t;
        }
      }
#pragma unroll
      for (int o = 8; o < 32; o <<= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, hi, o);
        const float ol = __shfl_xor_sync(0xffffffffu, lo, o);
        const float t = hi + oh;
        const float bp = t - hi;
        lo += ol + ((hi - (t - bp)) + (oh - bp));
        hi = t;
      }
      run += (double)hi + (double)lo;
      if (lane == 0) lcdf[c] = run;
    }
  }
  if (lane == 0) tot[seg] = run;
}

// Exclusive prefix of the segment totals, in place; tot[nb] = the sum.
__global__ void __launch_bounds__(1024)
    sample_offsets_kernel(double* tot, int nb) {
  constexpr int PER = (STABLE_MAX_SEGS + 1023) / 1024;
  double v[PER], s = 0.0;
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const int i = threadIdx.x * PER + k;
    v[k] = i < nb ? tot[i] : 0.0;
    s += v[k];
  }
  double total;
  double run = block_exclusive_scan(s, &total);
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const int i = threadIdx.x * PER + k;
    if (i < nb) tot[i] = run;
    run += v[k];
  }
  if (threadIdx.x == 0) tot[nb] = total;
}

// A segment of W consecutive lanes holds W * NV values in order (lane p of
// the segment holds values p * NV .. p * NV + NV - 1); every lane gets the
// Pick of the whole run (the first positive value whose inclusive prefix
// exceeds rem; without one the last positive value, -1 if none) and its
// exclusive prefix.  All 32 lanes call it together.
template <int W, int NV>
__device__ __forceinline__ int seg_pick(const float* v, float rem,
                                        float* excl_out) {
  const int lane = threadIdx.x & 31;
  const int p = lane & (W - 1);
  const unsigned seg = ((1u << W) - 1u) << (lane & ~(W - 1));
  float sum = 0.f;
#pragma unroll
  for (int j = 0; j < NV; ++j) sum += v[j];
  float incl = sum;
#pragma unroll
  for (int o = 1; o < W; o <<= 1) {
    const float t = __shfl_up_sync(0xffffffffu, incl, o, W);
    if (p >= o) incl += t;
  }
  const float up = __shfl_up_sync(0xffffffffu, incl, 1, W);
  Pick pk;
  pk.excl = p > 0 ? up : 0.f;
#pragma unroll
  for (int j = 0; j < NV; ++j) pk.add(v[j], p * NV + j, rem);
  const unsigned mp = __ballot_sync(0xffffffffu, pk.pick >= 0) & seg;
  const unsigned ml = __ballot_sync(0xffffffffu, pk.last >= 0) & seg;
  const bool use_pick = mp != 0;
  const int src = use_pick ? __ffs(mp) - 1
                  : ml    ? 31 - __clz(ml)
                          : (lane & ~(W - 1));
  const int idx = __shfl_sync(0xffffffffu,
                              use_pick ? pk.pick : pk.last, src);
  *excl_out = __shfl_sync(0xffffffffu,
                          use_pick ? pk.pick_excl : pk.last_excl, src);
  return idx;
}

__device__ __forceinline__ uint64_t shfl64(uint64_t x, int src) {
  const unsigned lo = __shfl_sync(0xffffffffu, (unsigned)x, src);
  const unsigned hi = __shfl_sync(0xffffffffu, (unsigned)(x >> 32), src);
  return ((uint64_t)hi << 32) | lo;
}

// SPT samples per thread in flight at once (independent search chains).
// The searches run per thread; the chunk's group sums (64 B) and the
// group's amplitudes (128 B) are then read cooperatively, 4 and 8 lanes
// per sample, so that one warp load touches 8 or 4 cache lines instead of
// 32 (the L1's per-line work bounded the per-thread version).  The sample
// loop is warp-uniform: all lanes take part in the shuffles.
template <int SPT>
__global__ void __launch_bounds__(256)
    sample_c64_kernel(const float4* psi, const double* lcdf,
                      const float* subs, const double* off, int nb,
                      uint64_t per, uint64_t nchunks, uint64_t num_samples,
                      uint64_t seed, int64_t* out) {
  extern __shared__ double soff[];  // segment offsets, then the total
  for (int i = threadIdx.x; i <= nb; i += blockDim.x) soff[i] = off[i];
  __syncthreads();
  const double total = soff[nb];
  const int lane = threadIdx.x & 31;
  const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
  const float4* subs4 = reinterpret_cast<const float4*>(subs);
  for (uint64_t wb = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31);
       wb < num_samples; wb += nthreads * SPT) {
    const uint64_t s0 = wb + lane;
    uint64_t c[SPT], lo[SPT], hi[SPT];
    double ub[SPT];
    bool live[SPT];
#pragma unroll
    for (int k = 0; k < SPT; ++k) {
      const uint64_t sidx = s0 + k * nthreads;
      live[k] = sidx < num_samples;
      const uint64_t h = mix64(seed ^ mix64(sidx));
      const double u = (double)(h >> 11) * (1.0 / 9007199254740992.0) * total;
      // the last segment whose offset is <= u (zero-mass segments are
      // skipped)
      int blo = 0, bhi = nb - 1;
      while (blo < bhi) {
        const int mid = (blo + bhi + 1) >> 1;
        if (soff[mid] <= u) blo = mid; else bhi = mid - 1;
      }
      ub[k] = u - soff[blo];
      lo[k] = (uint64_t)blo * per;
      hi[k] = lo[k] + per < nchunks ? lo[k] + per - 1 : nchunks - 1;
    }
    // first chunk of the segment whose local prefix exceeds the rest
    // (rounding can leave the rest above the segment's total: last chunk)
    bool busy = true;
    while (busy) {
      busy = false;
#pragma unroll
      for (int k = 0; k < SPT; ++k) {
        if (lo[k] < hi[k]) {
          const uint64_t mid = (lo[k] + hi[k]) >> 1;
          if (lcdf[mid] > ub[k]) hi[k] = mid; else lo[k] = mid + 1;
          busy = true;
        }
      }
    }
#pragma unroll
    for (int k = 0; k < SPT; ++k) {
      const uint64_t ck = lo[k];
      c[k] = ck;
      const uint64_t bfirst = (ck / per) * per;
      const double run = ck > bfirst ? lcdf[ck - 1] : 0.0;
      float rem = (float)(ub[k] - run);
      // group sums: in round r, lanes 4 q .. 4 q + 3 read the 16 group
      // sums of owner lane 8 r + q
      float4 gq[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const uint64_t co = shfl64(ck, 8 * r + (lane >> 2));
        gq[r] = subs4[co * (SGROUPS / 4) + (lane & 3)];
      }
      int grp = 0;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const float rem_o = __shfl_sync(0xffffffffu, rem, 8 * r + (lane >> 2));
        const float v[4] = {gq[r].x, gq[r].y, gq[r].z, gq[r].w};
        float ge;
        const int gi = seg_pick<4, 4>(v, rem_o, &ge);
        // owners 8 r .. 8 r + 7 take their segment's result
        const int src = ((lane - 8 * r) & 7) * 4;
        const int gi_o = __shfl_sync(0xffffffffu, gi, src);
        const float ge_o = __shfl_sync(0xffffffffu, ge, src);
        if ((lane >> 3) == r) {
          grp = gi_o < 0 ? 0 : gi_o;
          rem -= ge_o;
        }
      }
      // amplitudes: in round r, lanes 8 q .. 8 q + 7 read the 16 amplitudes
      // (two each) of owner lane 4 r + q
      const uint64_t gbase = ck * SCHUNK + (uint64_t)grp * SGROUP;
      float4 aq[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const uint64_t gb = shfl64(gbase, 4 * r + (lane >> 3));
        aq[r] = psi[gb / 2 + (lane & 7)];
      }
      int res = 0;
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const float rem_o = __shfl_sync(0xffffffffu, rem, 4 * r + (lane >> 3));
        const float v[2] = {fmaf(aq[r].x, aq[r].x, aq[r].y * aq[r].y),
                            fmaf(aq[r].z, aq[r].z, aq[r].w * aq[r].w)};
        float ae;
        const int ai = seg_pick<8, 2>(v, rem_o, &ae);
        const int src = ((lane - 4 * r) & 3) * 8;
        const int ai_o = __shfl_sync(0xffffffffu, ai, src);
        if ((lane >> 2) == r) res = ai_o < 0 ? 0 : ai_o;
      }
      if (live[k]) out[s0 + k * nthreads] = (int64_t)gbase + res;
    }
  }
}

static unsigned grid_for(uint64_t work) {
  uint64_t blocks = (work + 255) / 256;
  const uint64_t cap = (uint64_t)sm_count() * 32;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return (unsigned)blocks;
}

}  // namespace gbsv

using namespace gbsv;

extern "C" int gbsv_permute_qubits(const void* in, void* out, int dtype,
                                   int num_qubits, int64_t num_states,
                                   const int32_t* perm, void* stream) {
  if (dtype != GBSV_C64 && dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "state dtype must be complex");
  const int n = num_qubits;
  if (n < 0 || n > 62 || num_states < 0)
    return set_error(GBSV_ERR_INVALID_ARG, "bad sizes");
  if (num_states == 0) return GBSV_OK;
  if (!in || !out || (n > 0 && !perm))
    return set_error(GBSV_ERR_INVALID_ARG, "null pointer");
  if (in == out)
    return set_error(GBSV_ERR_INVALID_ARG, "permute_qubits is not in place");
  int src_pos[64], dst_pos[64];
  uint64_t seen = 0;
  for (int j = 0; j < n; ++j) {
    const int q = perm[j];
    if (q < 0 || q >= n || ((seen >> q) & 1))
      return set_error(GBSV_ERR_INVALID_ARG, "not a permutation of %d qubits",
                       n);
    seen |= uint64_t(1) << q;
    // output qubit j (bit n-1-j) reads input qubit q (bit n-1-q)
    src_pos[n - 1 - j] = n - 1 - q;
    dst_pos[n - 1 - q] = n - 1 - j;
  }
  PermArgs a{};
  a.n = n;
  const int tbmax = dtype == GBSV_C64 ? 12 : 11;
  const int cw = dtype == GBSV_C64 ? 6 : 5;
  const int c = n < cw ? n : cw;
  uint64_t tmask = (uint64_t(1) << c) - 1;
  for (int p = 0; p < c; ++p) tmask |= uint64_t(1) << src_pos[p];
  for (int b = 0; b < n && __builtin_popcountll(tmask) < tbmax; ++b)
    tmask |= uint64_t(1) << b;
  a.tb = __builtin_popcountll(tmask);
  // tile-local order: input bits 0..c-1 first, then the rest ascending
  int nl = 0;
  for (int b = 0; b < n; ++b)
    if ((tmask >> b) & 1) a.tin[nl++] = b;
  // output-local order: output positions of the tile bits, ascending
  int outs[PERM_MAX_TB], no = 0;
  for (int b = 0; b < n; ++b)
    if ((tmask >> src_pos[b]) & 1) outs[no++] = b;
  for (int k = 0; k < no; ++k) {
    a.wp[k] = outs[k];
    const int inb = src_pos[outs[k]];
    for (int j = 0; j < a.tb; ++j)
      if (a.tin[j] == inb) a.wl[k] = j;
  }
  int nr = 0;
  for (int b = 0; b < n; ++b)
    if (!((tmask >> b) & 1)) {
      a.rest_in[nr] = b;
      a.rest_out[nr] = dst_pos[b];
      ++nr;
    }
  a.tiles_per_state = uint64_t(1) << (n - a.tb);
  a.total_tiles = (uint64_t)num_states * a.tiles_per_state;
  // 8 elements per thread (tiles of 2^12 complex64 / 2^11 complex128: 512 /
  // 256 threads, the kernel's launch bound); a warp or less for tiny states
  const int M = 1 << a.tb;
  const int threads = M >= 256 ? M / 8 : (M < 32 ? M : 32);
  uint64_t grid = a.total_tiles;
  const uint64_t cap = (uint64_t)sm_count() * 4;
  if (grid > cap) grid = cap;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == GBSV_C64 && n <= 32)
    permute_kernel<float, uint32_t><<<(unsigned)grid, threads, 0, st>>>(
        static_cast<const float2*>(in), static_cast<float2*>(out), a);
  else if (dtype == GBSV_C64)
    permute_kernel<float, uint64_t><<<(unsigned)grid, threads, 0, st>>>(
        static_cast<const float2*>(in), static_cast<float2*>(out), a);
  else if (n <= 32)
    permute_kernel<double, uint32_t><<<(unsigned)grid, threads, 0, st>>>(
        static_cast<const double2*>(in), static_cast<double2*>(out), a);
  else
    permute_kernel<double, uint64_t><<<(unsigned)grid, threads, 0, st>>>(
        static_cast<const double2*>(in), static_cast<double2*>(out), a);
  return after_launch("permute_kernel");
}

extern "C" int gbsv_phase_flip(const void* in, void* out, int dtype,
                               int num_qubits, int64_t num_states,
                               const void* masks, int num_masks,
                               void* stream) {
  if (dtype != GBSV_C64 && dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "state dtype must be complex");
  if (num_qubits < 0 || num_qubits > 62 || num_states < 0 || num_masks < 0)
    return set_error(GBSV_ERR_INVALID_ARG, "bad sizes");
  if (num_masks > 256)
    return set_error(GBSV_ERR_UNSUPPORTED, "more than 256 masks");
  if (num_states == 0) return GBSV_OK;
  if (!in || !out || (num_masks > 0 && !masks))
    return set_error(GBSV_ERR_INVALID_ARG, "null pointer");
  const uint64_t total = (uint64_t)num_states << num_qubits;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const uint64_t* mk = static_cast<const uint64_t*>(masks);
  // 32-byte pieces need 4 (2) amplitudes per state and aligned buffers
  const bool wide = num_qubits >= 2 && (uintptr_t)in % 32 == 0 &&
                    (uintptr_t)out % 32 == 0;
  if (dtype == GBSV_C64) {
    auto i = static_cast<const float2*>(in);
    auto o = static_cast<float2*>(out);
    if (wide)
      phase_flip_kernel<float, 4><<<grid_for(total / 4), 256, 0, st>>>(
          i, o, total, num_qubits, mk, num_masks);
    else
      phase_flip_kernel<float, 1><<<grid_for(total), 256, 0, st>>>(
          i, o, total, num_qubits, mk, num_masks);
  } else {
    auto i = static_cast<const double2*>(in);
    auto o = static_cast<double2*>(out);
    if (wide)
      phase_flip_kernel<double, 2><<<grid_for(total / 2), 256, 0, st>>>(
          i, o, total, num_qubits, mk, num_masks);
    else
      phase_flip_kernel<double, 1><<<grid_for(total), 256, 0, st>>>(
          i, o, total, num_qubits, mk, num_masks);
  }
  return after_launch("phase_flip_kernel");
}

extern "C" int gbsv_multi_controlled_x(const void* in, void* out, int dtype,
                                       int num_qubits, int64_t num_states,
                                       const int32_t* controls,
                                       int num_controls, int target,
                                       void* stream) {
  if (dtype != GBSV_C64 && dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "state dtype must be complex");
  const int n = num_qubits;
  if (n < 1 || n > 62 || num_states < 0 || target < 0 || target >= n ||
      num_controls < 0)
    return set_error(GBSV_ERR_INVALID_ARG, "bad qubits");
  uint64_t cmask = 0;
  for (int k = 0; k < num_controls; ++k) {
    const int q = controls[k];
    if (q < 0 || q >= n || q == target)
      return set_error(GBSV_ERR_INVALID_ARG, "bad control qubit %d", q);
    cmask |= uint64_t(1) << (n - 1 - q);
  }
  if (num_states == 0) return GBSV_OK;
  if (!in || !out) return set_error(GBSV_ERR_INVALID_ARG, "null pointer");
  const uint64_t pairs = (uint64_t)num_states << (n - 1);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == GBSV_C64)
    mcx_kernel<float><<<grid_for(pairs), 256, 0, st>>>(
        static_cast<const float2*>(in), static_cast<float2*>(out), pairs, n,
        n - 1 - target, cmask);
  else
    mcx_kernel<double><<<grid_for(pairs), 256, 0, st>>>(
        static_cast<const double2*>(in), static_cast<double2*>(out), pairs,
        n, n - 1 - target, cmask);
  return after_launch("mcx_kernel");
}

// scratch: sums and cdf (one double per chunk each), group sums (32 per
// chunk), and 1024 segment totals
static uint64_t sample_chunks(int64_t dim) {
  return ((uint64_t)dim + CHUNK - 1) / CHUNK;
}

// The finer complex64 tables: segment-local chunk prefix (FP64) per
// 256-amplitude chunk, segment totals / offsets, group sums (FP32) per 16
// amplitudes.  Doubles before the group sums: the chunk prefix, the segment totals and
// their sum, rounded up to an even count so that the group sums start on
// a 16-byte boundary (they are read as float4).
static uint64_t sample2_doubles(uint64_t chunks) {
  return (chunks + STABLE_MAX_SEGS + 2 + 1) & ~uint64_t(1);
}

static size_t sample2_bytes(int64_t dim) {
  const uint64_t chunks = ((uint64_t)dim + SCHUNK - 1) / SCHUNK;
  return (size_t)sample2_doubles(chunks) * sizeof(double) +
         (size_t)chunks * SGROUPS * sizeof(float);
}

extern "C" size_t gbsv_sample_scratch_bytes(int64_t dim) {
  if (dim <= 0) return 0;
  const uint64_t chunks = sample_chunks(dim);
  // sums and CDF (FP64), group sums (FP32), scan totals
  const size_t one = (size_t)(chunks * 2 + 1024) * sizeof(double) +
                     (size_t)chunks * GROUP * sizeof(float);
  const size_t two = sample2_bytes(dim);
  return one > two ? one : two;
}

static int sample_c64_fine(const void* state, int64_t dim,
                           int64_t num_samples, uint64_t seed,
                           int64_t* out_indices, void* scratch,
                           cudaStream_t st) {
  const uint64_t nchunks = (uint64_t)dim / SCHUNK;
  // one segment per warp of one wave of the table pass (the occupancy
  // query once per device: it is host work before the first launch)
  static std::atomic<int> per_sm_of[64];
  int dev = 0;
  cudaGetDevice(&dev);
  int per_sm = per_sm_of[dev & 63].load(std::memory_order_relaxed);
  if (per_sm == 0) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, sample_table_c64_kernel, 256, 0);
    if (per_sm < 1) per_sm = 1;
    per_sm_of[dev & 63].store(per_sm, std::memory_order_relaxed);
  }
  uint64_t nb = (uint64_t)sm_count() * per_sm * 8;
  if (nb > STABLE_MAX_SEGS) nb = STABLE_MAX_SEGS;
  if (nb > (nchunks + 3) / 4) nb = (nchunks + 3) / 4;
  const uint64_t per = ((nchunks + nb - 1) / nb + 3) & ~uint64_t(3);
  nb = (nchunks + per - 1) / per;
  double* lcdf = static_cast<double*>(scratch);
  double* tot = lcdf + nchunks;  // nb totals, then the sum
  float* subs = reinterpret_cast<float*>(lcdf + sample2_doubles(nchunks));
  sample_table_c64_kernel<<<(unsigned)((nb + 7) / 8), 256, 0, st>>>(
      static_cast<const float4*>(state), nchunks, per, lcdf, subs, tot);
  int rc = after_launch("sample_table_c64_kernel");
  if (rc) return rc;
  sample_offsets_kernel<<<1, 1024, 0, st>>>(tot, (int)nb);
  rc = after_launch("sample_offsets_kernel");
  if (rc) return rc;
  constexpr int SPT = 4;
  uint64_t blocks = ((uint64_t)num_samples + 256 * SPT - 1) / (256 * SPT);
  const uint64_t cap = (uint64_t)sm_count() * 8;
  if (blocks > cap) blocks = cap;
  const size_t smem = (nb + 1) * sizeof(double);
  sample_c64_kernel<SPT><<<(unsigned)blocks, 256, smem, st>>>(
      static_cast<const float4*>(state), lcdf, subs, tot, (int)nb, per,
      nchunks, (uint64_t)num_samples, seed, out_indices);
  return after_launch("sample_c64_kernel");
}

extern "C" int gbsv_sample(const void* state, int dtype, int64_t dim,
                           int64_t num_samples, uint64_t seed,
                           int64_t* out_indices, void* scratch,
                           size_t scratch_bytes, void* stream) {
  if (dtype != GBSV_C64 && dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "state dtype must be complex");
  if (dim <= 0 || num_samples < 0)
    return set_error(GBSV_ERR_INVALID_ARG, "bad sizes");
  if (num_samples == 0) return GBSV_OK;
  if (!state || !out_indices)
    return set_error(GBSV_ERR_INVALID_ARG, "null pointer");
  const uint64_t chunks = sample_chunks(dim);
  if (dim % CHUNK != 0 && chunks > 1)
    return set_error(GBSV_ERR_INVALID_ARG, "dim must be a multiple of %d",
                     CHUNK);
  const size_t need = gbsv_sample_scratch_bytes(dim);
  if (!scratch || scratch_bytes < need)
    return set_error(GBSV_ERR_SCRATCH, "sampling needs %zu scratch bytes",
                     need);
  if ((uintptr_t)state % 16 || (uintptr_t)scratch % 16)
    return set_error(GBSV_ERR_INVALID_ARG,
                     "state and scratch must be 16-byte aligned");
  if (chunks > 0x7fffffffull)
    return set_error(GBSV_ERR_UNSUPPORTED, "state too large");
  cudaStream_t st0 = static_cast<cudaStream_t>(stream);
  if (dtype == GBSV_C64 && dim % SCHUNK == 0)
    return sample_c64_fine(state, dim, num_samples, seed, out_indices,
                           scratch, st0);
  double* sums = static_cast<double*>(scratch);
  double* cdf = sums + chunks;
  double* tot = cdf + chunks;
  float* subs = reinterpret_cast<float*>(tot + 1024);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  {
    uint64_t blocks = (chunks * 32 + 255) / 256;
    const uint64_t cap = (uint64_t)sm_count() * 16;
    if (blocks > cap) blocks = cap;
    if (dtype == GBSV_C64)
      chunk_sum_kernel<float><<<(unsigned)blocks, 256, 0, st>>>(
          static_cast<const float2*>(state), chunks, (uint64_t)dim, sums, subs);
    else
      chunk_sum_kernel<double><<<(unsigned)blocks, 256, 0, st>>>(
          static_cast<const double2*>(state), chunks, (uint64_t)dim, sums,
          subs);
  }
  int rc = after_launch("chunk_sum_kernel");
  if (rc) return rc;
  // segments of seg chunks (a multiple of 1024), at most 1024 of them
  uint64_t seg = 8192;
  while ((chunks + seg - 1) / seg > 1024) seg *= 2;
  const int nseg = (int)((chunks + seg - 1) / seg);
  scan_totals_kernel<<<nseg, 1024, 0, st>>>(sums, chunks, seg, tot);
  rc = after_launch("scan_totals_kernel");
  if (rc) return rc;
  scan_offsets_kernel<<<1, 1024, 0, st>>>(tot, nseg);
  rc = after_launch("scan_offsets_kernel");
  if (rc) return rc;
  scan_blocks_kernel<<<nseg, 1024, 0, st>>>(sums, chunks, seg, tot, cdf);
  rc = after_launch("scan_blocks_kernel");
  if (rc) return rc;
  uint64_t blocks = ((uint64_t)num_samples + 255) / 256;
  const uint64_t cap = (uint64_t)sm_count() * 8;
  if (blocks > cap) blocks = cap;
  if (dtype == GBSV_C64)
    sample_kernel<float><<<(unsigned)blocks, 256, 0, st>>>(
        static_cast<const float2*>(state), cdf, subs, chunks, (uint64_t)dim,
        (uint64_t)num_samples, seed, out_indices);
  else
    sample_kernel<double><<<(unsigned)blocks, 256, 0, st>>>(
        static_cast<const double2*>(state), cdf, subs, chunks, (uint64_t)dim,
        (uint64_t)num_samples, seed, out_indices);
  return after_launch("sample_kernel");
}
