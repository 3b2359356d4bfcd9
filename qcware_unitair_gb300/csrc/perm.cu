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
// gbsv_sample          draws indices from |psi|^2: FP64 sums of 1024-
//   amplitude chunks, a scan of those sums, then one warp per sample
//   (binary search over chunks, warp scan inside the chunk); uniforms come
//   from a counter-based hash of (seed, sample), so results do not depend on
//   launch order.  Replaces the Categorical sampling of measure
//   (src/unitair/simulation/measurement.py:9-70).
#include "common.cuh"

namespace gbsv {

struct PermArgs {
  int n;
  uint64_t total;
  int src_pos[64];  // output bit position p reads input bit position src_pos[p]
};

template <typename R>
__global__ void __launch_bounds__(256)
    permute_kernel(const Cx<R>* in, Cx<R>* out, PermArgs a) {
  const uint64_t nmask = (uint64_t(1) << a.n) - 1;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
       i < a.total; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t o = i & nmask;
    uint64_t src = 0;
    for (int p = 0; p < a.n; ++p) src |= ((o >> p) & 1) << a.src_pos[p];
    out[i] = in[(i - o) + src];
  }
}

template <typename R>
__global__ void __launch_bounds__(256)
    phase_flip_kernel(const Cx<R>* in, Cx<R>* out, uint64_t total, int n,
                      const uint64_t* masks, int num_masks) {
  __shared__ uint64_t sm[256];
  for (int k = threadIdx.x; k < num_masks; k += blockDim.x) sm[k] = masks[k];
  __syncthreads();
  const uint64_t nmask = (uint64_t(1) << n) - 1;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
       i < total; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t x = i & nmask;
    int parity = 0;
    for (int k = 0; k < num_masks; ++k) parity ^= (x & sm[k]) == sm[k];
    Cx<R> v = in[i];
    if (parity) {
      v.x = -v.x;
      v.y = -v.y;
    }
    out[i] = v;
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
constexpr int CHUNK = 1024;

template <typename R>
__global__ void __launch_bounds__(256)
    chunk_sum_kernel(const Cx<R>* psi, uint64_t num_chunks, uint64_t dim,
                     double* sums) {
  const uint64_t c = blockIdx.x;
  if (c >= num_chunks) return;
  const Cx<R>* p = psi + c * CHUNK;
  const uint64_t len = dim - c * CHUNK < (uint64_t)CHUNK ? dim - c * CHUNK
                                                         : (uint64_t)CHUNK;
  Acc<R> a;
  for (int i = threadIdx.x; i < (int)len; i += blockDim.x) {
    const Cx<R> v = p[i];
    a.add_prod(v.x, v.x);
    a.add_prod(v.y, v.y);
  }
  double acc = a.value();
  __shared__ double sh[8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
    sums[c] = t;
  }
}

// inclusive scan of num_chunks doubles by one block (sequential per thread
// over a contiguous slice, then a scan of the slice totals)
__global__ void __launch_bounds__(1024)
    scan_kernel(const double* sums, double* cdf, uint64_t num_chunks) {
  __shared__ double tot[1024];
  const uint64_t per = (num_chunks + blockDim.x - 1) / blockDim.x;
  const uint64_t lo = threadIdx.x * per;
  uint64_t hi = lo + per;
  if (hi > num_chunks) hi = num_chunks;
  double acc = 0.0;
  for (uint64_t i = lo; i < hi; ++i) acc += sums[i];
  tot[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double run = 0.0;
    for (int t = 0; t < (int)blockDim.x; ++t) {
      const double v = tot[t];
      tot[t] = run;
      run += v;
    }
  }
  __syncthreads();
  double run = tot[threadIdx.x];
  for (uint64_t i = lo; i < hi; ++i) {
    run += sums[i];
    cdf[i] = run;
  }
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  // splitmix64 finalizer (Steele, Lea, Flood 2014)
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

template <typename R>
__global__ void __launch_bounds__(256)
    sample_kernel(const Cx<R>* psi, const double* cdf, uint64_t num_chunks,
                  uint64_t dim, uint64_t num_samples, uint64_t seed,
                  int64_t* out) {
  const int lane = threadIdx.x & 31;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const double total = cdf[num_chunks - 1];
  for (uint64_t sidx = warp; sidx < num_samples; sidx += nwarps) {
    const uint64_t h = mix64(seed ^ mix64(sidx));
    const double u = (double)(h >> 11) * (1.0 / 9007199254740992.0) * total;
    // first chunk whose inclusive prefix exceeds u
    uint64_t lo = 0, hi = num_chunks - 1;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if (cdf[mid] > u) hi = mid; else lo = mid + 1;
    }
    double run = lo ? cdf[lo - 1] : 0.0;
    const uint64_t base = lo * CHUNK;
    uint64_t len = dim - base;
    if (len > CHUNK) len = CHUNK;
    int64_t found = -1;
    int64_t last_nonzero = -1;
    for (uint64_t off = 0; off < len && found < 0; off += 32) {
      double p = 0.0;
      if (off + lane < len) {
        const Cx<R> v = psi[base + off + lane];
        p = (double)v.x * v.x + (double)v.y * v.y;
      }
      double incl = p;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const double t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      const unsigned hit = __ballot_sync(0xffffffffu, p > 0.0 && run + incl > u);
      const unsigned nz = __ballot_sync(0xffffffffu, p > 0.0);
      if (nz) last_nonzero = (int64_t)(base + off) + 31 - __clz(nz);
      if (hit) found = (int64_t)(base + off) + __ffs(hit) - 1;
      run += __shfl_sync(0xffffffffu, incl, 31);
    }
    // rounding can leave u just above the chunk's own running sum
    if (found < 0) found = last_nonzero >= 0 ? last_nonzero : (int64_t)base;
    if (lane == 0) out[sidx] = found;
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
  PermArgs a{};
  a.n = n;
  a.total = (uint64_t)num_states << n;
  uint64_t seen = 0;
  for (int j = 0; j < n; ++j) {
    const int q = perm[j];
    if (q < 0 || q >= n || ((seen >> q) & 1))
      return set_error(GBSV_ERR_INVALID_ARG, "not a permutation of %d qubits",
                       n);
    seen |= uint64_t(1) << q;
    // output qubit j (bit n-1-j) reads input qubit q (bit n-1-q)
    a.src_pos[n - 1 - j] = n - 1 - q;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == GBSV_C64)
    permute_kernel<float><<<grid_for(a.total), 256, 0, st>>>(
        static_cast<const float2*>(in), static_cast<float2*>(out), a);
  else
    permute_kernel<double><<<grid_for(a.total), 256, 0, st>>>(
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
  if (dtype == GBSV_C64)
    phase_flip_kernel<float><<<grid_for(total), 256, 0, st>>>(
        static_cast<const float2*>(in), static_cast<float2*>(out), total,
        num_qubits, static_cast<const uint64_t*>(masks), num_masks);
  else
    phase_flip_kernel<double><<<grid_for(total), 256, 0, st>>>(
        static_cast<const double2*>(in), static_cast<double2*>(out), total,
        num_qubits, static_cast<const uint64_t*>(masks), num_masks);
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

extern "C" size_t gbsv_sample_scratch_bytes(int64_t dim) {
  if (dim <= 0) return 0;
  const uint64_t chunks = ((uint64_t)dim + CHUNK - 1) / CHUNK;
  return (size_t)chunks * 2 * sizeof(double);
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
  const uint64_t chunks = ((uint64_t)dim + CHUNK - 1) / CHUNK;
  if (dim % CHUNK != 0 && chunks > 1)
    return set_error(GBSV_ERR_INVALID_ARG, "dim must be a multiple of %d",
                     CHUNK);
  const size_t need = chunks * 2 * sizeof(double);
  if (!scratch || scratch_bytes < need)
    return set_error(GBSV_ERR_SCRATCH, "sampling needs %zu scratch bytes",
                     need);
  if (chunks > 0x7fffffffull)
    return set_error(GBSV_ERR_UNSUPPORTED, "state too large");
  double* sums = static_cast<double*>(scratch);
  double* cdf = sums + chunks;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int threads = dim < 256 ? 32 : 256;
  if (dtype == GBSV_C64)
    chunk_sum_kernel<float><<<(unsigned)chunks, threads, 0, st>>>(
        static_cast<const float2*>(state), chunks, (uint64_t)dim, sums);
  else
    chunk_sum_kernel<double><<<(unsigned)chunks, threads, 0, st>>>(
        static_cast<const double2*>(state), chunks, (uint64_t)dim, sums);
  int rc = after_launch("chunk_sum_kernel");
  if (rc) return rc;
  scan_kernel<<<1, 1024, 0, st>>>(sums, cdf, chunks);
  rc = after_launch("scan_kernel");
  if (rc) return rc;
  const uint64_t warps = (uint64_t)num_samples;
  uint64_t blocks = (warps * 32 + 255) / 256;
  const uint64_t cap = (uint64_t)sm_count() * 16;
  if (blocks > cap) blocks = cap;
  if (dtype == GBSV_C64)
    sample_kernel<float><<<(unsigned)blocks, 256, 0, st>>>(
        static_cast<const float2*>(state), cdf, chunks, (uint64_t)dim,
        (uint64_t)num_samples, seed, out_indices);
  else
    sample_kernel<double><<<(unsigned)blocks, 256, 0, st>>>(
        static_cast<const double2*>(state), cdf, chunks, (uint64_t)dim,
        (uint64_t)num_samples, seed, out_indices);
  return after_launch("sample_kernel");
}
