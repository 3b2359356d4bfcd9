// Gradient of a k-qubit gate application with respect to the operator:
//   G_s[a, c] = sum_rest g_s[rest | a] * conj(psi_s[rest | c])
// where g = dL/d(out) and (rest | a) is the amplitude whose target bits
// spell matrix index a.  This is torch's convention for out = U @ psi
// (grad_U = grad_out @ psi^H), summed over every non-target qubit.  With a
// shared operator (out_stride == 0) the per-state matrices are summed too.
//
// Grid: one block per (state, matrix entry, slice of groups); FP64 partials
// go to caller scratch when a matrix entry needs more than one block, and a
// second kernel sums them in a fixed order (deterministic, no atomics).
#include "common.cuh"

namespace gbsv {

constexpr int OG_THREADS = 256;

struct OpGradArgs {
  int n, k;
  int64_t num_states;
  int64_t in_stride;   // amplitudes between psi states (0 = broadcast)
  int64_t groups;      // 2^(n-k)
  int parts;
  int64_t part_len;    // groups per part
  int sorted[GBSV_MAX_DENSE_QUBITS];
  int pos[GBSV_MAX_DENSE_QUBITS];
};

__device__ __forceinline__ uint64_t offset_of(const OpGradArgs& a, int idx) {
  uint64_t o = 0;
  for (int j = 0; j < a.k; ++j)
    if ((idx >> (a.k - 1 - j)) & 1) o |= uint64_t(1) << a.pos[j];
  return o;
}

__device__ __forceinline__ double warp_sum_og(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename R>
__global__ void __launch_bounds__(OG_THREADS)
    opgrad_kernel(const Cx<R>* g, const Cx<R>* psi, OpGradArgs a,
                  void* out, int direct, double* partial) {
  const int d = 1 << a.k;
  const int64_t per_state = (int64_t)d * d * a.parts;
  const int64_t s = blockIdx.x / per_state;
  const int64_t rem = blockIdx.x % per_state;
  const int e = (int)(rem / a.parts);
  const int p = (int)(rem % a.parts);
  const int ra = e / d, rc = e % d;
  const uint64_t oa = offset_of(a, ra), oc = offset_of(a, rc);
  const Cx<R>* gs = g + (s << a.n);
  const Cx<R>* ps = psi + s * a.in_stride;
  const int64_t lo = (int64_t)p * a.part_len;
  int64_t hi = lo + a.part_len;
  if (hi > a.groups) hi = a.groups;
  Acc<R> ax, ay;
  for (int64_t t = lo + threadIdx.x; t < hi; t += OG_THREADS) {
    uint64_t base = (uint64_t)t;
    for (int j = 0; j < a.k; ++j) {
      const int q = a.sorted[j];
      base = ((base >> q) << (q + 1)) | (base & ((uint64_t(1) << q) - 1));
    }
    const Cx<R> u = gs[base + oa];
    const Cx<R> v = ps[base + oc];
    // u * conj(v)
    ax.add_prod(u.x, v.x);
    ax.add_prod(u.y, v.y);
    ay.add_prod(u.y, v.x);
    ay.add_prod(-u.x, v.y);
  }
  double x = ax.value(), y = ay.value();
  __shared__ double sx[OG_THREADS / 32], sy[OG_THREADS / 32];
  x = warp_sum_og(x);
  y = warp_sum_og(y);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sx[w] = x;
    sy[w] = y;
  }
  __syncthreads();
  if (w == 0) {
    x = l < OG_THREADS / 32 ? sx[l] : 0.0;
    y = l < OG_THREADS / 32 ? sy[l] : 0.0;
    x = warp_sum_og(x);
    y = warp_sum_og(y);
    if (l == 0) {
      if (direct) {
        Cx<R> r;
        r.x = (R)x;
        r.y = (R)y;
        static_cast<Cx<R>*>(out)[s * d * d + e] = r;
      } else {
        partial[2 * blockIdx.x] = x;
        partial[2 * blockIdx.x + 1] = y;
      }
    }
  }
}

// One block per (output matrix m, entry e): sum the partials in order.
template <typename R>
__global__ void __launch_bounds__(OG_THREADS)
    opgrad_finalize(const double* partial, int64_t num_states, int d2,
                    int parts, int shared, void* out) {
  const int64_t m = blockIdx.x / d2;
  const int e = blockIdx.x % d2;
  const int64_t s_lo = shared ? 0 : m;
  const int64_t s_hi = shared ? num_states : m + 1;
  const int64_t count = (s_hi - s_lo) * parts;
  double x = 0.0, y = 0.0;
  for (int64_t t = threadIdx.x; t < count; t += OG_THREADS) {
    const int64_t s = s_lo + t / parts;
    const int p = (int)(t % parts);
    const int64_t idx = (s * d2 + e) * parts + p;
    x += partial[2 * idx];
    y += partial[2 * idx + 1];
  }
  __shared__ double sx[OG_THREADS / 32], sy[OG_THREADS / 32];
  x = warp_sum_og(x);
  y = warp_sum_og(y);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sx[w] = x;
    sy[w] = y;
  }
  __syncthreads();
  if (w == 0) {
    x = l < OG_THREADS / 32 ? sx[l] : 0.0;
    y = l < OG_THREADS / 32 ? sy[l] : 0.0;
    x = warp_sum_og(x);
    y = warp_sum_og(y);
    if (l == 0) {
      Cx<R> r;
      r.x = (R)x;
      r.y = (R)y;
      static_cast<Cx<R>*>(out)[m * d2 + e] = r;
    }
  }
}

struct OgPlan {
  int parts;
  int64_t part_len;
  bool direct;
};

static OgPlan og_plan(int64_t num_states, int n, int k, bool shared) {
  OgPlan p{1, int64_t(1) << (n - k), true};
  const int64_t groups = int64_t(1) << (n - k);
  const int64_t d2 = int64_t(1) << (2 * k);
  const int64_t blocks = num_states * d2;
  const int64_t want = (int64_t)sm_count() * 4;
  if (blocks < want && groups > 4096) {
    int64_t parts = (want + blocks - 1) / blocks;
    const int64_t max_parts = (groups + 4095) / 4096;
    if (parts > max_parts) parts = max_parts;
    if (parts > 1) {
      p.part_len = (groups + parts - 1) / parts;
      p.parts = (int)((groups + p.part_len - 1) / p.part_len);
    }
  }
  p.direct = (p.parts == 1) && !(shared && num_states > 1);
  return p;
}

}  // namespace gbsv

using namespace gbsv;

extern "C" size_t gbsv_operator_grad_scratch_bytes(int64_t num_states, int n,
                                                   int k, int shared) {
  if (n < 0 || k < 0 || k > n || k > GBSV_MAX_DENSE_QUBITS || num_states <= 0)
    return 0;
  const OgPlan p = og_plan(num_states, n, k, shared != 0);
  if (p.direct) return 0;
  return (size_t)num_states * ((size_t)1 << (2 * k)) * p.parts * 2 *
         sizeof(double);
}

extern "C" int gbsv_operator_grad(const void* grad_out, const void* state_in,
                                  int dtype, int num_qubits,
                                  int64_t num_states, int64_t in_stride,
                                  const int32_t* qubits, int num_targets,
                                  void* grad_ops, int shared, void* scratch,
                                  size_t scratch_bytes, void* stream) {
  if (dtype != GBSV_C64 && dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "state dtype must be complex");
  const int n = num_qubits, k = num_targets;
  if (n < 0 || n > 62 || k < 0 || k > n)
    return set_error(GBSV_ERR_INVALID_ARG, "bad qubit counts n=%d k=%d", n, k);
  if (k > 6)
    return set_error(GBSV_ERR_UNSUPPORTED,
                     "operator gradients for more than 6 qubits");
  if (num_states < 0 || in_stride < 0)
    return set_error(GBSV_ERR_INVALID_ARG, "negative size or stride");
  if (num_states == 0) return GBSV_OK;
  if (!grad_out || !state_in || !grad_ops || (k > 0 && !qubits))
    return set_error(GBSV_ERR_INVALID_ARG, "null pointer");
  OpGradArgs a{};
  a.n = n;
  a.k = k;
  a.num_states = num_states;
  a.in_stride = in_stride;
  a.groups = int64_t(1) << (n - k);
  uint64_t seen = 0;
  for (int j = 0; j < k; ++j) {
    const int q = qubits[j];
    if (q < 0 || q >= n || ((seen >> q) & 1))
      return set_error(GBSV_ERR_INVALID_ARG, "bad or repeated qubit %d", q);
    seen |= uint64_t(1) << q;
    a.pos[j] = n - 1 - q;
    a.sorted[j] = a.pos[j];
  }
  for (int i = 1; i < k; ++i)
    for (int j = i; j > 0 && a.sorted[j - 1] > a.sorted[j]; --j) {
      const int t = a.sorted[j];
      a.sorted[j] = a.sorted[j - 1];
      a.sorted[j - 1] = t;
    }
  const OgPlan p = og_plan(num_states, n, k, shared != 0);
  a.parts = p.parts;
  a.part_len = p.part_len;
  const int d2 = 1 << (2 * k);
  const uint64_t blocks = (uint64_t)num_states * d2 * p.parts;
  if (blocks > 0x7fffffffull)
    return set_error(GBSV_ERR_UNSUPPORTED, "grid too large");
  if (!p.direct) {
    const size_t need = (size_t)blocks * 2 * sizeof(double);
    if (!scratch || scratch_bytes < need)
      return set_error(GBSV_ERR_SCRATCH,
                       "operator gradient needs %zu scratch bytes", need);
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* partial = static_cast<double*>(scratch);
  if (dtype == GBSV_C64)
    opgrad_kernel<float><<<(unsigned)blocks, OG_THREADS, 0, st>>>(
        static_cast<const float2*>(grad_out),
        static_cast<const float2*>(state_in), a, grad_ops, p.direct, partial);
  else
    opgrad_kernel<double><<<(unsigned)blocks, OG_THREADS, 0, st>>>(
        static_cast<const double2*>(grad_out),
        static_cast<const double2*>(state_in), a, grad_ops, p.direct,
        partial);
  int rc = after_launch("opgrad_kernel");
  if (rc || p.direct) return rc;
  const int64_t outs = shared ? 1 : num_states;
  const unsigned fblocks = (unsigned)(outs * d2);
  if (dtype == GBSV_C64)
    opgrad_finalize<float><<<fblocks, OG_THREADS, 0, st>>>(
        partial, num_states, d2, p.parts, shared, grad_ops);
  else
    opgrad_finalize<double><<<fblocks, OG_THREADS, 0, st>>>(
        partial, num_states, d2, p.parts, shared, grad_ops);
  return after_launch("opgrad_finalize");
}
