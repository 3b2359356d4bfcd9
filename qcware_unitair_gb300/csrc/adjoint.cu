// Adjoint differentiation of expectation values.
//
// For E = <psi_L| H |psi_L> with psi_l = U_l psi_{l-1} and rotation gates
// U(theta) = exp(-i theta/2 P) (P = X, Y or Z on one qubit; RX(theta) =
// unitair's exp_x(theta/2)), the backward sweep keeps two states, psi_l and
// lambda_l = U_{l+1}^dag ... U_L^dag H psi_L, and for each rotation
//   dE/dtheta_l = 2 Re <lambda_l| dU/dtheta |psi_{l-1}> = Im <lambda_l|P|psi_l>
// then uncomputes both: psi_{l-1} = U^dag psi_l, lambda_{l-1} = U^dag lambda_l.
// No intermediate state is stored, so memory is two states (plus optional
// checkpoints) instead of one per gate as in autograd through
// apply_operator (src/unitair/simulation/operations.py:45-148 under torch
// autograd).
//
// gbsv_pauli_sum_apply:        lambda = H psi for H = sum_k c_k P_k.
// gbsv_adjoint_rotation_step:  one pass over (psi, lambda) per rotation:
//   reads each amplitude pair of both states once, accumulates the FP64
//   gradient partial, writes U^dag applied to both.  Partials per block go
//   to caller scratch; a second kernel sums them per state in a fixed order
//   and adds the result to grad[s * grad_stride].
#include "common.cuh"

namespace gbsv {

constexpr int ADJ_THREADS = 256;
constexpr int PAULI_MAX_TERMS = 256;

struct PauliTerm {
  uint64_t xmask;  // bit positions flipped (X or Y)
  uint64_t zmask;  // bit positions with a Z factor (Z or Y)
  double re, im;   // coefficient times i^(number of Y)
};

template <typename R>
__global__ void __launch_bounds__(256)
    pauli_apply_kernel(const Cx<R>* psi, Cx<R>* out, uint64_t total, int n,
                       const PauliTerm* terms, int num_terms) {
  __shared__ PauliTerm st[PAULI_MAX_TERMS];
  for (int k = threadIdx.x; k < num_terms; k += blockDim.x) st[k] = terms[k];
  __syncthreads();
  const uint64_t nmask = (uint64_t(1) << n) - 1;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
       i < total; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t x = i & nmask;
    const Cx<R>* p = psi + (i - x);
    // computed in the state's precision: the result is stored there
    R ar = 0, ai = 0;
    for (int k = 0; k < num_terms; ++k) {
      const uint64_t y = x ^ st[k].xmask;
      // (X^xm Z^zm)|y> = (-1)^popc(y & zm) |y ^ xm>, so
      // (P psi)[x] = c * (-1)^popc(y & zm) * psi[y] with y = x ^ xm
      const Cx<R> v = p[y];
      const R sgn = (__popcll(y & st[k].zmask) & 1) ? R(-1) : R(1);
      const R cr = sgn * (R)st[k].re, ci = sgn * (R)st[k].im;
      ar = fma(cr, v.x, fma(-ci, v.y, ar));
      ai = fma(cr, v.y, fma(ci, v.x, ai));
    }
    Cx<R> o;
    o.x = ar;
    o.y = ai;
    out[i] = o;
  }
}

// The same with V consecutive amplitudes (one 32-byte block) per thread:
// for each term the partner amplitudes y = x ^ xmask of the block are again
// one 32-byte block, read with one vector load, their order permuted by the
// low bits of xmask.
template <typename R, int V>
__global__ void __launch_bounds__(256)
    pauli_apply_block_kernel(const Cx<R>* psi, Cx<R>* out, uint64_t total,
                             int n, const PauliTerm* terms, int num_terms) {
  using C = Cx<R>;
  __shared__ PauliTerm st[PAULI_MAX_TERMS];
  for (int k = threadIdx.x; k < num_terms; k += blockDim.x) st[k] = terms[k];
  __syncthreads();
  const uint64_t nmask = (uint64_t(1) << n) - 1;
  for (uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * V;
       i < total; i += (uint64_t)gridDim.x * blockDim.x * V) {
    const uint64_t x = i & nmask;  // block start, low log2(V) bits zero
    const C* p = psi + (i - x);
    R ar[V], ai[V];
#pragma unroll
    for (int e = 0; e < V; ++e) ar[e] = ai[e] = 0;
    for (int k = 0; k < num_terms; ++k) {
      const uint64_t xm = st[k].xmask, zm = st[k].zmask;
      C b[V];
      load_chunk<V>(p + ((x ^ xm) & ~uint64_t(V - 1)), b);
      // b[e] holds amplitude ((x ^ xm) & ~(V-1)) + e; amplitude e of this
      // thread's block needs partner (x + e) ^ xm, i.e. b[e ^ (xm & (V-1))]
      if (xm & 1) {
#pragma unroll
        for (int e = 0; e < V; e += 2) {
          const C t = b[e];
          b[e] = b[e + 1];
          b[e + 1] = t;
        }
      }
      if constexpr (V == 4) {
        if (xm & 2) {
          C t = b[0];
          b[0] = b[2];
          b[2] = t;
          t = b[1];
          b[1] = b[3];
          b[3] = t;
        }
      }
      const R re = (R)st[k].re, im = (R)st[k].im;
#pragma unroll
      for (int e = 0; e < V; ++e) {
        const uint64_t y = (x + e) ^ xm;
        const R sgn = (__popcll(y & zm) & 1) ? R(-1) : R(1);
        const R cr = sgn * re, ci = sgn * im;
        ar[e] = fma(cr, b[e].x, fma(-ci, b[e].y, ar[e]));
        ai[e] = fma(cr, b[e].y, fma(ci, b[e].x, ai[e]));
      }
    }
    C o[V];
#pragma unroll
    for (int e = 0; e < V; ++e) {
      o[e].x = ar[e];
      o[e].y = ai[e];
    }
    store_chunk<V>(out + i, o);
  }
}

struct AdjArgs {
  int n, pos;             // qubits, target bit position
  int gen;                // 0 = X, 1 = Y, 2 = Z
  int64_t pairs;          // 2^(n-1) per state
  int parts;
  int64_t part_len;       // pairs per part
  const void* angles;
  int angle_f64;
  int64_t angle_stride;
  double angle_scale;
};

__device__ __forceinline__ double warp_sum_adj(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Warp sum of float values carried as an unevaluated pair (hi, lo): each
// butterfly step adds the partner's pair with TwoSum, so the result keeps
// about twice float precision with FP32 operations only (GB300 issues FP64
// at a small fraction of its FP32 rate).  Every lane ends with the same
// pair; the caller converts one lane's pair to double.
__device__ __forceinline__ void warp_sum_pair(float& hi, float& lo) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, hi, o);
    const float ol = __shfl_xor_sync(0xffffffffu, lo, o);
    const float s = hi + oh;
    const float bp = s - hi;
    const float e = (hi - (s - bp)) + (oh - bp);
    lo = lo + ol + e;
    hi = s;
  }
}

template <typename R>
__global__ void __launch_bounds__(ADJ_THREADS)
    adjoint_rot_kernel(Cx<R>* psi, Cx<R>* lam, AdjArgs a, double* partial) {
  using C = Cx<R>;
  const int64_t s = blockIdx.x / a.parts;
  const int part = blockIdx.x % a.parts;
  // U^dag = exp(+i theta/2 P) = cos I + i sin P; one FP64 sincos per block
  __shared__ R cs_sh[2];
  if (threadIdx.x == 0) {
    const double theta =
        a.angle_scale *
        (a.angle_f64
             ? static_cast<const double*>(a.angles)[s * a.angle_stride]
             : (double)static_cast<const float*>(a.angles)[s * a.angle_stride]);
    double sn, cs;
    sincos(0.5 * theta, &sn, &cs);
    cs_sh[0] = (R)cs;
    cs_sh[1] = (R)sn;
  }
  __syncthreads();
  const R c = cs_sh[0], sr = cs_sh[1];
  C* ps = psi + (s << a.n);
  C* ls = lam + (s << a.n);
  const int64_t lo = (int64_t)part * a.part_len;
  int64_t hi = lo + a.part_len;
  if (hi > a.pairs) hi = a.pairs;
  Acc<R> gacc;  // accumulates Im <lambda|P|psi>
  for (int64_t j = lo + threadIdx.x; j < hi; j += ADJ_THREADS) {
    const uint64_t i0 = insert_zero((uint64_t)j, a.pos);
    const uint64_t i1 = i0 | (uint64_t(1) << a.pos);
    const C p0 = ps[i0], p1 = ps[i1], l0 = ls[i0], l1 = ls[i1];
    // <lambda|P|psi> restricted to the pair, imaginary part only
    if (a.gen == 0) {  // conj(l0) p1 + conj(l1) p0
      gacc.add_prod(l0.x, p1.y);
      gacc.add_prod(-l0.y, p1.x);
      gacc.add_prod(l1.x, p0.y);
      gacc.add_prod(-l1.y, p0.x);
    } else if (a.gen == 1) {  // conj(l0)(-i p1) + conj(l1)(i p0)
      gacc.add_prod(l1.x, p0.x);
      gacc.add_prod(l1.y, p0.y);
      gacc.add_prod(-l0.x, p1.x);
      gacc.add_prod(-l0.y, p1.y);
    } else {  // conj(l0) p0 - conj(l1) p1
      gacc.add_prod(l0.x, p0.y);
      gacc.add_prod(-l0.y, p0.x);
      gacc.add_prod(-l1.x, p1.y);
      gacc.add_prod(l1.y, p1.x);
    }
    C q0, q1, m0, m1;
    if (a.gen == 0) {  // [[c, i s], [i s, c]]
      q0.x = c * p0.x - sr * p1.y; q0.y = c * p0.y + sr * p1.x;
      q1.x = c * p1.x - sr * p0.y; q1.y = c * p1.y + sr * p0.x;
      m0.x = c * l0.x - sr * l1.y; m0.y = c * l0.y + sr * l1.x;
      m1.x = c * l1.x - sr * l0.y; m1.y = c * l1.y + sr * l0.x;
    } else if (a.gen == 1) {  // [[c, s], [-s, c]]
      q0.x = c * p0.x + sr * p1.x; q0.y = c * p0.y + sr * p1.y;
      q1.x = c * p1.x - sr * p0.x; q1.y = c * p1.y - sr * p0.y;
      m0.x = c * l0.x + sr * l1.x; m0.y = c * l0.y + sr * l1.y;
      m1.x = c * l1.x - sr * l0.x; m1.y = c * l1.y - sr * l0.y;
    } else {  // diag(c + i s, c - i s)
      q0.x = c * p0.x - sr * p0.y; q0.y = c * p0.y + sr * p0.x;
      q1.x = c * p1.x + sr * p1.y; q1.y = c * p1.y - sr * p1.x;
      m0.x = c * l0.x - sr * l0.y; m0.y = c * l0.y + sr * l0.x;
      m1.x = c * l1.x + sr * l1.y; m1.y = c * l1.y - sr * l1.x;
    }
    ps[i0] = q0;
    ps[i1] = q1;
    ls[i0] = m0;
    ls[i1] = m1;
  }
  __shared__ double sh[ADJ_THREADS / 32];
  double gr = warp_sum_adj(gacc.value());
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = gr;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < ADJ_THREADS / 32 ? sh[threadIdx.x] : 0.0;
    v = warp_sum_adj(v);
    if (threadIdx.x == 0) partial[blockIdx.x] = v;
  }
}

__global__ void adjoint_finalize(const double* partial, int parts,
                                 int64_t num_states, double* grad,
                                 int64_t grad_stride, double factor) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= num_states) return;
  double acc = 0.0;
  for (int p = 0; p < parts; ++p) acc += partial[s * parts + p];
  grad[s * grad_stride] += factor * acc;
}

static int adj_parts(int64_t num_states, int64_t pairs, int64_t* len) {
  const int64_t want = (int64_t)sm_count() * 8;
  int64_t parts = (want + num_states - 1) / num_states;
  const int64_t max_parts = (pairs + 1023) / 1024;
  if (parts > max_parts) parts = max_parts;
  if (parts < 1) parts = 1;
  if (parts > 4096) parts = 4096;
  *len = (pairs + parts - 1) / parts;
  return (int)((pairs + *len - 1) / *len);
}

}  // namespace gbsv

using namespace gbsv;

extern "C" int gbsv_pauli_sum_apply(const void* psi, void* out, int dtype,
                                    int num_qubits, int64_t num_states,
                                    const void* terms, int num_terms,
                                    void* stream) {
  if (dtype != GBSV_C64 && dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "state dtype must be complex");
  if (num_qubits < 0 || num_qubits > 62 || num_states < 0 || num_terms < 0)
    return set_error(GBSV_ERR_INVALID_ARG, "bad sizes");
  if (num_terms > PAULI_MAX_TERMS)
    return set_error(GBSV_ERR_UNSUPPORTED, "more than %d Pauli terms",
                     PAULI_MAX_TERMS);
  if (num_states == 0) return GBSV_OK;
  if (!psi || !out || (num_terms > 0 && !terms))
    return set_error(GBSV_ERR_INVALID_ARG, "null pointer");
  if (psi == out)
    return set_error(GBSV_ERR_INVALID_ARG, "pauli_sum_apply is not in place");
  const uint64_t total = (uint64_t)num_states << num_qubits;
  uint64_t blocks = (total + 255) / 256;
  const uint64_t cap = (uint64_t)sm_count() * 16;
  if (blocks > cap) blocks = cap;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // 32-byte blocks need 4 (complex64) / 2 (complex128) amplitudes per state
  // and 32-byte aligned buffers
  const int V = dtype == GBSV_C64 ? 4 : 2;
  if ((num_qubits >= 2 || (dtype != GBSV_C64 && num_qubits >= 1)) &&
      (uintptr_t)psi % 32 == 0 && (uintptr_t)out % 32 == 0) {
    uint64_t vb = (total / V + 255) / 256;
    const uint64_t cap = (uint64_t)sm_count() * 32;
    if (vb > cap) vb = cap;
    if (vb < 1) vb = 1;
    if (dtype == GBSV_C64)
      pauli_apply_block_kernel<float, 4><<<(unsigned)vb, 256, 0, st>>>(
          static_cast<const float2*>(psi), static_cast<float2*>(out), total,
          num_qubits, static_cast<const PauliTerm*>(terms), num_terms);
    else
      pauli_apply_block_kernel<double, 2><<<(unsigned)vb, 256, 0, st>>>(
          static_cast<const double2*>(psi), static_cast<double2*>(out),
          total, num_qubits, static_cast<const PauliTerm*>(terms),
          num_terms);
    (void)V;
    return after_launch("pauli_apply_block_kernel");
  }
  if (dtype == GBSV_C64)
    pauli_apply_kernel<float><<<(unsigned)blocks, 256, 0, st>>>(
        static_cast<const float2*>(psi), static_cast<float2*>(out), total,
        num_qubits, static_cast<const PauliTerm*>(terms), num_terms);
  else
    pauli_apply_kernel<double><<<(unsigned)blocks, 256, 0, st>>>(
        static_cast<const double2*>(psi), static_cast<double2*>(out), total,
        num_qubits, static_cast<const PauliTerm*>(terms), num_terms);
  return after_launch("pauli_apply_kernel");
}

extern "C" size_t gbsv_adjoint_scratch_bytes(int64_t num_states,
                                             int num_qubits) {
  if (num_states <= 0 || num_qubits < 1 || num_qubits > 62) return 0;
  int64_t len = 0;
  const int parts =
      adj_parts(num_states, int64_t(1) << (num_qubits - 1), &len);
  return (size_t)num_states * parts * sizeof(double);
}

extern "C" int gbsv_adjoint_rotation_step(
    void* psi, void* lam, int dtype, int num_qubits, int64_t num_states,
    int qubit, int generator, const void* angles, int angle_dtype,
    int64_t angle_stride, double angle_scale, double* grad,
    int64_t grad_stride, double grad_factor, void* scratch,
    size_t scratch_bytes, void* stream) {
  if (dtype != GBSV_C64 && dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "state dtype must be complex");
  if (angle_dtype != GBSV_F32 && angle_dtype != GBSV_F64)
    return set_error(GBSV_ERR_INVALID_ARG, "angles must be float32/float64");
  const int n = num_qubits;
  if (n < 1 || n > 62 || qubit < 0 || qubit >= n || generator < 0 ||
      generator > 2 || num_states < 0 || angle_stride < 0)
    return set_error(GBSV_ERR_INVALID_ARG,
                     "bad adjoint step (n=%d qubit=%d generator=%d)", n, qubit,
                     generator);
  if (num_states == 0) return GBSV_OK;
  if (!psi || !lam || !angles || !grad || psi == lam)
    return set_error(GBSV_ERR_INVALID_ARG, "null or aliased pointer");
  AdjArgs a{};
  a.n = n;
  a.pos = n - 1 - qubit;
  a.gen = generator;
  a.pairs = int64_t(1) << (n - 1);
  a.parts = adj_parts(num_states, a.pairs, &a.part_len);
  a.angles = angles;
  a.angle_f64 = angle_dtype == GBSV_F64;
  a.angle_stride = angle_stride;
  a.angle_scale = angle_scale;
  const size_t need = (size_t)num_states * a.parts * sizeof(double);
  if (!scratch || scratch_bytes < need)
    return set_error(GBSV_ERR_SCRATCH, "adjoint step needs %zu scratch bytes",
                     need);
  const uint64_t blocks = (uint64_t)num_states * a.parts;
  if (blocks > 0x7fffffffull)
    return set_error(GBSV_ERR_UNSUPPORTED, "grid too large");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* partial = static_cast<double*>(scratch);
  if (dtype == GBSV_C64)
    adjoint_rot_kernel<float><<<(unsigned)blocks, ADJ_THREADS, 0, st>>>(
        static_cast<float2*>(psi), static_cast<float2*>(lam), a, partial);
  else
    adjoint_rot_kernel<double><<<(unsigned)blocks, ADJ_THREADS, 0, st>>>(
        static_cast<double2*>(psi), static_cast<double2*>(lam), a, partial);
  int rc = after_launch("adjoint_rot_kernel");
  if (rc) return rc;
  const unsigned fb = (unsigned)((num_states + 255) / 256);
  adjoint_finalize<<<fb, 256, 0, st>>>(partial, a.parts, num_states, grad,
                                       grad_stride, grad_factor);
  return after_launch("adjoint_finalize");
}

// ---------------------------------------------------------------------------
// Fused backward stages: one read and one write of psi and lambda per stage
// instead of per gate.  A stage holds the tiles of both states (same tile
// bits as a forward stage) in shared memory and walks its ops (the circuit's
// gates in reverse):
//   rotation U = exp(-i theta/2 P) on tile bit b (P = Z may also sit on a
//     bit outside the tile): accumulates Im <lambda|P|psi> over the tile,
//     block-reduces it into partial[slot][tile], and applies U^dag to both
//     tiles in the same sweep;
//   fixed gate: its adjoint (a gate record as in the forward stages, with
//     the conjugate-transposed matrix) is applied to both tiles; diagonal
//     factors from bits outside the tile multiply both states equally, so
//     they are deferred to the store and leave <lambda|P|psi> unchanged.
// A second kernel sums the partials of each (rotation, state) over the
// state's tiles in index order and adds them to the gradient.
namespace gbsv {

struct AdjOp {
  int32_t kind;   // 0 rotation, 1 fixed gate
  int32_t gen;    // rotation generator: 0 X, 1 Y, 2 Z
  int32_t bit;    // rotation: tile bit, or -1 - position (Z only)
  int32_t slot;   // rotation: gradient slot in this stage
  int32_t pidx;   // rotation: parameter index
  int32_t pad_;
  double scale;   // rotation: theta = scale * params[s, pidx]
  FusedGate g;    // fixed gate: record of its adjoint
};

struct AdjStageArgs {
  int n, m, c;
  int hpos[14];
  int spos[14];
  const AdjOp* ops;
  int num_ops;
  const void* params;
  int params_f64;
  int64_t num_params;
  int num_slots;
  const double* angles;  // (cos, sin) per (state, slot), from adjoint_angles
};

__device__ __forceinline__ int aswz(int l) {
  const int u = l >> 1;
  return ((u ^ ((u >> 3) & 7)) << 1) | (l & 1);
}

// A fixed gate's adjoint (record g, values mp) on both tiles, psi and
// lambda, in one sweep.
template <typename R>
__device__ __forceinline__ void adj_fixed(Cx<R>* SA, Cx<R>* SB, int M,
                                          uint64_t base, const FusedGate& g,
                                          const Cx<R>* mp) {
  using C = Cx<R>;
  constexpr int PER = 16 / sizeof(C);
  const int T = blockDim.x, tid = threadIdx.x;
  if (g.kind == 0) {  // dense 2x2 on tile bit b0
    const C m0 = mp[0], m1 = mp[1], m2 = mp[2], m3 = mp[3];
    for (int j = tid; j < (M >> 1); j += T) {
      const int i0 = (int)insert_zero((uint64_t)j, g.b0);
      const int i1 = i0 | (1 << g.b0);
      const int p0 = PER == 2 ? aswz(i0) : i0, p1 = PER == 2 ? aswz(i1) : i1;
      const C x0 = SA[p0], x1 = SA[p1], y0 = SB[p0], y1 = SB[p1];
      SA[p0] = cmad(m1, x1, cmul(m0, x0));
      SA[p1] = cmad(m3, x1, cmul(m2, x0));
      SB[p0] = cmad(m1, y1, cmul(m0, y0));
      SB[p1] = cmad(m3, y1, cmul(m2, y0));
    }
  } else if (g.kind == 1) {  // dense 4x4 on tile bits b0 (MSB), b1
    const int hi = g.b0 > g.b1 ? g.b0 : g.b1, lo = g.b0 > g.b1 ? g.b1 : g.b0;
    const int M0 = 1 << g.b0, M1 = 1 << g.b1;
    for (int j = tid; j < (M >> 2); j += T) {
      const int i = (int)insert_zero(insert_zero((uint64_t)j, lo), hi);
      int p[4] = {i, i | M1, i | M0, i | M0 | M1};
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (PER == 2) p[k] = aswz(p[k]);
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        C* S = t ? SB : SA;
        C v[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) v[k] = S[p[k]];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          C acc = cmul(mp[4 * r], v[0]);
          acc = cmad(mp[4 * r + 1], v[1], acc);
          acc = cmad(mp[4 * r + 2], v[2], acc);
          acc = cmad(mp[4 * r + 3], v[3], acc);
          S[p[r]] = acc;
        }
      }
    }
  } else {  // diagonal on nq qubits (tile bits or -1 - position); the
            // caller handles gates with every qubit outside the tile
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
    for (int l = tid; l < M; l += T) {
      int idx = gidx;
      if (lb0 >= 0) idx |= ((l >> lb0) & 1) << (g.nq - 1);
      if (lb1 >= 0) idx |= ((l >> lb1) & 1);
      const C f = mp[idx];
      if (f.x == 1 && f.y == 0) continue;
      const int pl = PER == 2 ? aswz(l) : l;
      SA[pl] = cmul(f, SA[pl]);
      SB[pl] = cmul(f, SB[pl]);
    }
  }
}

// One rotation's step on one amplitude pair (x0, x1 of psi, l0, l1 of
// lambda along the rotation's bit): adds Im <lambda|P|psi> restricted to the
// pair to g, then uncomputes both with U^dag = cos I + i sin P.
template <typename C, typename R>
__device__ __forceinline__ void adj_pair(int gen, R c, R sr, C& x0, C& x1,
                                         C& l0, C& l1, R& g) {
  C q0, q1, m0, m1;
  if (gen == 0) {  // X: conj(l0) x1 + conj(l1) x0
    g = fma(l0.x, x1.y, g);
    g = fma(-l0.y, x1.x, g);
    g = fma(l1.x, x0.y, g);
    g = fma(-l1.y, x0.x, g);
    q0.x = c * x0.x - sr * x1.y; q0.y = c * x0.y + sr * x1.x;
    q1.x = c * x1.x - sr * x0.y; q1.y = c * x1.y + sr * x0.x;
    m0.x = c * l0.x - sr * l1.y; m0.y = c * l0.y + sr * l1.x;
    m1.x = c * l1.x - sr * l0.y; m1.y = c * l1.y + sr * l0.x;
  } else if (gen == 1) {  // Y
    g = fma(l1.x, x0.x, g);
    g = fma(l1.y, x0.y, g);
    g = fma(-l0.x, x1.x, g);
    g = fma(-l0.y, x1.y, g);
    q0.x = c * x0.x + sr * x1.x; q0.y = c * x0.y + sr * x1.y;
    q1.x = c * x1.x - sr * x0.x; q1.y = c * x1.y - sr * x0.y;
    m0.x = c * l0.x + sr * l1.x; m0.y = c * l0.y + sr * l1.y;
    m1.x = c * l1.x - sr * l0.x; m1.y = c * l1.y - sr * l0.y;
  } else {  // Z
    g = fma(l0.x, x0.y, g);
    g = fma(-l0.y, x0.x, g);
    g = fma(-l1.x, x1.y, g);
    g = fma(l1.y, x1.x, g);
    q0.x = c * x0.x - sr * x0.y; q0.y = c * x0.y + sr * x0.x;
    q1.x = c * x1.x + sr * x1.y; q1.y = c * x1.y - sr * x1.x;
    m0.x = c * l0.x - sr * l0.y; m0.y = c * l0.y + sr * l0.x;
    m1.x = c * l1.x + sr * l1.y; m1.y = c * l1.y - sr * l1.x;
  }
  x0 = q0;
  x1 = q1;
  l0 = m0;
  l1 = m1;
}

// Warp partial of a rotation's gradient into wred[slot * warps + warp]:
// for complex64 the float pair itself (8 bytes), converted to double only
// in the end-of-stage reduction, where the lanes run over rotation slots
// (a conversion here would be a whole FP64 warp instruction per rotation).
template <typename R>
__device__ __forceinline__ void adj_warp_partial(R gsum, double* wred,
                                                 int slot, int T, int tid) {
  if constexpr (sizeof(R) == 4) {
    float hi = gsum, lo = 0.f;
    warp_sum_pair(hi, lo);
    if ((tid & 31) == 0)
      reinterpret_cast<float2*>(wred)[slot * (T >> 5) + (tid >> 5)] =
          make_float2(hi, lo);
  } else {
    const double gr = warp_sum_adj(gsum);
    if ((tid & 31) == 0) wred[slot * (T >> 5) + (tid >> 5)] = gr;
  }
}

// (cos, sin) of theta / 2 for every (state, rotation slot) of a stage, FP64
__global__ void adjoint_angles_kernel(AdjStageArgs a, int64_t num_states,
                                      double* out) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint64_t)num_states * a.num_ops) return;
  const uint64_t s = i / a.num_ops;
  const AdjOp& op = a.ops[i % a.num_ops];
  if (op.kind != 0) return;
  const double th =
      op.scale *
      (a.params_f64
           ? static_cast<const double*>(a.params)[s * a.num_params + op.pidx]
           : (double)static_cast<const float*>(
                 a.params)[s * a.num_params + op.pidx]);
  double sn, cs;
  sincos(0.5 * th, &sn, &cs);
  out[(s * a.num_slots + op.slot) * 2] = cs;
  out[(s * a.num_slots + op.slot) * 2 + 1] = sn;
}

template <typename R>
__global__ void __launch_bounds__(512, sizeof(R) == 4 ? 2 : 1)
    adjoint_stage_kernel(Cx<R>* psi, Cx<R>* lam, const Cx<R>* pool,
                         AdjStageArgs a, double* partial) {
  using C = Cx<R>;
  constexpr int PER = 16 / sizeof(C);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int M = 1 << a.m;
  C* SP = reinterpret_cast<C*>(smem_raw);
  C* SL = SP + M;
  // per-warp gradient partials of every rotation: wred[slot * warps + w]
  double* wred = reinterpret_cast<double*>(SL + M);
  __shared__ C scale_sh;
  const int T = blockDim.x, tid = threadIdx.x;
  const uint64_t tiles_per_state = uint64_t(1) << (a.n - a.m);
  const uint64_t s = blockIdx.x / tiles_per_state;
  uint64_t base = blockIdx.x % tiles_per_state;
  for (int j = 0; j < a.m; ++j) base = insert_zero(base, a.spos[j]);
  C* gp = psi + (s << a.n) + base;
  C* gl = lam + (s << a.n) + base;
  const int run = 1 << a.c;
  for (int l = tid * PER; l < M; l += T * PER) {
    const int r = l >> a.c;
    uint64_t off = (uint64_t)(l & (run - 1));
    for (int j = 0; j < a.m - a.c; ++j)
      if ((r >> j) & 1) off += uint64_t(1) << a.hpos[j];
    const int pl = PER == 2 ? aswz(l) : l;
    cp_async16<R>(&SP[pl], gp + off);
    cp_async16<R>(&SL[pl], gl + off);
  }
  if (tid == 0) {
    scale_sh.x = 1;
    scale_sh.y = 0;
  }
  // cos and sin of every rotation of the stage for this state, computed
  // once per state by adjoint_angles_kernel
  R* csn = reinterpret_cast<R*>(wred + a.num_slots * (T >> 5));
  for (int k = tid; k < 2 * a.num_slots; k += T)
    csn[k] = (R)a.angles[s * 2 * a.num_slots + k];
  cp_async_wait_all();
  __syncthreads();

  for (int oi = 0; oi < a.num_ops; ++oi) {
    const AdjOp& op = a.ops[oi];
    if (op.kind == 1) {
      if ((base & op.g.cmask) != op.g.cval) continue;
      const C* mp = pool + op.g.mat + (int64_t)s * op.g.mat_bstride;
      const bool all_global = op.g.kind == 2 && op.g.b0 < 0 &&
                              (op.g.nq < 2 || op.g.b1 < 0);
      if (all_global) {
        // one factor per tile, applied once to both states at the store
        if (tid == 0) {
          int gidx = 0;
          for (int q = 0; q < op.g.nq; ++q) {
            const int b = q == 0 ? op.g.b0 : op.g.b1;
            gidx |= (int)((base >> (-1 - b)) & 1) << (op.g.nq - 1 - q);
          }
          scale_sh = cmul(scale_sh, mp[gidx]);
        }
        continue;
      }
      adj_fixed<R>(SP, SL, M, base, op.g, mp);
      __syncthreads();
      continue;
    }
    const R c = csn[2 * op.slot], sr = csn[2 * op.slot + 1];
    // a thread sums only its few pairs of the tile (plain FMA); precision
    // is kept where the sums grow: across lanes, warps and tiles
    R gsum = 0;
    // the following rotations on tile bits share this sweep while the run
    // touches at most two bits (up to 4 rotations): pairs on one bit, quads
    // on two, kept in registers between the rotations
    int ng = 1, gb1 = op.bit, gb2 = -1;
    if (op.bit >= 0) {
      while (ng < 4 && oi + ng < a.num_ops) {
        const AdjOp& nx = a.ops[oi + ng];
        if (nx.kind != 0 || nx.bit < 0) break;
        if (nx.bit != gb1 && nx.bit != gb2) {
          if (gb2 >= 0) break;
          gb2 = nx.bit;
        }
        ++ng;
      }
    }
    if (op.bit < 0) {
      // Z on a bit outside the tile: the tile sits at z = +/-1
      const int zb = (int)((base >> (-1 - op.bit)) & 1);
      const R sgn = zb ? R(-1) : R(1);
      for (int l = tid; l < M; l += T) {
        const int pl = PER == 2 ? aswz(l) : l;
        const C p = SP[pl], q = SL[pl];
        gsum = fma(sgn * q.x, p.y, gsum);
        gsum = fma(-sgn * q.y, p.x, gsum);
      }
      if (tid == 0) {
        // U^dag = diag(e^{+i th/2}, e^{-i th/2}) restricted to this tile
        C f;
        f.x = c;
        f.y = zb ? -sr : sr;
        scale_sh = cmul(scale_sh, f);
        // a per-tile factor multiplies psi and lambda alike
      }
      adj_warp_partial<R>(gsum, wred, op.slot, T, tid);
    } else {
      R gs[4] = {0, 0, 0, 0};
      R cc[4], ss[4];
      int gen[4], bitk[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const AdjOp& rop = a.ops[oi + (r < ng ? r : 0)];
        cc[r] = csn[2 * rop.slot];
        ss[r] = csn[2 * rop.slot + 1];
        gen[r] = rop.gen;
        bitk[r] = rop.bit;
      }
      if (gb2 < 0) {
        for (int j = tid; j < (M >> 1); j += T) {
          const int i0 = (int)insert_zero((uint64_t)j, gb1);
          const int i1 = i0 | (1 << gb1);
          const int p0 = PER == 2 ? aswz(i0) : i0;
          const int p1 = PER == 2 ? aswz(i1) : i1;
          C x0 = SP[p0], x1 = SP[p1], l0 = SL[p0], l1 = SL[p1];
#pragma unroll
          for (int r = 0; r < 4; ++r)
            if (r < ng)
              adj_pair<C, R>(gen[r], cc[r], ss[r], x0, x1, l0, l1, gs[r]);
          SP[p0] = x0;
          SP[p1] = x1;
          SL[p0] = l0;
          SL[p1] = l1;
        }
      } else {
        const int lo_b = gb1 < gb2 ? gb1 : gb2, hi_b = gb1 < gb2 ? gb2 : gb1;
        for (int j = tid; j < (M >> 2); j += T) {
          const int i00 =
              (int)insert_zero(insert_zero((uint64_t)j, lo_b), hi_b);
          const int i10 = i00 | (1 << gb1), i01 = i00 | (1 << gb2);
          const int i11 = i10 | (1 << gb2);
          const int pa = PER == 2 ? aswz(i00) : i00;
          const int pb = PER == 2 ? aswz(i10) : i10;
          const int pc = PER == 2 ? aswz(i01) : i01;
          const int pd = PER == 2 ? aswz(i11) : i11;
          C xa = SP[pa], xb = SP[pb], xc = SP[pc], xd = SP[pd];
          C la = SL[pa], lb = SL[pb], lc = SL[pc], ld = SL[pd];
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            if (r >= ng) continue;
            if (bitk[r] == gb1) {  // pairs (a, b), (c, d)
              adj_pair<C, R>(gen[r], cc[r], ss[r], xa, xb, la, lb, gs[r]);
              adj_pair<C, R>(gen[r], cc[r], ss[r], xc, xd, lc, ld, gs[r]);
            } else {  // along gb2: pairs (a, c), (b, d)
              adj_pair<C, R>(gen[r], cc[r], ss[r], xa, xc, la, lc, gs[r]);
              adj_pair<C, R>(gen[r], cc[r], ss[r], xb, xd, lb, ld, gs[r]);
            }
          }
          SP[pa] = xa;
          SP[pb] = xb;
          SP[pc] = xc;
          SP[pd] = xd;
          SL[pa] = la;
          SL[pb] = lb;
          SL[pc] = lc;
          SL[pd] = ld;
        }
      }
#pragma unroll
      for (int r = 0; r < 4; ++r)
        if (r < ng)
          adj_warp_partial<R>(gs[r], wred, a.ops[oi + r].slot, T, tid);
      oi += ng - 1;  // the group's other rotations are done
    }
    __syncthreads();  // the next op reads amplitudes this one wrote
  }
  // one block reduction for all rotations of the stage
  {
    const int warps = T >> 5;
    for (int k = tid; k < a.num_slots; k += T) {
      double t = 0.0;
      for (int w = 0; w < warps; ++w) {
        if constexpr (sizeof(R) == 4) {
          const float2 q = reinterpret_cast<const float2*>(wred)[k * warps + w];
          t += (double)q.x + (double)q.y;
        } else {
          t += wred[k * warps + w];
        }
      }
      partial[(uint64_t)k * gridDim.x + blockIdx.x] = t;
    }
  }

  __syncthreads();  // scale_sh may have been updated by thread 0 alone
  const C sc = scale_sh;
  const bool scaled = !(sc.x == 1 && sc.y == 0);
  for (int l = tid * PER; l < M; l += T * PER) {
    const int r = l >> a.c;
    uint64_t off = (uint64_t)(l & (run - 1));
    for (int j = 0; j < a.m - a.c; ++j)
      if ((r >> j) & 1) off += uint64_t(1) << a.hpos[j];
    const int pl = PER == 2 ? aswz(l) : l;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      C p = SP[pl + k], q = SL[pl + k];
      if (scaled) {
        p = cmul(sc, p);
        q = cmul(sc, q);
      }
      gp[off + k] = p;
      gl[off + k] = q;
    }
  }
}

// grad[s * P + pidx[slot]] += scale[slot] * sum over the state's tiles
__global__ void adjoint_stage_finalize(const double* partial, int num_slots,
                                       uint64_t tiles_per_state,
                                       uint64_t num_tiles,
                                       const int32_t* pidx,
                                       const double* scale, double* grad,
                                       int64_t num_params) {
  const uint64_t item = blockIdx.x;  // slot * num_states + state
  const uint64_t num_states = num_tiles / tiles_per_state;
  const int slot = (int)(item / num_states);
  const uint64_t s = item % num_states;
  if (slot >= num_slots) return;
  double acc = 0.0;
  for (uint64_t t = threadIdx.x; t < tiles_per_state; t += blockDim.x)
    acc += partial[(uint64_t)slot * num_tiles + s * tiles_per_state + t];
  __shared__ double red[8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    grad[s * num_params + pidx[slot]] += scale[slot] * t;
  }
}

}  // namespace gbsv

using namespace gbsv;

extern "C" int gbsv_adjoint_stage(
    void* psi, void* lam, int dtype, int num_qubits, int64_t num_states,
    int tile_qubits, int contiguous_qubits, const int32_t* tile_positions,
    const void* ops, int num_ops, const void* pool, const void* params,
    int params_dtype, int64_t num_params, int num_slots,
    const int32_t* slot_param, const double* slot_scale, double* grad,
    void* scratch, size_t scratch_bytes, void* stream) {
  if (dtype != GBSV_C64 && dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "state dtype must be complex");
  if (params_dtype != GBSV_F32 && params_dtype != GBSV_F64)
    return set_error(GBSV_ERR_INVALID_ARG, "params must be float32/float64");
  const int n = num_qubits, m = tile_qubits, c = contiguous_qubits;
  const int mmax = dtype == GBSV_C64 ? 13 : 12;
  if (n < 1 || n > 62 || m < 1 || m > n || m > mmax ||
      c < (dtype == GBSV_C64 ? 1 : 0) || c > m || num_states < 0 ||
      num_ops < 0 || num_slots < 0 || num_params < 0)
    return set_error(GBSV_ERR_INVALID_ARG,
                     "bad adjoint stage n=%d m=%d c=%d", n, m, c);
  if (num_states == 0) return GBSV_OK;
  if (!psi || !lam || psi == lam || !tile_positions ||
      (num_ops > 0 && (!ops || !pool)) ||
      (num_slots > 0 && (!params || !slot_param || !slot_scale || !grad)))
    return set_error(GBSV_ERR_INVALID_ARG, "null or aliased pointer");
  if ((uintptr_t)psi % 16 || (uintptr_t)lam % 16)
    return set_error(GBSV_ERR_INVALID_ARG,
                     "psi and lambda must be 16-byte aligned");
  AdjStageArgs a{};
  a.n = n;
  a.m = m;
  a.c = c;
  a.ops = static_cast<const AdjOp*>(ops);
  a.num_ops = num_ops;
  a.params = params;
  a.params_f64 = params_dtype == GBSV_F64;
  a.num_params = num_params;
  a.num_slots = num_slots;
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
  const uint64_t tiles_per_state = uint64_t(1) << (n - m);
  const uint64_t tiles = (uint64_t)num_states * tiles_per_state;
  if (tiles > 0x7fffffffull)
    return set_error(GBSV_ERR_UNSUPPORTED, "too many tiles");
  // scratch: per-tile partials, then (cos, sin) per (state, slot)
  const size_t part_bytes = (size_t)num_slots * tiles * sizeof(double);
  const size_t need =
      part_bytes + (size_t)num_slots * num_states * 2 * sizeof(double);
  if (num_slots > 0 && (!scratch || scratch_bytes < need))
    return set_error(GBSV_ERR_SCRATCH, "adjoint stage needs %zu scratch bytes",
                     need);
  const int amp = dtype_bytes(dtype);
  int threads = (1 << m) / 4;
  if (threads > 512) threads = 512;
  if (threads < 32) threads = 32;
  const size_t smem = ((size_t)2 * amp << m) +
                      (size_t)num_slots * (threads / 32) * 8 +
                      (size_t)num_slots * amp;
  if (smem > 200 * 1024)
    return set_error(GBSV_ERR_UNSUPPORTED,
                     "adjoint stage with %d rotations needs %zu bytes of "
                     "shared memory", num_slots, smem);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* partial = static_cast<double*>(scratch);
  if (num_slots > 0) {
    double* angles = reinterpret_cast<double*>(
        static_cast<unsigned char*>(scratch) + part_bytes);
    a.angles = angles;
    const uint64_t items = (uint64_t)num_states * num_ops;
    if (items > 0) {
      adjoint_angles_kernel<<<(unsigned)((items + 255) / 256), 256, 0, st>>>(
          a, num_states, angles);
      const int rc = after_launch("adjoint_angles_kernel");
      if (rc) return rc;
    }
  }
  if (dtype == GBSV_C64) {
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(adjoint_stage_kernel<float>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           200 * 1024);
      attr = true;
    }
    adjoint_stage_kernel<float><<<(unsigned)tiles, threads, smem, st>>>(
        static_cast<float2*>(psi), static_cast<float2*>(lam),
        static_cast<const float2*>(pool), a, partial);
  } else {
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(adjoint_stage_kernel<double>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           200 * 1024);
      attr = true;
    }
    adjoint_stage_kernel<double><<<(unsigned)tiles, threads, smem, st>>>(
        static_cast<double2*>(psi), static_cast<double2*>(lam),
        static_cast<const double2*>(pool), a, partial);
  }
  int rc = after_launch("adjoint_stage_kernel");
  if (rc || num_slots == 0) return rc;
  const uint64_t items = (uint64_t)num_slots * num_states;
  if (items > 0x7fffffffull)
    return set_error(GBSV_ERR_UNSUPPORTED, "too many gradient slots");
  adjoint_stage_finalize<<<(unsigned)items, 256, 0, st>>>(
      partial, num_slots, tiles_per_state, tiles, slot_param, slot_scale,
      grad, num_params);
  return after_launch("adjoint_stage_finalize");
}
