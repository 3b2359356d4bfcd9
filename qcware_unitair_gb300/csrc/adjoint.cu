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
    double ar = 0.0, ai = 0.0;
    for (int k = 0; k < num_terms; ++k) {
      const uint64_t y = x ^ st[k].xmask;
      // (X^xm Z^zm)|y> = (-1)^popc(y & zm) |y ^ xm>, so
      // (P psi)[x] = c * (-1)^popc(y & zm) * psi[y] with y = x ^ xm
      const Cx<R> v = p[y];
      const double sgn = (__popcll(y & st[k].zmask) & 1) ? -1.0 : 1.0;
      const double cr = sgn * st[k].re, ci = sgn * st[k].im;
      ar += cr * (double)v.x - ci * (double)v.y;
      ai += cr * (double)v.y + ci * (double)v.x;
    }
    Cx<R> o;
    o.x = (R)ar;
    o.y = (R)ai;
    out[i] = o;
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

template <typename R>
__global__ void __launch_bounds__(ADJ_THREADS)
    adjoint_rot_kernel(Cx<R>* psi, Cx<R>* lam, AdjArgs a, double* partial) {
  using C = Cx<R>;
  const int64_t s = blockIdx.x / a.parts;
  const int part = blockIdx.x % a.parts;
  const double theta =
      a.angle_scale * (a.angle_f64
                           ? static_cast<const double*>(a.angles)[s * a.angle_stride]
                           : (double)static_cast<const float*>(a.angles)[s * a.angle_stride]);
  double sn, cs;
  sincos(0.5 * theta, &sn, &cs);
  // U^dag = exp(+i theta/2 P) = cos I + i sin P
  const R c = (R)cs, sr = (R)sn;
  C* ps = psi + (s << a.n);
  C* ls = lam + (s << a.n);
  const int64_t lo = (int64_t)part * a.part_len;
  int64_t hi = lo + a.part_len;
  if (hi > a.pairs) hi = a.pairs;
  double gr = 0.0;  // accumulates Im <lambda|P|psi>
  for (int64_t j = lo + threadIdx.x; j < hi; j += ADJ_THREADS) {
    const uint64_t i0 = insert_zero((uint64_t)j, a.pos);
    const uint64_t i1 = i0 | (uint64_t(1) << a.pos);
    const C p0 = ps[i0], p1 = ps[i1], l0 = ls[i0], l1 = ls[i1];
    // <lambda|P|psi> restricted to the pair, imaginary part only
    double im;
    if (a.gen == 0) {  // conj(l0) p1 + conj(l1) p0
      im = (double)l0.x * p1.y - (double)l0.y * p1.x + (double)l1.x * p0.y -
           (double)l1.y * p0.x;
    } else if (a.gen == 1) {  // conj(l0)(-i p1) + conj(l1)(i p0)
      im = -((double)l0.x * p1.x + (double)l0.y * p1.y) +
           ((double)l1.x * p0.x + (double)l1.y * p0.y);
    } else {  // conj(l0) p0 - conj(l1) p1
      im = (double)l0.x * p0.y - (double)l0.y * p0.x -
           ((double)l1.x * p1.y - (double)l1.y * p1.x);
    }
    gr += im;
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
  gr = warp_sum_adj(gr);
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
