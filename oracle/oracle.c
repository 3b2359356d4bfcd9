/*
 * CPU oracle for the state-vector hot path.  TEST INFRASTRUCTURE ONLY:
 * imported by tests/, by __graft_entry__.smoke() to check its result, and
 * by bench.py's CPU-baseline / reference arm.  The engine never calls it.
 *
 * It restates, in plain C, what unitair computes for
 *   apply_operator   src/unitair/simulation/operations.py:45-148
 *   (apply_operator_tensor :151-186, act_first_qubits_tensor :258-329)
 * on one already-broadcast batch: for every state s and every assignment of
 * the non-target qubits, the 2^k amplitudes selected by the target qubits
 * are gathered in matrix order (first listed qubit = matrix MSB, qubit 0 =
 * MSB of the amplitude index, conversions.py:5-45) and multiplied by the
 * operator: out[a] = sum_b op[a, b] * in[b]  (the einsum at :322).
 * The permute -> contiguous -> einsum -> permute data movement of the
 * reference is not restated; only its arithmetic result is.
 *
 * oracle_apply_c128: complex128 in/out and arithmetic (the parity oracle).
 * oracle_apply_c64:  complex64 in/out, float arithmetic, OpenMP threads
 *                    (the timed CPU port of the reference's c64 path).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_MAX_K 12

void oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int oracle_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static uint64_t insert_zeros(uint64_t x, const int* sorted_pos, int k) {
  for (int j = 0; j < k; ++j) {
    const int p = sorted_pos[j];
    const uint64_t lo = x & ((UINT64_C(1) << p) - 1);
    x = ((x >> p) << (p + 1)) | lo;
  }
  return x;
}

static int prepare(int n, const int* qubits, int k, int* pos, int* sorted,
                   uint64_t* offs) {
  if (k < 0 || k > ORACLE_MAX_K || k > n) return 1;
  for (int j = 0; j < k; ++j) {
    if (qubits[j] < 0 || qubits[j] >= n) return 1;
    for (int i = 0; i < j; ++i)
      if (qubits[i] == qubits[j]) return 1;
    pos[j] = n - 1 - qubits[j];
    sorted[j] = pos[j];
  }
  for (int i = 1; i < k; ++i) /* insertion sort, ascending */
    for (int j = i; j > 0 && sorted[j - 1] > sorted[j]; --j) {
      int t = sorted[j];
      sorted[j] = sorted[j - 1];
      sorted[j - 1] = t;
    }
  const int d = 1 << k;
  for (int b = 0; b < d; ++b) {
    uint64_t o = 0;
    for (int j = 0; j < k; ++j)
      if ((b >> (k - 1 - j)) & 1) o |= UINT64_C(1) << pos[j];
    offs[b] = o;
  }
  return 0;
}

int oracle_apply_c128(const double* in, double* out, int64_t num_states,
                      int n, int64_t in_stride, const double* ops,
                      int64_t op_stride, const int* qubits, int k) {
  int pos[ORACLE_MAX_K], sorted[ORACLE_MAX_K];
  static __thread uint64_t offs[1 << ORACLE_MAX_K];
  if (prepare(n, qubits, k, pos, sorted, offs)) return 1;
  const int d = 1 << k;
  const int64_t groups = (int64_t)1 << (n - k);
  const int64_t N = (int64_t)1 << n;
  double* buf = (double*)malloc(sizeof(double) * 4 * d);
  if (!buf) return 2;
  double* vin = buf;
  double* vout = buf + 2 * d;
  for (int64_t s = 0; s < num_states; ++s) {
    const double* src = in + 2 * s * in_stride;
    double* dst = out + 2 * s * N;
    const double* m = ops + 2 * s * op_stride;
    for (int64_t g = 0; g < groups; ++g) {
      const uint64_t base = insert_zeros((uint64_t)g, sorted, k);
      for (int b = 0; b < d; ++b) {
        vin[2 * b] = src[2 * (base + offs[b])];
        vin[2 * b + 1] = src[2 * (base + offs[b]) + 1];
      }
      for (int a = 0; a < d; ++a) {
        double re = 0.0, im = 0.0;
        for (int b = 0; b < d; ++b) {
          const double mr = m[2 * (a * d + b)], mi = m[2 * (a * d + b) + 1];
          re += mr * vin[2 * b] - mi * vin[2 * b + 1];
          im += mr * vin[2 * b + 1] + mi * vin[2 * b];
        }
        vout[2 * a] = re;
        vout[2 * a + 1] = im;
      }
      for (int a = 0; a < d; ++a) {
        dst[2 * (base + offs[a])] = vout[2 * a];
        dst[2 * (base + offs[a]) + 1] = vout[2 * a + 1];
      }
    }
  }
  free(buf);
  return 0;
}

/* complex64 port: float arithmetic, groups split across OpenMP threads. */
int oracle_apply_c64(const float* in, float* out, int64_t num_states, int n,
                     int64_t in_stride, const float* ops, int64_t op_stride,
                     const int* qubits, int k) {
  int pos[ORACLE_MAX_K], sorted[ORACLE_MAX_K];
  uint64_t* offs = (uint64_t*)malloc(sizeof(uint64_t) << (k < 0 ? 0 : k));
  if (!offs) return 2;
  if (prepare(n, qubits, k, pos, sorted, offs)) {
    free(offs);
    return 1;
  }
  const int d = 1 << k;
  const int64_t groups = (int64_t)1 << (n - k);
  const int64_t N = (int64_t)1 << n;
  const int64_t total = num_states * groups;
#pragma omp parallel
  {
    float* vin = (float*)malloc(sizeof(float) * 2 * d);
#pragma omp for schedule(static)
    for (int64_t t = 0; t < total; ++t) {
      const int64_t s = t / groups, g = t % groups;
      const float* src = in + 2 * s * in_stride;
      float* dst = out + 2 * s * N;
      const float* m = ops + 2 * s * op_stride;
      const uint64_t base = insert_zeros((uint64_t)g, sorted, k);
      for (int b = 0; b < d; ++b) {
        vin[2 * b] = src[2 * (base + offs[b])];
        vin[2 * b + 1] = src[2 * (base + offs[b]) + 1];
      }
      for (int a = 0; a < d; ++a) {
        float re = 0.f, im = 0.f;
        for (int b = 0; b < d; ++b) {
          const float mr = m[2 * (a * d + b)], mi = m[2 * (a * d + b) + 1];
          re += mr * vin[2 * b] - mi * vin[2 * b + 1];
          im += mr * vin[2 * b + 1] + mi * vin[2 * b];
        }
        dst[2 * (base + offs[a])] = re;
        dst[2 * (base + offs[a]) + 1] = im;
      }
    }
    free(vin);
  }
  free(offs);
  return 0;
}

/* sum_i |psi_i|^2 per state, complex128 accumulation (innerprod.py:29-46). */
void oracle_norm_squared_c128(const double* psi, int64_t num_states,
                              int64_t dim, double* out) {
  for (int64_t s = 0; s < num_states; ++s) {
    double acc = 0.0;
    const double* p = psi + 2 * s * dim;
    for (int64_t i = 0; i < dim; ++i)
      acc += p[2 * i] * p[2 * i] + p[2 * i + 1] * p[2 * i + 1];
    out[s] = acc;
  }
}
