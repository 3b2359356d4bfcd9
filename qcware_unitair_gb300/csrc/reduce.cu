// Batched state reductions with FP64 accumulation: norm_squared,
// inner_product, diag_expectation_value, and the elementwise abs_squared.
//
// unitair computes these with torch elementwise temporaries and a sum in the
// state's own precision (src/unitair/states/innerprod.py:4-65), i.e. fp32
// accumulation for complex64 states.  Here each row is read once and
// accumulated in double; the result is rounded once to the output type.
//
// Plan: rows are split into `parts` slices so that the grid fills the GPU.
// With parts == 1 one block owns a row and writes the result directly.
// Otherwise every block writes an FP64 partial into caller-provided scratch
// and a second kernel sums the partials of each row in a fixed order, so the
// result is deterministic (no atomics).
#include <type_traits>

#include "common.cuh"

namespace gbsv {

constexpr int RED_THREADS = 256;

struct RowArgs {
  int64_t rows;
  int64_t dim;
  int parts;
  int64_t part_len;  // elements per part
  int ndim;          // row broadcast dims
  int64_t shape[GBSV_MAX_DIMS];
  int64_t sa[GBSV_MAX_DIMS];
  int64_t sb[GBSV_MAX_DIMS];
  int64_t ia, ib;    // inner strides (0 or 1)
};

struct Plan {
  int parts;
  int64_t part_len;
};

// blocks_per_sm: the launching kernel's resident blocks per SM, so that a
// single row splits into one wave; 16 (the most any reduction kernel keeps
// resident) gives the largest split, which sizes the scratch
static Plan make_plan(int64_t rows, int64_t dim, int blocks_per_sm = 16) {
  Plan p{1, dim};
  if (rows <= 0 || dim <= 0) return p;
  const int64_t want_blocks = (int64_t)sm_count() * blocks_per_sm;
  const int64_t min_len = 8192;
  if (rows >= want_blocks || dim <= min_len) return p;
  int64_t parts = (want_blocks + rows - 1) / rows;
  const int64_t max_parts = (dim + min_len - 1) / min_len;
  if (parts > max_parts) parts = max_parts;
  if (parts > 4096) parts = 4096;
  if (parts <= 1) return p;
  int64_t len = (dim + parts - 1) / parts;
  len = (len + 7) & ~int64_t(7);  // keep slices 16-byte aligned for c64
  parts = (dim + len - 1) / len;
  p.parts = (int)parts;
  p.part_len = len;
  return p;
}

// Resident blocks per SM of a RED_THREADS-thread reduction kernel (1..16).
template <typename Kernel>
static int resident_blocks(Kernel kernel) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, RED_THREADS,
                                                    0) != cudaSuccess) {
    (void)cudaGetLastError();
    nb = 16;
  }
  return nb < 1 ? 1 : (nb > 16 ? 16 : nb);
}

__device__ __forceinline__ void row_offsets(const RowArgs& a, int64_t row,
                                            int64_t* oa, int64_t* ob) {
  int64_t r = row, xa = 0, xb = 0;
  for (int d = a.ndim - 1; d >= 0; --d) {
    const int64_t idx = r % a.shape[d];
    r /= a.shape[d];
    xa += idx * a.sa[d];
    xb += idx * a.sb[d];
  }
  *oa = xa;
  *ob = xb;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of (x, y); result valid in thread 0.
__device__ __forceinline__ double2 block_sum2(double x, double y) {
  __shared__ double sx[RED_THREADS / 32], sy[RED_THREADS / 32];
  x = warp_sum(x);
  y = warp_sum(y);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sx[w] = x;
    sy[w] = y;
  }
  __syncthreads();
  double2 r = make_double2(0.0, 0.0);
  if (w == 0) {
    x = l < RED_THREADS / 32 ? sx[l] : 0.0;
    y = l < RED_THREADS / 32 ? sy[l] : 0.0;
    r.x = warp_sum(x);
    r.y = warp_sum(y);
  }
  return r;
}

template <typename T> __device__ __forceinline__ void store_out(T* p, double v);
template <> __device__ __forceinline__ void store_out<float>(float* p, double v) {
  *p = (float)v;
}
template <> __device__ __forceinline__ void store_out<double>(double* p, double v) {
  *p = v;
}

// ---- norm squared: contiguous rows ------------------------------------
template <typename R>
__global__ void __launch_bounds__(RED_THREADS)
    norm2_kernel(const Cx<R>* psi, int64_t dim, int parts, int64_t part_len,
                 void* out, int out_f64, double* partial) {
  const int64_t row = blockIdx.x / parts;
  const int part = blockIdx.x % parts;
  const int64_t lo = (int64_t)part * part_len;
  int64_t hi = lo + part_len;
  if (hi > dim) hi = dim;
  const Cx<R>* p = psi + row * dim;
  Acc<R> acc;
  int64_t i = lo + threadIdx.x;
  // four elements per step; the next step's loads are in flight while this
  // step's sums run
  Cx<R> v[4];
  bool have = i + 3 * RED_THREADS < hi;
  if (have) {
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = __ldcs(p + i + k * RED_THREADS);
  }
  while (have) {
    const int64_t ni = i + 4 * RED_THREADS;
    const bool next = ni + 3 * RED_THREADS < hi;
    Cx<R> vn[4];
    if (next) {
#pragma unroll
      for (int k = 0; k < 4; ++k) vn[k] = __ldcs(p + ni + k * RED_THREADS);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      acc.add_prod(v[k].x, v[k].x);
      acc.add_prod(v[k].y, v[k].y);
    }
    i = ni;
    have = next;
    if (next) {
#pragma unroll
      for (int k = 0; k < 4; ++k) v[k] = vn[k];
    }
  }
  for (; i < hi; i += RED_THREADS) {
    const Cx<R> v = __ldcs(p + i);
    acc.add_prod(v.x, v.x);
    acc.add_prod(v.y, v.y);
  }
  const double2 s = block_sum2(acc.value(), 0.0);
  if (threadIdx.x == 0) {
    if (parts == 1) {
      if (out_f64)
        store_out(static_cast<double*>(out) + row, s.x);
      else
        store_out(static_cast<float*>(out) + row, s.x);
    } else {
      partial[blockIdx.x] = s.x;
    }
  }
}

// Sum `parts` partials (real or complex) of each row in index order.
__global__ void __launch_bounds__(RED_THREADS)
    finalize_kernel(const double* partial, int parts, int complex_parts,
                    int64_t rows, void* out, int out_dtype) {
  const int64_t row = blockIdx.x;
  if (row >= rows) return;
  double x = 0.0, y = 0.0;
  const int w = complex_parts ? 2 : 1;
  for (int j = threadIdx.x; j < parts; j += RED_THREADS) {
    x += partial[(row * parts + j) * w];
    if (complex_parts) y += partial[(row * parts + j) * w + 1];
  }
  const double2 s = block_sum2(x, y);
  if (threadIdx.x == 0) {
    switch (out_dtype) {
      case GBSV_F32: static_cast<float*>(out)[row] = (float)s.x; break;
      case GBSV_F64: static_cast<double*>(out)[row] = s.x; break;
      case GBSV_C64:
        static_cast<float2*>(out)[row] = make_float2((float)s.x, (float)s.y);
        break;
      default:
        static_cast<double2*>(out)[row] = s;
        break;
    }
  }
}

// ---- inner product over broadcast rows --------------------------------
template <typename R>
__global__ void __launch_bounds__(RED_THREADS)
    inner_kernel(const Cx<R>* a, const Cx<R>* b, RowArgs ra, void* out,
                 int out_dtype, double* partial) {
  const int64_t row = blockIdx.x / ra.parts;
  const int part = blockIdx.x % ra.parts;
  int64_t oa, ob;
  row_offsets(ra, row, &oa, &ob);
  const int64_t lo = (int64_t)part * ra.part_len;
  int64_t hi = lo + ra.part_len;
  if (hi > ra.dim) hi = ra.dim;
  Acc<R> x, y;
  auto step = [&](const Cx<R>& u, const Cx<R>& v) {  // += conj(u) * v
    x.add_prod(u.x, v.x);
    x.add_prod(u.y, v.y);
    y.add_prod(u.x, v.y);
    y.add_prod(-u.y, v.x);
  };
  int64_t i = lo + threadIdx.x;
  // four elements of each input per step; the next step's loads are in
  // flight while this step's sums run
  auto load4 = [&](int64_t j, Cx<R>* u, Cx<R>* v) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      u[k] = __ldcs(a + oa + (j + k * RED_THREADS) * ra.ia);
      v[k] = __ldcs(b + ob + (j + k * RED_THREADS) * ra.ib);
    }
  };
  Cx<R> u[4], v[4];
  bool have = i + 3 * RED_THREADS < hi;
  if (have) load4(i, u, v);
  while (have) {
    const int64_t ni = i + 4 * RED_THREADS;
    const bool next = ni + 3 * RED_THREADS < hi;
    Cx<R> un[4], vn[4];
    if (next) load4(ni, un, vn);
#pragma unroll
    for (int k = 0; k < 4; ++k) step(u[k], v[k]);
    i = ni;
    have = next;
    if (next) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        u[k] = un[k];
        v[k] = vn[k];
      }
    }
  }
  for (; i < hi; i += RED_THREADS)
    step(a[oa + i * ra.ia], b[ob + i * ra.ib]);
  const double2 s = block_sum2(x.value(), y.value());
  if (threadIdx.x == 0) {
    if (ra.parts == 1) {
      if (out_dtype == GBSV_C64)
        static_cast<float2*>(out)[row] = make_float2((float)s.x, (float)s.y);
      else
        static_cast<double2*>(out)[row] = s;
    } else {
      partial[2 * blockIdx.x] = s.x;
      partial[2 * blockIdx.x + 1] = s.y;
    }
  }
}

// ---- diagonal expectation over broadcast rows -------------------------
template <typename RD, typename R>
__global__ void __launch_bounds__(RED_THREADS)
    diag_kernel(const RD* d, const Cx<R>* psi, RowArgs ra, void* out,
                int out_dtype, double* partial) {
  const int64_t row = blockIdx.x / ra.parts;
  const int part = blockIdx.x % ra.parts;
  int64_t oa, ob;
  row_offsets(ra, row, &oa, &ob);
  const int64_t lo = (int64_t)part * ra.part_len;
  int64_t hi = lo + ra.part_len;
  if (hi > ra.dim) hi = ra.dim;
  // diag * |psi|^2 in the state's precision (FP64 when either input is)
  using W = typename std::conditional<(sizeof(RD) > sizeof(R)), RD, R>::type;
  Acc<W> acc;
  auto step = [&](const RD dv, const Cx<R>& v) {
    const W w = (W)dv;
    const W x = (W)v.x, y = (W)v.y;
    acc.add_prod(w * x, x);
    acc.add_prod(w * y, y);
  };
  int64_t i = lo + threadIdx.x;
  for (; i + 3 * RED_THREADS < hi; i += 4 * RED_THREADS) {
    RD dv[4];
    Cx<R> v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      dv[k] = __ldcs(d + oa + (i + k * RED_THREADS) * ra.ia);
      v[k] = __ldcs(psi + ob + (i + k * RED_THREADS) * ra.ib);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) step(dv[k], v[k]);
  }
  for (; i < hi; i += RED_THREADS) step(d[oa + i * ra.ia], psi[ob + i * ra.ib]);
  const double2 s = block_sum2(acc.value(), 0.0);
  if (threadIdx.x == 0) {
    if (ra.parts == 1) {
      if (out_dtype == GBSV_F32)
        static_cast<float*>(out)[row] = (float)s.x;
      else
        static_cast<double*>(out)[row] = s.x;
    } else {
      partial[blockIdx.x] = s.x;
    }
  }
}

// ---- abs squared (elementwise) ----------------------------------------
template <typename R>
__global__ void __launch_bounds__(256)
    abs2_kernel(const Cx<R>* psi, R* out, uint64_t count) {
  // four amplitudes per thread and step (several loads in flight)
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < count; i += 4 * stride) {
    Cx<R> v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = __ldcs(psi + i + k * stride);
#pragma unroll
    for (int k = 0; k < 4; ++k)
      __stcs(out + i + k * stride, v[k].x * v[k].x + v[k].y * v[k].y);
  }
  for (; i < count; i += stride) {
    const Cx<R> v = __ldcs(psi + i);
    __stcs(out + i, v.x * v.x + v.y * v.y);
  }
}

// complex64 with 16-byte aligned buffers: four consecutive amplitudes per
// thread and step (two 16-byte loads, one 16-byte store), two steps' loads
// in flight
__global__ void __launch_bounds__(256)
    abs2_c64_vec_kernel(const float4* psi, float4* out, uint64_t quads,
                        const float2* psi_tail, float* out_tail,
                        uint64_t count) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  auto sq = [](const float4& a, const float4& b) {
    return make_float4(a.x * a.x + a.y * a.y, a.z * a.z + a.w * a.w,
                       b.x * b.x + b.y * b.y, b.z * b.z + b.w * b.w);
  };
  for (; j + stride < quads; j += 2 * stride) {
    const float4 a0 = __ldcs(psi + 2 * j), b0 = __ldcs(psi + 2 * j + 1);
    const float4 a1 = __ldcs(psi + 2 * (j + stride));
    const float4 b1 = __ldcs(psi + 2 * (j + stride) + 1);
    __stcs(out + j, sq(a0, b0));
    __stcs(out + j + stride, sq(a1, b1));
  }
  for (; j < quads; j += stride)
    __stcs(out + j, sq(__ldcs(psi + 2 * j), __ldcs(psi + 2 * j + 1)));
  // the last count % 4 amplitudes
  const uint64_t t = quads * 4 + (uint64_t)blockIdx.x * blockDim.x +
                     threadIdx.x;
  if (t < count) {
    const float2 v = psi_tail[t];
    out_tail[t] = v.x * v.x + v.y * v.y;
  }
}

static int fill_rows(RowArgs* ra, const gbsv_bcast_t* bc, int64_t dim,
                     int64_t ia, int64_t ib) {
  if (!bc || bc->ndim < 0 || bc->ndim > GBSV_MAX_DIMS)
    return set_error(GBSV_ERR_INVALID_ARG, "bad broadcast descriptor");
  if (dim < 0 || ia < 0 || ia > 1 || ib < 0 || ib > 1)
    return set_error(GBSV_ERR_INVALID_ARG, "bad inner dimension or stride");
  ra->ndim = bc->ndim;
  int64_t rows = 1;
  for (int d = 0; d < bc->ndim; ++d) {
    if (bc->shape[d] < 0)
      return set_error(GBSV_ERR_INVALID_ARG, "negative extent");
    ra->shape[d] = bc->shape[d];
    ra->sa[d] = bc->stride_a[d];
    ra->sb[d] = bc->stride_b[d];
    rows *= bc->shape[d];
  }
  ra->rows = rows;
  ra->dim = dim;
  ra->ia = ia;
  ra->ib = ib;
  return GBSV_OK;
}

static int check_scratch(const Plan& p, int64_t rows, int complex_parts,
                         void* scratch, size_t bytes) {
  if (p.parts == 1) return GBSV_OK;
  const size_t need = (size_t)rows * p.parts * sizeof(double) *
                      (complex_parts ? 2 : 1);
  if (!scratch || bytes < need)
    return set_error(GBSV_ERR_SCRATCH,
                     "reduction needs %zu scratch bytes, got %zu", need,
                     scratch ? bytes : (size_t)0);
  if ((uintptr_t)scratch % 16)
    return set_error(GBSV_ERR_SCRATCH, "scratch must be 16-byte aligned");
  return GBSV_OK;
}


// ---- renormalisation checkpoint ---------------------------------------
// psi[row] *= sqrt(target[row] / norm[row]); a block covers `per_block`
// amplitudes of one row and computes the row's factor once (FP64).
template <typename R>
__global__ void __launch_bounds__(RED_THREADS)
    rescale_kernel(Cx<R>* psi, int64_t dim, int64_t per_block,
                   const double* target, const double* norm) {
  const int64_t blocks_per_row = dim / per_block;
  const int64_t row = blockIdx.x / blocks_per_row;
  const int64_t lo = row * dim + (blockIdx.x % blocks_per_row) * per_block;
  __shared__ R fac;
  if (threadIdx.x == 0) {
    const double n = norm[row];
    fac = (R)(n > 0.0 ? sqrt(target[row] / n) : 1.0);
  }
  __syncthreads();
  const R f = fac;
  for (int64_t i = lo + threadIdx.x; i < lo + per_block; i += RED_THREADS) {
    Cx<R> v = psi[i];
    v.x *= f;
    v.y *= f;
    psi[i] = v;
  }
}

static int finalize(const Plan& p, double* partial, int complex_parts,
                    int64_t rows, void* out, int out_dtype, cudaStream_t st) {
  if (p.parts == 1) return GBSV_OK;
  finalize_kernel<<<(unsigned)rows, RED_THREADS, 0, st>>>(
      partial, p.parts, complex_parts, rows, out, out_dtype);
  return after_launch("finalize_kernel");
}

static int check_grid(const Plan& p, int64_t rows) {
  if ((uint64_t)rows * (uint64_t)p.parts > 0x7fffffffull)
    return set_error(GBSV_ERR_UNSUPPORTED, "too many rows (%lld)",
                     (long long)rows);
  return GBSV_OK;
}

}  // namespace gbsv

using namespace gbsv;

extern "C" size_t gbsv_reduce_scratch_bytes(int64_t num_rows, int64_t dim) {
  const Plan p = make_plan(num_rows, dim);
  if (p.parts == 1) return 0;
  return (size_t)num_rows * p.parts * 2 * sizeof(double);
}

extern "C" int gbsv_norm_squared(const void* state, int dtype,
                                 int64_t num_rows, int64_t dim, void* out,
                                 int out_dtype, void* scratch,
                                 size_t scratch_bytes, void* stream) {
  if (dtype != GBSV_C64 && dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "state must be complex");
  if (out_dtype != GBSV_F32 && out_dtype != GBSV_F64)
    return set_error(GBSV_ERR_INVALID_ARG, "output must be float32/float64");
  if (num_rows < 0 || dim < 0)
    return set_error(GBSV_ERR_INVALID_ARG, "negative size");
  if (num_rows == 0) return GBSV_OK;
  if (!out || (dim > 0 && !state))
    return set_error(GBSV_ERR_INVALID_ARG, "null pointer");
  // two waves of the read-only kernel (measured 2% faster on a 30-qubit
  // row than one wave)
  const Plan p = make_plan(num_rows, dim);
  int rc = check_scratch(p, num_rows, 0, scratch, scratch_bytes);
  if (!rc) rc = check_grid(p, num_rows);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned blocks = (unsigned)(num_rows * p.parts);
  double* partial = static_cast<double*>(scratch);
  if (dtype == GBSV_C64)
    norm2_kernel<float><<<blocks, RED_THREADS, 0, st>>>(
        static_cast<const float2*>(state), dim, p.parts, p.part_len, out,
        out_dtype == GBSV_F64, partial);
  else
    norm2_kernel<double><<<blocks, RED_THREADS, 0, st>>>(
        static_cast<const double2*>(state), dim, p.parts, p.part_len, out,
        out_dtype == GBSV_F64, partial);
  rc = after_launch("norm2_kernel");
  if (rc) return rc;
  return finalize(p, partial, 0, num_rows, out, out_dtype, st);
}

extern "C" int gbsv_renormalize(void* state, int dtype, int64_t num_rows,
                                int64_t dim, const void* target_norms,
                                void* norms_out, void* scratch,
                                size_t scratch_bytes, void* stream) {
  if (dtype != GBSV_C64 && dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "state must be complex");
  if (num_rows < 0 || dim < 0)
    return set_error(GBSV_ERR_INVALID_ARG, "negative size");
  if (num_rows == 0 || dim == 0) return GBSV_OK;
  if (dim & (dim - 1))
    return set_error(GBSV_ERR_INVALID_ARG, "dim must be a power of two");
  if (!state || !target_norms || !norms_out)
    return set_error(GBSV_ERR_INVALID_ARG, "null pointer");
  int rc = gbsv_norm_squared(state, dtype, num_rows, dim, norms_out,
                             GBSV_F64, scratch, scratch_bytes, stream);
  if (rc) return rc;
  const int64_t per_block = dim < 8192 ? dim : 8192;
  const uint64_t blocks = (uint64_t)num_rows * (uint64_t)(dim / per_block);
  if (blocks > 0x7fffffffull)
    return set_error(GBSV_ERR_UNSUPPORTED, "too many rows (%lld)",
                     (long long)num_rows);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == GBSV_C64)
    rescale_kernel<float><<<(unsigned)blocks, RED_THREADS, 0, st>>>(
        static_cast<float2*>(state), dim, per_block,
        static_cast<const double*>(target_norms),
        static_cast<const double*>(norms_out));
  else
    rescale_kernel<double><<<(unsigned)blocks, RED_THREADS, 0, st>>>(
        static_cast<double2*>(state), dim, per_block,
        static_cast<const double*>(target_norms),
        static_cast<const double*>(norms_out));
  return after_launch("rescale_kernel");
}

extern "C" int gbsv_abs_squared(const void* state, int dtype, int64_t count,
                                void* out, void* stream) {
  if (dtype != GBSV_C64 && dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "state must be complex");
  if (count < 0) return set_error(GBSV_ERR_INVALID_ARG, "negative size");
  if (count == 0) return GBSV_OK;
  if (!state || !out) return set_error(GBSV_ERR_INVALID_ARG, "null pointer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  uint64_t blocks = ((uint64_t)count + 255) / 256;
  const uint64_t cap = (uint64_t)sm_count() * 32;
  if (blocks > cap) blocks = cap;
  if (dtype == GBSV_C64 && (uintptr_t)state % 16 == 0 &&
      (uintptr_t)out % 16 == 0) {
    const uint64_t quads = (uint64_t)count / 4;
    uint64_t vb = (quads + 255) / 256;
    if (vb > cap) vb = cap;
    if (vb < 1) vb = 1;
    abs2_c64_vec_kernel<<<(unsigned)vb, 256, 0, st>>>(
        static_cast<const float4*>(state), static_cast<float4*>(out), quads,
        static_cast<const float2*>(state), static_cast<float*>(out), count);
    return after_launch("abs2_c64_vec_kernel");
  }
  if (dtype == GBSV_C64)
    abs2_kernel<float><<<(unsigned)blocks, 256, 0, st>>>(
        static_cast<const float2*>(state), static_cast<float*>(out), count);
  else
    abs2_kernel<double><<<(unsigned)blocks, 256, 0, st>>>(
        static_cast<const double2*>(state), static_cast<double*>(out), count);
  return after_launch("abs2_kernel");
}

extern "C" int gbsv_inner_product(const void* a, const void* b, int dtype,
                                  const gbsv_bcast_t* bc, int64_t dim,
                                  int64_t inner_stride_a,
                                  int64_t inner_stride_b, void* out,
                                  int out_dtype, void* scratch,
                                  size_t scratch_bytes, void* stream) {
  if (dtype != GBSV_C64 && dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "states must be complex");
  if (out_dtype != GBSV_C64 && out_dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "output must be complex");
  RowArgs ra{};
  int rc = fill_rows(&ra, bc, dim, inner_stride_a, inner_stride_b);
  if (rc) return rc;
  if (ra.rows == 0) return GBSV_OK;
  if (!out || (dim > 0 && (!a || !b)))
    return set_error(GBSV_ERR_INVALID_ARG, "null pointer");
  static const int nb_f = resident_blocks(inner_kernel<float>);
  static const int nb_d = resident_blocks(inner_kernel<double>);
  const Plan p = make_plan(ra.rows, dim, dtype == GBSV_C64 ? nb_f : nb_d);
  ra.parts = p.parts;
  ra.part_len = p.part_len;
  rc = check_scratch(p, ra.rows, 1, scratch, scratch_bytes);
  if (!rc) rc = check_grid(p, ra.rows);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned blocks = (unsigned)(ra.rows * p.parts);
  double* partial = static_cast<double*>(scratch);
  if (dtype == GBSV_C64)
    inner_kernel<float><<<blocks, RED_THREADS, 0, st>>>(
        static_cast<const float2*>(a), static_cast<const float2*>(b), ra, out,
        out_dtype, partial);
  else
    inner_kernel<double><<<blocks, RED_THREADS, 0, st>>>(
        static_cast<const double2*>(a), static_cast<const double2*>(b), ra,
        out, out_dtype, partial);
  rc = after_launch("inner_kernel");
  if (rc) return rc;
  return finalize(p, partial, 1, ra.rows, out, out_dtype, st);
}

extern "C" int gbsv_diag_expectation(const void* diag, int diag_dtype,
                                     const void* state, int state_dtype,
                                     const gbsv_bcast_t* bc, int64_t dim,
                                     int64_t inner_stride_diag,
                                     int64_t inner_stride_state, void* out,
                                     int out_dtype, void* scratch,
                                     size_t scratch_bytes, void* stream) {
  if (state_dtype != GBSV_C64 && state_dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "state must be complex");
  if (diag_dtype != GBSV_F32 && diag_dtype != GBSV_F64)
    return set_error(GBSV_ERR_INVALID_ARG, "diagonal must be float32/float64");
  if (out_dtype != GBSV_F32 && out_dtype != GBSV_F64)
    return set_error(GBSV_ERR_INVALID_ARG, "output must be float32/float64");
  RowArgs ra{};
  int rc = fill_rows(&ra, bc, dim, inner_stride_diag, inner_stride_state);
  if (rc) return rc;
  if (ra.rows == 0) return GBSV_OK;
  if (!out || (dim > 0 && (!diag || !state)))
    return set_error(GBSV_ERR_INVALID_ARG, "null pointer");
  const Plan p = make_plan(ra.rows, dim);
  ra.parts = p.parts;
  ra.part_len = p.part_len;
  rc = check_scratch(p, ra.rows, 0, scratch, scratch_bytes);
  if (!rc) rc = check_grid(p, ra.rows);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned blocks = (unsigned)(ra.rows * p.parts);
  double* partial = static_cast<double*>(scratch);
  const bool d64 = diag_dtype == GBSV_F64, s64 = state_dtype == GBSV_C128;
  if (!d64 && !s64)
    diag_kernel<float, float><<<blocks, RED_THREADS, 0, st>>>(
        static_cast<const float*>(diag), static_cast<const float2*>(state),
        ra, out, out_dtype, partial);
  else if (d64 && !s64)
    diag_kernel<double, float><<<blocks, RED_THREADS, 0, st>>>(
        static_cast<const double*>(diag), static_cast<const float2*>(state),
        ra, out, out_dtype, partial);
  else if (!d64 && s64)
    diag_kernel<float, double><<<blocks, RED_THREADS, 0, st>>>(
        static_cast<const float*>(diag), static_cast<const double2*>(state),
        ra, out, out_dtype, partial);
  else
    diag_kernel<double, double><<<blocks, RED_THREADS, 0, st>>>(
        static_cast<const double*>(diag), static_cast<const double2*>(state),
        ra, out, out_dtype, partial);
  rc = after_launch("diag_kernel");
  if (rc) return rc;
  return finalize(p, partial, 0, ra.rows, out, out_dtype, st);
}

// ---------------------------------------------------------------------------
// Allocation-free norm_squared.
//
// Some callers cannot call cudaMalloc: a host program that reaches this
// library through a thin FFI and only holds buffers another runtime handed
// it has no device allocator to call, and a latency-critical loop must not
// call it because cudaMalloc can synchronize the device and stall work
// queued on other streams.  gbsv_norm_squared_noalloc serves them: it takes
// the same inputs and outputs as gbsv_norm_squared but keeps its FP64
// partial sums in the file-scope device array below instead of caller
// scratch.
//
// The array is NOALLOC_SCRATCH_BYTES (64 KiB) and lives on every GPU that
// loads this library until the process exits.  Requests whose partials
// would not fit are rejected with GBSV_ERR_UNSUPPORTED.  Every call shares
// the array and it keeps the last call's contents; nothing in it has to
// start at zero, because each call writes every partial it later reads.
// Calls whose kernels overlap on the GPU (for instance on two streams) race
// on the array.
namespace gbsv {

constexpr size_t NOALLOC_SCRATCH_BYTES = 64 * 1024;
static __device__ __align__(256) double
    g_noalloc_partials[NOALLOC_SCRATCH_BYTES / sizeof(double)];

// Device address of g_noalloc_partials in the current device's context.
// Host code may not use the symbol's host-side name as a device pointer, so
// the address is looked up on every call: the lookup allocates nothing and
// does not synchronize, and a cached address would go stale when the
// context is torn down and recreated (cudaDeviceReset).  Under lazy module
// loading the first lookup on a device loads this module, which can
// synchronize; a warm-up call before a latency-critical loop or a stream
// capture moves that cost out of the loop.
static int noalloc_scratch(double** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
  if (e != cudaSuccess || !p)
    return set_error(GBSV_ERR_CUDA, "cudaGetSymbolAddress: %s",
                     cudaGetErrorString(e));
  *out = static_cast<double*>(p);
  return GBSV_OK;
}

}  // namespace gbsv

extern "C" int gbsv_norm_squared_noalloc(const void* state, int dtype,
                                         int64_t num_rows, int64_t dim,
                                         void* out, int out_dtype,
                                         void* stream) {
  if (dtype != GBSV_C64 && dtype != GBSV_C128)
    return set_error(GBSV_ERR_INVALID_ARG, "state must be complex");
  if (out_dtype != GBSV_F32 && out_dtype != GBSV_F64)
    return set_error(GBSV_ERR_INVALID_ARG, "output must be float32/float64");
  if (num_rows < 0 || dim < 0)
    return set_error(GBSV_ERR_INVALID_ARG, "negative size");
  if (num_rows == 0) return GBSV_OK;
  if (!out || (dim > 0 && !state))
    return set_error(GBSV_ERR_INVALID_ARG, "null pointer");
  const Plan p = make_plan(num_rows, dim);
  int rc = check_grid(p, num_rows);
  if (rc) return rc;
  double* partial = nullptr;
  if (p.parts > 1) {
    const size_t need = (size_t)num_rows * p.parts * sizeof(double);
    if (need > NOALLOC_SCRATCH_BYTES)
      return set_error(GBSV_ERR_UNSUPPORTED,
                       "norm_squared_noalloc: %lld rows of %lld amplitudes "
                       "need %zu scratch bytes, more than its fixed %zu",
                       (long long)num_rows, (long long)dim, need,
                       NOALLOC_SCRATCH_BYTES);
    rc = noalloc_scratch(&partial);
    if (rc) return rc;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned blocks = (unsigned)(num_rows * p.parts);
  if (dtype == GBSV_C64)
    norm2_kernel<float><<<blocks, RED_THREADS, 0, st>>>(
        static_cast<const float2*>(state), dim, p.parts, p.part_len, out,
        out_dtype == GBSV_F64, partial);
  else
    norm2_kernel<double><<<blocks, RED_THREADS, 0, st>>>(
        static_cast<const double2*>(state), dim, p.parts, p.part_len, out,
        out_dtype == GBSV_F64, partial);
  rc = after_launch("norm2_kernel");
  if (rc) return rc;
  return finalize(p, partial, 0, num_rows, out, out_dtype, st);
}
