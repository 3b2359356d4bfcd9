// Tensor-core fused stages (complex64).
//
// A stage owns 12 "tile bits" of the amplitude index (the lowest c bits and
// 12 - c higher ones, as in the register stages of fused.cu), so every tile
// is 4096 amplitudes (32 KiB) and the stage costs one read and one write of
// the state.  The host planner groups the stage's gates into "blocks": the
// product of a run of gates on at most 5 tile bits is one 32x32 complex
// matrix U, multiplied into the tile on the tensor cores.
//
// Per block, the tile is viewed as a 32 x 128 matrix: row index = the 5
// block bits, column = the other 7 tile bits.  Thread r (one warpgroup,
// r = 0..127) gathers column r from shared memory (32 amplitudes), writes
// it to tensor memory as row r of the MMA's A operand (K = 64 reals), and
// tcgen05.mma multiplies it by the real form of U^T (64 x 64, B operand in
// shared memory): D = A * B, M = 128 columns, N = 64 output reals.  The
// result comes back with tcgen05.ld into the same thread, which scatters it
// into the tile for the next block.
//
// Precision (kind::f16, FP32 accumulation).  GB300's tensor cores truncate
// the FP32 accumulation (measured: sums round toward zero), so a plain
// fp16 split would shrink every amplitude a little per block.  Instead the
// split makes the dominant product exact:
//   * each thread scales its 64 reals by a power of two s so the largest is
//     below 2^10, and splits x*s = hi + lo * 2^-11 with hi an integer
//     (|hi| <= 1024, exact in fp16) and lo rounded to fp16;
//   * the host splits 1024 * B the same way into an integer matrix Bh and
//     an fp16 residual Bl (|1024 * B - Bh| <= 1/2, stored times 2^11);
//   * D1 = hi * Bh is a sum of integer products bounded by
//     1024 * (1024 * 8 + 32) < 2^24 (a unitary's real-form columns have
//     L1 norm <= 8), so every partial sum is an exact FP32 integer and the
//     truncating accumulator makes no error;
//   * D2 = lo * Bh + hi * Bl (three-product split, Ootomo & Yokota 2022)
//     carries the correction at 2^-11 of D1's scale, where truncation
//     costs about 2^-35 relative;
//   * y = (D1 + D2 * 2^-11) / (1024 s), exact power-of-two scalings.
// The representation error is about 2^-22 of each column's largest
// amplitude per block.
//
// Diagonal gates whose bits are all outside a block's bits (thread bits,
// or positions outside the tile) commute with the block: the planner
// attaches them to the block as "post-diagonals", folded into a per-thread
// factor applied when the block's result is written back.
//
// Pipeline (two CTAs of 128 threads per SM, 97 KiB of shared memory and
// 256 tensor-memory columns each): the next tile streams in by 16-byte
// cp.async while the current tile's blocks run; block matrices (16 KiB
// images: fp16 Bh then Bl, in the canonical K-major no-swizzle layout) are
// resident when a stage has at most two blocks and otherwise stream through
// two buffers by cp.async.bulk, one block ahead.  While one CTA waits for
// its MMAs the other gathers, splits or scatters.  Every wait on an
// mbarrier is bounded; a wait that runs out records an error (read with
// gbsv_tc_status), drains what is in flight and ends the CTA.
#include "common.cuh"

#include <cuda_fp16.h>

#include <algorithm>

namespace gbsv {

constexpr int TC_M = 12;             // tile bits
constexpr int TC_RB = 5;             // block (register) bits
constexpr int TC_TB = TC_M - TC_RB;  // thread bits
constexpr int TC_THREADS = 1 << TC_TB;
constexpr int TC_TILE = 1 << TC_M;
constexpr int TC_MAX_BLOCKS = 64;
constexpr int TC_IMG_BYTES = 16384;
constexpr int TC_IMG_HALF = 8192;
constexpr int TC_SMEM_BYTES = 2 * TC_TILE * 8 + 2 * TC_IMG_BYTES + 1024;

// Block record (gbsv_tc_block_t).  Shared-memory offsets are in amplitudes
// after the tile swizzle; the swizzle is linear over GF(2), so amplitude
// (thread bits of r) | (register bits of i) sits at
// XOR(tspo[j] : bit j of r) ^ XOR(rspo[k] : bit k of i).
struct TcBlock {
  int32_t rspo[TC_RB];  // register-index bit k -> swizzled offset
  int32_t tspo[TC_TB];  // thread-index bit j -> swizzled offset
  int32_t mat;          // image index (16 KiB each)
  int32_t first_diag;   // post-diagonals [first_diag, first_diag + num_diag)
  int32_t num_diag;
  int32_t flags;        // TC_PAIRS: register bit 0 is tile bit 0
};
static_assert(sizeof(TcBlock) == 64, "gbsv_tc_block_t is 64 bytes");
constexpr int TC_PAIRS = 1;

// Post-diagonal: a 1- or 2-qubit diagonal applied after its block.  Each
// qubit is encoded as a register bit (0..4), a thread-index bit (5 + j) or
// -1 - its position outside the tile; the first qubit is the index MSB.
struct TcDiag {
  int32_t nq;
  int32_t enc[2];
  int32_t reg;  // nonzero when a qubit is a register bit
  float2 d[4];
};
static_assert(sizeof(TcDiag) == 48, "gbsv_tc_diag_t is 48 bytes");

struct TcArgs {
  int n, c, num_blocks;
  int64_t num_states;
  int64_t in_stride;       // amplitudes between input states (0 = bcast)
  int hpos[TC_M];          // global position of tile bit c + j
  int spos[TC_M];          // all tile positions, ascending
  const TcBlock* blocks;
  const TcDiag* diags;
  const unsigned char* images;
};

static __device__ int g_tc_status;  // nonzero after a bounded wait ran out

// Tile swizzle: amplitude bits 1-3 ^= bits 4-6 ^ 7-9 ^ 10-12.  Bit 0 stays,
// so 16-byte pieces (two amplitudes) stay whole for the copies, and every
// tile bit >= 1 has a non-zero image in the bank bits.
__device__ __forceinline__ int tc_swz(int l) {
  return l ^ ((((l >> 4) ^ (l >> 7) ^ (l >> 10)) & 7) << 1);
}

__device__ __forceinline__ uint32_t tc_smem(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Wait for phase `parity` of an mbarrier, for at most about 2^31 cycles.
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  while (true) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > (1ll << 31)) return false;
  }
}

__device__ __forceinline__ void tc_load_image(uint32_t dst, const void* src,
                                              uint32_t bar) {
  asm volatile(
      "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
      "r"(TC_IMG_BYTES)
      : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(TC_IMG_BYTES), "r"(bar)
      : "memory");
}

// Shared-memory matrix descriptor: K-major, no swizzle; core matrices of
// 8 rows x 16 bytes, K-adjacent ones 128 bytes apart (leading byte offset),
// 8-row groups 1024 bytes apart (stride byte offset).
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) |
         ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46);
}

// D (f32) = A (f16, tensor memory) * B (f16, shared memory), M = 128,
// N = 64, K = 16; accumulate into D when acc != 0.
__device__ __forceinline__ void tc_mma(uint32_t d, uint32_t a, uint64_t b,
                                       uint32_t acc) {
  constexpr uint32_t idesc = (1u << 4)  // D f32; A, B f16; both K-major
                             | ((uint32_t)(64 >> 3) << 17) |
                             ((uint32_t)(128 >> 4) << 24);
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(
          d),
      "r"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

#define TC_R32(r)                                                            \
  "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]),          \
      "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]),    \
      "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]),            \
      "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]),            \
      "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]),            \
      "r"(r[27]), "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
#define TC_W32(r)                                                            \
  "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),    \
      "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]),           \
      "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),       \
      "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),       \
      "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),       \
      "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),       \
      "=r"(r[31])
#define TC_LIST32                                                            \
  "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20," \
  "%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32}"
#define TC_LIST32_OUT                                                        \
  "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"  \
  "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}"

// 32 consecutive 32-bit columns of this thread's lane.
__device__ __forceinline__ void tc_st32(uint32_t taddr, const uint32_t* r) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], " TC_LIST32
               ";" ::"r"(taddr),
               TC_R32(r)
               : "memory");
}
__device__ __forceinline__ void tc_ld32(uint32_t taddr, uint32_t* r) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 " TC_LIST32_OUT
               ", [%32];"
               : TC_W32(r)
               : "r"(taddr)
               : "memory");
}

__device__ __forceinline__ uint32_t tc_pack(float lo_k, float hi_k) {
  const __half2 h = __floats2half2_rn(lo_k, hi_k);
  return *reinterpret_cast<const uint32_t*>(&h);
}

__device__ __forceinline__ uint64_t tc_tile_base(const TcArgs& a,
                                                 uint64_t t) {
  uint64_t base = t;
#pragma unroll
  for (int j = 0; j < TC_M; ++j) base = insert_zero(base, a.spos[j]);
  return base;
}

// Global offset of tile amplitude l (bits < c contiguous, bit c + j at
// position hpos[j]).
__device__ __forceinline__ uint64_t tc_tile_offset(const TcArgs& a, int l) {
  uint64_t off = (uint64_t)(l & ((1 << a.c) - 1));
  const int r = l >> a.c;
  for (int j = 0; j < TC_M - a.c; ++j)
    if ((r >> j) & 1) off += uint64_t(1) << a.hpos[j];
  return off;
}

__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_stage_kernel(const float2* in, float2* out, TcArgs a) {
  extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
  // 1024-byte alignment of the dynamic area is not guaranteed: round up
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
  float2* const tiles = reinterpret_cast<float2*>(smem);
  unsigned char* const imgs = smem + 2 * TC_TILE * 8;
  __shared__ TcBlock sblk[TC_MAX_BLOCKS];
  __shared__ uint64_t offh[16];
  __shared__ __align__(8) uint64_t mbar_img[2];
  __shared__ __align__(8) uint64_t mbar_mma;
  __shared__ uint32_t s_tmem;

  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int nb = a.num_blocks;
  const uint64_t tps = uint64_t(1) << (a.n - TC_M);
  const uint64_t num_tiles = (uint64_t)a.num_states * tps;
  const uint64_t t0 = (uint64_t)blockIdx.x * num_tiles / gridDim.x;
  const uint64_t t1 = (uint64_t)(blockIdx.x + 1) * num_tiles / gridDim.x;
  if (t0 >= t1) return;

  if (warp == 0) {
    asm volatile(
        "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::
            "r"(tc_smem(&s_tmem))
        : "memory");
    asm volatile(
        "tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::
            : "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(
        tc_smem(&mbar_img[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(
        tc_smem(&mbar_img[1])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(
        tc_smem(&mbar_mma)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int i = tid; i < nb * 16; i += TC_THREADS)
    reinterpret_cast<int32_t*>(sblk)[i] =
        reinterpret_cast<const int32_t*>(a.blocks)[i];
  if (tid < 16) offh[tid] = tc_tile_offset(a, 256 * tid);
  const uint64_t offt = tc_tile_offset(a, 2 * tid);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = s_tmem;
  const uint32_t lane = (uint32_t)(warp * 32) << 16;
  const uint32_t tA_hi = tmem, tA_lo = tmem + 32, tD1 = tmem + 64,
                 tD2 = tmem + 128;

  // block-matrix images: resident (nb <= 2) or streamed one exec ahead
  const bool resident = nb <= 2;
  const uint64_t total_exec = (t1 - t0) * (uint64_t)nb;
  uint32_t img_phase = 0;   // bit b: parity of the next load into buffer b
  int img_pending = 0;      // loads issued and not yet waited (tid 0)
  if (tid == 0) {
    const int first = resident ? nb : (total_exec < 2 ? (int)total_exec : 2);
    for (int e = 0; e < first; ++e) {
      tc_load_image(tc_smem(imgs + e * TC_IMG_BYTES),
                    a.images + (size_t)sblk[e % nb].mat * TC_IMG_BYTES,
                    tc_smem(&mbar_img[e]));
      img_pending |= 1 << e;
    }
  }

  auto prefetch = [&](uint64_t t, float2* S) {
    const uint64_t s = t / tps;
    const float2* src =
        in + (int64_t)s * a.in_stride + tc_tile_base(a, t % tps) + offt;
#pragma unroll
    for (int it = 0; it < 16; ++it) {
      const int l = 2 * (tid + TC_THREADS * it);
      cp_async16<float>(&S[tc_swz(l)], src + offh[it]);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };

  prefetch(t0, tiles);
  uint32_t mma_phase = 0;
  uint64_t e = 0;  // block executions so far
  bool bad = false;
  bool mma_late = false;  // an MMA wait ran out
  for (uint64_t t = t0; t < t1 && !bad; ++t) {
    float2* const S = tiles + (int)((t - t0) & 1) * TC_TILE;
    cp_async_wait_all();
    __syncthreads();
    if (t + 1 < t1) prefetch(t + 1, tiles + (int)((t + 1 - t0) & 1) * TC_TILE);
    const uint64_t s = t / tps;
    const uint64_t base = tc_tile_base(a, t % tps);

    for (int bi = 0; bi < nb; ++bi, ++e) {
      const TcBlock& B = sblk[bi];
      int sb = 0;
#pragma unroll
      for (int j = 0; j < TC_TB; ++j)
        if ((tid >> j) & 1) sb ^= B.tspo[j];
      int rs[TC_RB];
#pragma unroll
      for (int k = 0; k < TC_RB; ++k) rs[k] = B.rspo[k];
      auto roff = [&](int i) {
        int x = sb;
#pragma unroll
        for (int k = 0; k < TC_RB; ++k)
          if ((i >> k) & 1) x ^= rs[k];
        return x;
      };
      const bool pairs = B.flags & TC_PAIRS;

      // gather column tid
      float2 v[32];
      if (pairs) {
#pragma unroll
        for (int i = 0; i < 32; i += 2) {
          const float4 w = *reinterpret_cast<const float4*>(&S[roff(i)]);
          v[i] = make_float2(w.x, w.y);
          v[i + 1] = make_float2(w.z, w.w);
        }
      } else {
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = S[roff(i)];
      }

      // power-of-two scaling and the exact-integer / residual split
      uint32_t emax = 0;
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        emax = max(emax, __float_as_uint(v[i].x) & 0x7f800000u);
        emax = max(emax, __float_as_uint(v[i].y) & 0x7f800000u);
      }
      const int E = max((int)(emax >> 23), 20);
      const float sc = __uint_as_float((uint32_t)(263 - E) << 23);  // 2^(136-E)
      const float sc2 = sc * 2048.f;
      const float inv = __uint_as_float((uint32_t)(E - 19) << 23);  // 2^(E-146)
      {
        uint32_t hi[32], lo[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const float hr = rintf(v[i].x * sc), hm = rintf(v[i].y * sc);
          const float lr = fmaf(v[i].x, sc2, -2048.f * hr);
          const float lm = fmaf(v[i].y, sc2, -2048.f * hm);
          hi[i] = tc_pack(hr, hm);
          lo[i] = tc_pack(lr, lm);
        }
        tc_st32(tA_hi + lane, hi);
        tc_st32(tA_lo + lane, lo);
      }
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();

      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int buf = resident ? bi : (int)(e & 1);
        bool ok = true;
        if ((img_pending >> buf) & 1) {
          ok = tc_wait(tc_smem(&mbar_img[buf]), (img_phase >> buf) & 1);
          img_pending &= ~(1 << buf);
          img_phase ^= 1u << buf;
        }
        if (ok) {
          const uint32_t bh = tc_smem(imgs + buf * TC_IMG_BYTES);
          const uint32_t bl = bh + TC_IMG_HALF;
#pragma unroll
          for (int j = 0; j < 4; ++j)
            tc_mma(tD1, tA_hi + 8 * j, tc_desc(bh + 256 * j), j > 0);
#pragma unroll
          for (int j = 0; j < 4; ++j)
            tc_mma(tD2, tA_lo + 8 * j, tc_desc(bh + 256 * j), j > 0);
#pragma unroll
          for (int j = 0; j < 4; ++j)
            tc_mma(tD2, tA_hi + 8 * j, tc_desc(bl + 256 * j), 1);
        } else {
          atomicOr(&g_tc_status, 1);
        }
        // commit even after a failed wait: it then arrives at once
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::"
            "cluster.b64 [%0];" ::"r"(tc_smem(&mbar_mma))
            : "memory");
        bad |= !ok;
      }
      if (!tc_wait(tc_smem(&mbar_mma), mma_phase)) {
        bad = true;
        mma_late = true;
        atomicOr(&g_tc_status, 2);
      }
      mma_phase ^= 1;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // the image buffer of this execution is free: stream the one after
      // next into it
      if (tid == 0 && !resident && !bad && e + 2 < total_exec) {
        const int buf = (int)(e & 1);
        tc_load_image(tc_smem(imgs + buf * TC_IMG_BYTES),
                      a.images +
                          (size_t)sblk[(int)((e + 2) % nb)].mat * TC_IMG_BYTES,
                      tc_smem(&mbar_img[buf]));
        img_pending |= 1 << buf;
      }

      // per-thread factor of the post-diagonals on thread / outside bits
      float2 f = make_float2(inv, 0.f);
      bool regdiag = false;
      for (int q = B.first_diag; q < B.first_diag + B.num_diag; ++q) {
        const TcDiag& dg = a.diags[q];
        if (dg.reg) {
          regdiag = true;
          continue;
        }
        int idx = 0;
        for (int u = 0; u < dg.nq; ++u) {
          const int en = dg.enc[u];
          const int bit = en >= TC_RB ? (tid >> (en - TC_RB)) & 1
                                      : (int)((base >> (-1 - en)) & 1);
          idx = (idx << 1) | bit;
        }
        f = cmul(f, dg.d[idx]);
      }
      // read back D1, D2 and combine
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        uint32_t d1[32], d2[32];
        tc_ld32(tD1 + lane + 32 * h, d1);
        tc_ld32(tD2 + lane + 32 * h, d2);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const float re = fmaf(__uint_as_float(d2[2 * j]), 1.f / 2048.f,
                                __uint_as_float(d1[2 * j]));
          const float im = fmaf(__uint_as_float(d2[2 * j + 1]), 1.f / 2048.f,
                                __uint_as_float(d1[2 * j + 1]));
          v[16 * h + j] = cmul(f, make_float2(re, im));
        }
      }
      if (regdiag) {
        for (int q = B.first_diag; q < B.first_diag + B.num_diag; ++q) {
          const TcDiag& dg = a.diags[q];
          if (!dg.reg) continue;
#pragma unroll
          for (int i = 0; i < 32; ++i) {
            int idx = 0;
            for (int u = 0; u < dg.nq; ++u) {
              const int en = dg.enc[u];
              const int bit = en < 0 ? (int)((base >> (-1 - en)) & 1)
                              : en < TC_RB ? (i >> en) & 1
                                           : (tid >> (en - TC_RB)) & 1;
              idx = (idx << 1) | bit;
            }
            v[i] = cmul(dg.d[idx], v[i]);
          }
        }
      }
      // scatter back (the same addresses the gather read)
      if (pairs) {
#pragma unroll
        for (int i = 0; i < 32; i += 2)
          *reinterpret_cast<float4*>(&S[roff(i)]) =
              make_float4(v[i].x, v[i].y, v[i + 1].x, v[i + 1].y);
      } else {
#pragma unroll
        for (int i = 0; i < 32; ++i) S[roff(i)] = v[i];
      }
      bad = __syncthreads_or(bad);
      if (bad) break;
    }
    if (bad) break;

    float2* dst = out + (s << a.n) + base + offt;
#pragma unroll
    for (int it = 0; it < 16; ++it) {
      const int l = 2 * (tid + TC_THREADS * it);
      const float4 w = *reinterpret_cast<const float4*>(&S[tc_swz(l)]);
      __stcs(reinterpret_cast<float4*>(dst + offh[it]), w);
    }
  }
  // drain: tile copies, image loads and MMAs in flight
  cp_async_wait_all();
  if (mma_late && !tc_wait(tc_smem(&mbar_mma), mma_phase ^ 1))
    atomicOr(&g_tc_status, 8);
  if (tid == 0) {
    for (int b = 0; b < 2; ++b)
      if ((img_pending >> b) & 1)
        if (!tc_wait(tc_smem(&mbar_img[b]), (img_phase >> b) & 1))
          atomicOr(&g_tc_status, 4);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile(
        "tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem)
        : "memory");
  }
}

}  // namespace gbsv

using gbsv::set_error;

extern "C" int gbsv_run_stage_tc(const void* state_in, void* state_out,
                                 int dtype, int n, int64_t num_states,
                                 int64_t in_stride, int m, int c,
                                 const int32_t* positions,
                                 const void* blocks, int num_blocks,
                                 const void* diags, const void* images,
                                 void* stream) {
  using namespace gbsv;
  if (dtype != GBSV_C64)
    return set_error(GBSV_ERR_UNSUPPORTED,
                     "tensor-core stages are complex64 only");
  if (m != TC_M)
    return set_error(GBSV_ERR_INVALID_ARG, "tensor-core stages use %d tile "
                     "bits, got %d", TC_M, m);
  if (n < TC_M || n > 40)
    return set_error(GBSV_ERR_INVALID_ARG, "need %d..40 qubits, got %d", TC_M,
                     n);
  if (num_blocks < 1 || num_blocks > TC_MAX_BLOCKS)
    return set_error(GBSV_ERR_INVALID_ARG, "num_blocks %d not in 1..%d",
                     num_blocks, TC_MAX_BLOCKS);
  if (c < 1 || c > TC_M)
    return set_error(GBSV_ERR_INVALID_ARG, "contiguous bits %d not in 1..%d",
                     c, TC_M);
  if (num_states < 0) return set_error(GBSV_ERR_INVALID_ARG, "num_states < 0");
  if (num_states == 0) return GBSV_OK;
  if (!state_in || !state_out || !positions || !blocks || !images)
    return set_error(GBSV_ERR_INVALID_ARG, "null pointer");
  if ((reinterpret_cast<uintptr_t>(state_in) |
       reinterpret_cast<uintptr_t>(state_out) |
       reinterpret_cast<uintptr_t>(images)) & 15)
    return set_error(GBSV_ERR_INVALID_ARG, "states and images must be "
                     "16-byte aligned");
  TcArgs a{};
  a.n = n;
  a.c = c;
  a.num_blocks = num_blocks;
  a.num_states = num_states;
  a.in_stride = in_stride;
  uint64_t seen = 0;
  for (int j = 0; j < TC_M; ++j) {
    const int p = positions[j];
    if (p < 0 || p >= n || ((seen >> p) & 1))
      return set_error(GBSV_ERR_INVALID_ARG, "bad tile position %d", p);
    if (j < c && p != j)
      return set_error(GBSV_ERR_INVALID_ARG,
                       "tile bit %d must be position %d", j, j);
    seen |= uint64_t(1) << p;
    a.spos[j] = p;
    if (j >= c) a.hpos[j - c] = p;
  }
  for (int i = 1; i < TC_M; ++i)
    for (int j = i; j > 0 && a.spos[j - 1] > a.spos[j]; --j) {
      const int tmp = a.spos[j];
      a.spos[j] = a.spos[j - 1];
      a.spos[j - 1] = tmp;
    }
  a.blocks = static_cast<const TcBlock*>(blocks);
  a.diags = static_cast<const TcDiag*>(diags);
  a.images = static_cast<const unsigned char*>(images);
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(tc_stage_kernel,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         TC_SMEM_BYTES);
    attr_set = true;
  }
  const uint64_t tiles =
      (uint64_t)num_states << (n - TC_M);
  const uint64_t grid = std::min<uint64_t>(tiles, (uint64_t)sm_count() * 2);
  tc_stage_kernel<<<(unsigned)grid, TC_THREADS, TC_SMEM_BYTES,
                    static_cast<cudaStream_t>(stream)>>>(
      static_cast<const float2*>(state_in), static_cast<float2*>(state_out),
      a);
  return after_launch("tc_stage_kernel");
}

extern "C" int gbsv_tc_status(int* status, int clear) {
  if (!status) return set_error(GBSV_ERR_INVALID_ARG, "null pointer");
  cudaError_t e = cudaMemcpyFromSymbol(status, gbsv::g_tc_status, sizeof(int));
  if (e != cudaSuccess)
    return set_error(GBSV_ERR_CUDA, "tc status: %s", cudaGetErrorString(e));
  if (clear) {
    const int zero = 0;
    e = cudaMemcpyToSymbol(gbsv::g_tc_status, &zero, sizeof(int));
    if (e != cudaSuccess)
      return set_error(GBSV_ERR_CUDA, "tc status: %s", cudaGetErrorString(e));
  }
  return GBSV_OK;
}
