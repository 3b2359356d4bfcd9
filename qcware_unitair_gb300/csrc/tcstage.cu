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
//     below 2^10, and splits x*s = hi + lo with hi an integer (|hi| <=
//     1024, exact in fp16) and lo (|lo| <= 1/2) rounded to fp16;
//   * the host splits 1024 * B the same way into an integer matrix Bh and
//     an fp16 residual Bl = 1024 * B - Bh (|Bl| <= 1/2);
//   * D1 = hi * Bh is a sum of integer products bounded by
//     1024 * (1024 * 8 + 32) < 2^24 (a unitary's real-form columns have
//     L1 norm <= 8), so every partial sum is an exact FP32 integer and the
//     truncating accumulator makes no error;
//   * Dc = hi * Bl + lo * Bh (the three-product split of Ootomo & Yokota
//     2022, as one K = 128 product [hi | lo] * [Bl; Bh]) carries the
//     correction, about 2^-11 of D1's magnitude, where the truncation
//     costs about 2^-34 relative;
//   * y = (D1 + Dc) / (1024 s), an exact power-of-two scaling.
// The representation error is about 2^-22 of each column's largest
// amplitude per block.
//
// Diagonal gates whose bits are all outside a block's bits (thread bits,
// or positions outside the tile) commute with the block.  The host folds
// them into a per-block table of per-thread factors indexed by up to 5 bits
// outside the tile; the rare rest stay a list of post-diagonals.
//
// Work is split by role (two CTAs of 192 threads per SM, 107 KiB of shared
// memory and 256 tensor-memory columns each): four compute warps (gather,
// split, tcgen05.st, tcgen05.ld, scatter), one warp whose lane 0 issues the
// MMAs and streams block images (16 KiB, resident when a stage has at most
// two blocks, otherwise two buffers by cp.async.bulk), and one warp that
// loads tiles by 16-byte cp.async into two buffers and writes finished
// tiles back, so the memory pipeline never stalls the compute warps.
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
constexpr int TC_MAX_SDIAG = 64;     // post-diagonals staged in shared memory
constexpr int TC_IMG_BYTES = 16384;
constexpr int TC_SMEM_BYTES = 2 * TC_TILE * 8 + 2 * TC_IMG_BYTES + 1024;

// Block record (gbsv_tc_block_t).  Shared-memory offsets are in amplitudes
// after the tile swizzle; the swizzle is linear over GF(2), so amplitude
// (thread bits of r) | (register bits of i) sits at
// XOR(tspo[j] : bit j of r) ^ XOR(rspo[k] : bit k of i).
struct TcBlock {
  int16_t rspo[TC_RB];  // register-index bit k -> swizzled offset
  int16_t tspo[TC_TB];  // thread-index bit j -> swizzled offset
  int32_t mat;          // image index (16 KiB each)
  int32_t first_diag;   // post-diagonals [first_diag, first_diag + num_diag)
  int32_t num_diag;
  int32_t flags;        // TC_PAIRS: register bit 0 is tile bit 0
  int32_t fac;          // factor table: factors[fac + p * 128 + thread]
  int8_t nout;          // p's bits: the state's bits at positions opos[]
  int8_t opos[7];
  int32_t pad_[3];
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
  const float2* factors;
};

static __device__ int g_tc_status;  // nonzero after a bounded wait ran out

// Tile swizzle: amplitude bits 1-3 ^= bits 4-6 ^ 7-9 ^ 10-12.  Bit 0 stays,
// so 16-byte pieces (two amplitudes) stay whole for the copies, and every
// tile bit >= 1 has a non-zero image in the bank bits.
__device__ __forceinline__ int tc_swz(int l) {
  return l ^ ((((l >> 4) ^ (l >> 7) ^ (l >> 10)) & 7) << 1);
}

// Lowest set bit of a (compile-time) register index.
__host__ __device__ constexpr int tc_ctz(int i) {
  return (i & 1) ? 0 : (i & 2) ? 1 : (i & 4) ? 2 : (i & 8) ? 3 : 4;
}

__device__ __forceinline__ uint32_t tc_smem(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Wait for phase `parity` of an mbarrier, for at most about 2^31 cycles.
// try_wait suspends the thread until the phase completes or the hinted
// time (1 ms) passes, so a waiting warp takes no issue slots.
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  while (true) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity), "r"(1000000u)
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
// 8-row groups 2048 bytes apart (stride byte offset).
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) |
         ((uint64_t)(2048 >> 4) << 32) | ((uint64_t)1 << 46);
}

// D (f32) = A (f16, tensor memory) * B (f16, shared memory), M = 128,
// N = 64 or 128, K = 16; accumulate into D when acc != 0.
template <int N>
__device__ __forceinline__ void tc_mma(uint32_t d, uint32_t a, uint64_t b,
                                       uint32_t acc) {
  constexpr uint32_t idesc = (1u << 4)  // D f32; A, B f16; both K-major
                             | ((uint32_t)(N >> 3) << 17) |
                             ((uint32_t)(128 >> 4) << 24);
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(
          d),
      "r"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

#define TC_R16(r)                                                            \
  "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]),          \
      "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]),    \
      "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])

// 16 consecutive 32-bit columns of this thread's lane.
__device__ __forceinline__ void tc_st16(uint32_t taddr, const uint32_t* r) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
      "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(taddr),
      TC_R16(r)
      : "memory");
}

#define TC_W32(r)                                                            \
  "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),    \
      "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]),           \
      "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),       \
      "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),       \
      "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),       \
      "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),       \
      "=r"(r[31])
__device__ __forceinline__ void tc_ld32(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
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

// Roles (192 threads): warps 0-3 compute (thread r owns column r of the
// tile and TMEM lane r), warp 4 lane 0 issues the MMAs and streams block
// images, warp 5 loads and stores tiles.  They hand over through mbarriers:
//   full[b]   tile buffer b loaded      (warp 5 cp.async -> compute)
//   empty[b]  tile buffer b computed    (compute -> warp 5: store, refill)
//   a_ready   A written to TMEM         (compute -> MMA lane)
//   mma_done  MMAs of a block complete  (tcgen05.commit -> compute)
//   img[b]    block image b landed      (cp.async.bulk -> MMA lane)
// Every wait is bounded (tc_wait); one that runs out sets the CTA's abort
// flag and the error status, and every role then leaves its loop.
constexpr int TC_ROLE_THREADS = TC_THREADS + 64;

// Barrier 1 over the compute warps, returning the OR of x over them.
__device__ __forceinline__ bool tc_compute_sync_or(bool x) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\t"
      "bar.red.or.pred q, 1, %2, p;\n\tselp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)x), "n"(TC_THREADS)
      : "memory");
  return r != 0;
}

__global__ void __launch_bounds__(TC_ROLE_THREADS, 2)
    tc_stage_kernel(const float2* in, float2* out, TcArgs a) {
  extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
  // 1024-byte alignment of the dynamic area is not guaranteed: round up
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
  float2* const tiles = reinterpret_cast<float2*>(smem);
  unsigned char* const imgs = smem + 2 * TC_TILE * 8;
  __shared__ TcBlock sblk[TC_MAX_BLOCKS];
  __shared__ TcDiag sdiag[TC_MAX_SDIAG];
  __shared__ uint64_t offh[16];
  __shared__ __align__(8) uint64_t bar_full[2], bar_empty[2], bar_img[2];
  __shared__ __align__(8) uint64_t bar_a, bar_mma;
  __shared__ uint32_t s_tmem;
  __shared__ volatile int s_abort;

  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int lane_id = tid & 31;
  const int nb = a.num_blocks;
  const uint64_t tps = uint64_t(1) << (a.n - TC_M);
  const uint64_t num_tiles = (uint64_t)a.num_states * tps;
  const uint64_t t0 = (uint64_t)blockIdx.x * num_tiles / gridDim.x;
  const uint64_t t1 = (uint64_t)(blockIdx.x + 1) * num_tiles / gridDim.x;
  if (t0 >= t1) return;
  const uint64_t ntile = t1 - t0;
  const uint64_t total_exec = ntile * (uint64_t)nb;

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
    auto init = [](uint64_t* bar, int count) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(
                       tc_smem(bar)),
                   "r"(count));
    };
    init(&bar_full[0], 32);  // one cp.async arrival per loader lane
    init(&bar_full[1], 32);
    init(&bar_empty[0], TC_THREADS);
    init(&bar_empty[1], TC_THREADS);
    init(&bar_img[0], 1);
    init(&bar_img[1], 1);
    init(&bar_a, TC_THREADS);
    init(&bar_mma, 1);
    s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int i = tid; i < nb * 16; i += TC_ROLE_THREADS)
    reinterpret_cast<int32_t*>(sblk)[i] =
        reinterpret_cast<const int32_t*>(a.blocks)[i];
  // the stage's post-diagonals: one contiguous range, staged in shared
  // memory when it fits (read from global memory otherwise)
  const int dfirst = a.blocks[0].first_diag;
  const int dcount =
      a.blocks[nb - 1].first_diag + a.blocks[nb - 1].num_diag - dfirst;
  const bool dshared = dcount <= TC_MAX_SDIAG;
  if (dshared)
    for (int i = tid; i < dcount * 12; i += TC_ROLE_THREADS)
      reinterpret_cast<int32_t*>(sdiag)[i] =
          reinterpret_cast<const int32_t*>(a.diags + dfirst)[i];
  const TcDiag* const dtab = dshared ? sdiag - dfirst : a.diags;
  if (tid < 16) offh[tid] = tc_tile_offset(a, 256 * tid);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = s_tmem;

  // tiles of a CTA are consecutive: the base (the tile's amplitude bits
  // outside the tile) steps by a masked increment over the outside bits
  uint64_t tmask = ~((uint64_t(1) << a.n) - 1);
  for (int j = 0; j < TC_M; ++j) tmask |= uint64_t(1) << a.spos[j];
  auto next_base = [&](uint64_t b) { return ((b | tmask) + 1) & ~tmask; };
  auto fail = [&](int code) {
    s_abort = 1;
    atomicOr(&g_tc_status, code);
  };

  if (warp == 5) {
    // ---------------------------------------------- tile loader / storer
    // lane l moves 16-byte pieces l, l + 32, ... (amplitudes 2 * piece);
    // piece p = 32 i + l has tile index 2p = 64 i + 2 l
    const uint64_t offl = tc_tile_offset(a, 2 * lane_id);
    uint64_t offs[4];  // 64 i = 256 (i >> 2) + 64 (i & 3)
#pragma unroll
    for (int q = 0; q < 4; ++q) offs[q] = tc_tile_offset(a, 64 * q) + offl;
    auto load = [&](uint64_t s, uint64_t base, int b) {
      float2* S = tiles + b * TC_TILE;
      const float2* src = in + (int64_t)s * a.in_stride + base;
#pragma unroll 8
      for (int i = 0; i < 64; ++i) {
        const int l = 64 * i + 2 * lane_id;
        cp_async16<float>(&S[tc_swz(l)], src + offh[i >> 2] + offs[i & 3]);
      }
      asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::
                       "r"(tc_smem(&bar_full[b]))
                   : "memory");
    };
    uint64_t s = t0 / tps, base = tc_tile_base(a, t0 % tps);
    uint64_t ls = s, lbase = base;  // next tile to load
    for (uint64_t k = 0; k < 2 && k < ntile; ++k) {
      load(ls, lbase, (int)k);
      lbase = next_base(lbase);
      ls += lbase == 0;
    }
    for (uint64_t k = 0; k < ntile; ++k) {
      const int b = (int)(k & 1);
      if (!tc_wait(tc_smem(&bar_empty[b]), (uint32_t)((k >> 1) & 1))) {
        fail(16);
        break;
      }
      const float2* S = tiles + b * TC_TILE;
      float2* dst = out + (s << a.n) + base;
#pragma unroll 8
      for (int i = 0; i < 64; ++i) {
        const int l = 64 * i + 2 * lane_id;
        const float4 w = *reinterpret_cast<const float4*>(&S[tc_swz(l)]);
        __stcs(reinterpret_cast<float4*>(dst + offh[i >> 2] + offs[i & 3]),
               w);
      }
      __syncwarp();  // every lane's reads done before the buffer refills
      if (k + 2 < ntile) {
        load(ls, lbase, b);
        lbase = next_base(lbase);
        ls += lbase == 0;
      }
      base = next_base(base);
      s += base == 0;
      if (s_abort) break;
    }
    cp_async_wait_all();
  } else if (warp == 4) {
    // -------------------------------------------------------- MMA issuer
    if (lane_id == 0) {
      const bool resident = nb <= 2;
      uint32_t img_phase = 0;  // bit b: parity of the next wait on img[b]
      int img_pending = 0;
      const int first = resident ? nb : (total_exec < 2 ? (int)total_exec : 2);
      for (int e = 0; e < first; ++e) {
        tc_load_image(tc_smem(imgs + e * TC_IMG_BYTES),
                      a.images + (size_t)sblk[e % nb].mat * TC_IMG_BYTES,
                      tc_smem(&bar_img[e]));
        img_pending |= 1 << e;
      }
      for (uint64_t e = 0; e < total_exec; ++e) {
        const int bi = (int)(e % nb);
        const int buf = resident ? bi : (int)(e & 1);
        if (!tc_wait(tc_smem(&bar_a), (uint32_t)(e & 1))) {
          fail(32);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        bool ok = true;
        if ((img_pending >> buf) & 1) {
          ok = tc_wait(tc_smem(&bar_img[buf]), (img_phase >> buf) & 1);
          img_pending &= ~(1 << buf);
          img_phase ^= 1u << buf;
        }
        if (ok) {
          // image: [Bl; Bh] as a K = 128 x N = 64 operand (8-row groups
          // 2048 bytes apart); Bh alone starts 1024 bytes in
          const uint32_t im = tc_smem(imgs + buf * TC_IMG_BYTES);
#pragma unroll
          for (int j = 0; j < 4; ++j)
            tc_mma<64>(tmem + 64, tmem + 8 * j, tc_desc(im + 1024 + 256 * j),
                       j > 0);
#pragma unroll
          for (int j = 0; j < 8; ++j)
            tc_mma<64>(tmem + 128, tmem + 8 * j, tc_desc(im + 256 * j), j > 0);
        } else {
          fail(1);
        }
        // commit even after a failed wait: it then arrives at once
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::"
            "cluster.b64 [%0];" ::"r"(tc_smem(&bar_mma))
            : "memory");
        if (!ok) break;
        if (!resident && e + 2 < total_exec) {
          // image buffer `buf` is free once these MMAs complete
          if (!tc_wait(tc_smem(&bar_mma), (uint32_t)(e & 1))) {
            fail(2);
            break;
          }
          tc_load_image(
              tc_smem(imgs + buf * TC_IMG_BYTES),
              a.images + (size_t)sblk[(int)((e + 2) % nb)].mat * TC_IMG_BYTES,
              tc_smem(&bar_img[buf]));
          img_pending |= 1 << buf;
        }
        if (s_abort) break;
      }
      for (int b = 0; b < 2; ++b)
        if ((img_pending >> b) & 1)
          if (!tc_wait(tc_smem(&bar_img[b]), (img_phase >> b) & 1)) fail(4);
    }
  } else {
    // ---------------------------------------------------------- compute
    const uint32_t lane = (uint32_t)(warp * 32) << 16;
    const uint32_t tA = tmem, tD1 = tmem + 64, tDc = tmem + 128;
    uint64_t s = t0 / tps, base = tc_tile_base(a, t0 % tps);
    // A wait that runs out only sets `bad`: every compute thread runs the
    // same tcgen05 and barrier sequence, and all leave together after the
    // reduction barrier that ends each block.
    uint64_t e = 0;
    bool bad = false;
    bool late = false;  // an MMA completion wait ran out
    for (uint64_t k = 0; k < ntile && !bad; ++k) {
      const int b = (int)(k & 1);
      float2* const S = tiles + b * TC_TILE;
      if (!tc_wait(tc_smem(&bar_full[b]), (uint32_t)((k >> 1) & 1))) {
        fail(64);
        bad = true;
      }
      for (int bi = 0; bi < nb; ++bi, ++e) {
        const TcBlock& B = sblk[bi];
        int sb = 0;
#pragma unroll
        for (int j = 0; j < TC_TB; ++j)
          if ((tid >> j) & 1) sb ^= B.tspo[j];
        int rs[TC_RB];
#pragma unroll
        for (int j = 0; j < TC_RB; ++j) rs[j] = B.rspo[j];
        const bool pairs = B.flags & TC_PAIRS;
        // this thread's factor of the diagonals folded into the block's
        // table, loaded now and used after the MMAs
        float2 fv = make_float2(1.f, 0.f);
        const int fac = B.fac;
        if (fac >= 0) {
          int p = 0;
          for (int j = 0; j < B.nout; ++j)
            p |= (int)((base >> B.opos[j]) & 1) << j;
          fv = __ldg(a.factors + fac + p * TC_THREADS + tid);
        }
        // register i lives at sb ^ (XOR of rs[j] over the bits j of i)
        int ad[32];
        auto addresses = [&]() {
          ad[0] = sb;
#pragma unroll
          for (int i = 1; i < 32; ++i)
            ad[i] = ad[i & (i - 1)] ^ rs[tc_ctz(i)];
        };
        addresses();
        float2 v[32];
        if (pairs) {
#pragma unroll
          for (int i = 0; i < 32; i += 2) {
            const float4 w = *reinterpret_cast<const float4*>(&S[ad[i]]);
            v[i] = make_float2(w.x, w.y);
            v[i + 1] = make_float2(w.z, w.w);
          }
        } else {
#pragma unroll
          for (int i = 0; i < 32; ++i) v[i] = S[ad[i]];
        }
        // power-of-two scaling (largest |x| of the column, tree reduction)
        float mx[16];
#pragma unroll
        for (int i = 0; i < 16; ++i)
          mx[i] = fmaxf(fmaxf(fabsf(v[i].x), fabsf(v[i].y)),
                        fmaxf(fabsf(v[i + 16].x), fabsf(v[i + 16].y)));
#pragma unroll
        for (int w = 8; w > 0; w >>= 1)
#pragma unroll
          for (int i = 0; i < w; ++i) mx[i] = fmaxf(mx[i], mx[i + w]);
        const int E = max((int)(__float_as_uint(mx[0]) >> 23), 20);
        const float sc = __uint_as_float((uint32_t)(263 - E) << 23);
        const float inv = __uint_as_float((uint32_t)(E - 19) << 23);
        // x * sc = hi + lo: hi = x * sc rounded to an integer (adding and
        // removing 1.5 * 2^23 rounds to nearest; |x * sc| < 2^10), lo the
        // exact remainder (|lo| <= 1/2), both to fp16
        constexpr float RND = 12582912.f;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          uint32_t hi[16], lo[16];
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const float2 x = v[16 * h + j];
            const float hr = fmaf(x.x, sc, RND) - RND;
            const float hm = fmaf(x.y, sc, RND) - RND;
            hi[j] = tc_pack(hr, hm);
            lo[j] = tc_pack(fmaf(x.x, sc, -hr), fmaf(x.y, sc, -hm));
          }
          tc_st16(tA + lane + 16 * h, hi);
          tc_st16(tA + 32 + lane + 16 * h, lo);
        }
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(
                         tc_smem(&bar_a))
                     : "memory");
        // post-diagonals left in the list (a register bit, or too many
        // outside bits), while the MMAs run
        float2 f = make_float2(fv.x * inv, fv.y * inv);
        bool regdiag = false;
        const bool has_diag = B.num_diag > 0 || fac >= 0;
        for (int q = B.first_diag; q < B.first_diag + B.num_diag; ++q) {
          const TcDiag& dg = dtab[q];
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
        if (!tc_wait(tc_smem(&bar_mma), (uint32_t)(e & 1))) {
          fail(2);
          late = true;
          bad = true;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // read back D1 + Dc, undo the scaling, apply the factors
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          uint32_t d1[32], dc[32];
          tc_ld32(tD1 + lane + 32 * h, d1);
          tc_ld32(tDc + lane + 32 * h, dc);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const float re =
                __uint_as_float(d1[2 * j]) + __uint_as_float(dc[2 * j]);
            const float im = __uint_as_float(d1[2 * j + 1]) +
                             __uint_as_float(dc[2 * j + 1]);
            v[16 * h + j] = has_diag ? cmul(f, make_float2(re, im))
                                     : make_float2(re * inv, im * inv);
          }
        }
        if (regdiag) {
          for (int q = B.first_diag; q < B.first_diag + B.num_diag; ++q) {
            const TcDiag& dg = dtab[q];
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
        addresses();
        if (pairs) {
#pragma unroll
          for (int i = 0; i < 32; i += 2)
            *reinterpret_cast<float4*>(&S[ad[i]]) =
                make_float4(v[i].x, v[i].y, v[i + 1].x, v[i + 1].y);
        } else {
#pragma unroll
          for (int i = 0; i < 32; ++i) S[ad[i]] = v[i];
        }
        // the next block reads other threads' results; errors anywhere
        // stop every compute thread here
        bad = tc_compute_sync_or(bad || s_abort);
        if (bad) break;
      }
      if (bad) break;
      // this thread's part of the tile is final: the storer may take it
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(
                       tc_smem(&bar_empty[b]))
                   : "memory");
      base = next_base(base);
      s += base == 0;
    }
    if (late && !tc_wait(tc_smem(&bar_mma), (uint32_t)((e & 1)))) fail(8);
  }
  // every role is done (waits are bounded): free tensor memory
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
                                 const void* factors, void* stream) {
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
  a.factors = static_cast<const float2*>(factors);
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
  tc_stage_kernel<<<(unsigned)grid, TC_ROLE_THREADS, TC_SMEM_BYTES,
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
