// The main loop shared by the tensor-core scans: D = A . B' on tcgen05 with
// A the 0/1/2 codings of 128 (SNP, term) rows, decoded in shared memory from
// the packed 2-bit codes, and B any bf16 matrix of n_pad columns (the
// residual digits of the RB scan, the model columns of the Schur scan).
//
// A persistent CTA walks the tiles (tile = blockIdx.x + i gridDim.x, m tile =
// tile % m_tiles).  Warps 0-3 decode A, warp 4 issues the TMA loads of the
// packed rows and of B, warp 5 owns 512 TMEM columns and issues the MMAs of
// tile i into accumulator i & 1;
// the kernel's own epilogue warps (from warp 6 on) drain the other one and
// hand it back through acc_empty.  Every wait is bounded; a timeout sets
// abort_flag and every role leaves its loop after draining its own
// asynchronous work.
//
// A is staged in one of two places:
//  - tensor memory (a_tmem): the decode warps write each stage's 128 x 64
//    bf16 block into one of a_stages slots of 32 TMEM columns after the two
//    accumulators, and the MMA reads A from there.  Shared memory then
//    carries only B and the packed codes (the main loop is bound by
//    shared-memory bandwidth and by the latency of the TMA loads), so its
//    ring can be deeper than the TMEM ring.  Slot g % a_stages is free once
//    the MMA of stage g - a_stages has completed: the decode waits for that
//    stage's empty_bar phase, which cannot have moved on before stage g is
//    decoded (a later phase needs the MMA of stage g - a_stages + stages);
//  - shared memory, 128-byte swizzled, when the accumulators leave no room
//    (more than 192 columns each, as in the Schur scan of large models).
#ifndef BMG_TC_MAINLOOP_CUH_
#define BMG_TC_MAINLOOP_CUH_

#include "common.cuh"
#include "tc_common.cuh"

namespace {

constexpr int TC_MAX_STAGES = 8;    // shared-memory ring (B and packed codes)
constexpr int TC_MAX_A_STAGES = 4;  // TMEM ring of A when A is in tensor memory
constexpr int TC_BM = 128;          // rows of D per tile
constexpr int TC_BK = 64;           // individuals per stage (128 bytes of bf16)
constexpr uint32_t TC_ACC_COLS = 256;  // widest accumulator
constexpr uint32_t TC_TMEM_COLS = 512; // two accumulators (+ the A stages)
constexpr uint32_t TC_A_COLS = TC_BK / 2;  // TMEM columns of one A stage

struct TcParams {
  uint32_t tpad;           // rows per SNP (terms rounded up to 1, 2 or 4)
  uint32_t snps_per_tile;  // TC_BM / tpad
  uint32_t chains_tile;    // chains per N tile
  uint32_t n_mma;          // N of the MMA (chains_tile * L rounded up to 16)
  uint32_t k_chunks;       // n_pad / TC_BK
  uint32_t stages;         // shared-memory ring depth (2..TC_MAX_STAGES)
  uint32_t a_stages;       // A ring depth: TMEM slots (a_tmem), else = stages
  uint32_t m_tiles, n_tiles, tiles;
  uint32_t xr_bytes;       // epilogue shared memory after the stages
  uint32_t b_rows_per_tile;  // B rows between consecutive N tiles
  uint32_t stage_bytes;
  uint32_t b_bytes, a_bytes, pk_bytes;  // a_bytes = 0 when A is in TMEM
  uint32_t acc_cols;       // TMEM column stride of the two accumulators
  uint32_t a_tmem;         // 1: A stage st at TMEM column 2 acc_cols + st TC_A_COLS
  int32_t term_of_row[4];  // term of row u of a SNP (-1: unused)
};

// Where the accumulators and A go: A in TMEM when two accumulators of n_mma
// columns (rounded up to 32) leave room for at least two A slots; else A in
// shared memory (a_stages is then set to the ring depth by the caller).
__host__ __device__ inline void tc_place_a(TcParams& P)
{
  const uint32_t acc = ((P.n_mma + 31) / 32) * 32;
  const uint32_t room = TC_TMEM_COLS >= 2 * acc ? (TC_TMEM_COLS - 2 * acc) / TC_A_COLS : 0;
  const uint32_t st = room < (uint32_t)TC_MAX_A_STAGES ? room : (uint32_t)TC_MAX_A_STAGES;
  if (st >= 2) {
    P.a_tmem = 1;
    P.a_stages = st;
    P.acc_cols = acc;
    P.a_bytes = 0;
  } else {
    P.a_tmem = 0;
    P.a_stages = 0;
    P.acc_cols = TC_ACC_COLS;
    P.a_bytes = TC_BM * 128;
  }
}


// barriers and flags of one CTA
struct TcCtl {
  uint64_t full_bar[TC_MAX_STAGES], aready_bar[TC_MAX_STAGES], empty_bar[TC_MAX_STAGES];
  uint64_t acc_full[2], acc_empty[2], drain_bar;
  uint32_t tmem_base;
  volatile int abort_flag;
};

// Decode table of one term: entry x (a nibble of packed codes, two
// individuals) holds their bf16 values, the first in the low half.  16 entries
// of 4 bytes sit in 16 distinct banks, so a warp's lookups never conflict.
// Row TC_LUT_ZERO is all zeros (rows of a SNP beyond its terms).
constexpr int TC_LUT_ZERO = 4;
typedef uint32_t TcLut[TC_LUT_ZERO + 1][16];

// All threads: decode tables, barriers, tensor memory.  Returns the TMEM base.
__device__ __forceinline__ uint32_t tc_setup(const TcParams& P, TcCtl& ctl, TcLut& lut, int threads, int epi_warps)
{
  const int tid = threadIdx.x, warp = tid >> 5;
  // bf16 bit patterns of 0, 1, 2 are 0x0000, 0x3F80, 0x4000
  for (int e = tid; e < (TC_LUT_ZERO + 1) * 16; e += threads) {
    const int term = e >> 4, x = e & 15;
    uint32_t h[2];
    for (int q = 0; q < 2; ++q) {
      const int v = term == TC_LUT_ZERO ? 0 : term_value((x >> (2 * q)) & 3, term);
      h[q] = v == 0 ? 0 : (v == 1 ? 0x3F80 : 0x4000);
    }
    lut[term][x] = h[0] | (h[1] << 16);
  }
  if (tid == 0) {
    for (uint32_t st = 0; st < P.stages; ++st) {
      mbar_init(&ctl.full_bar[st], 1);
      mbar_init(&ctl.empty_bar[st], 1);
    }
    for (uint32_t t = 0; t < P.a_stages; ++t) mbar_init(&ctl.aready_bar[t], 4);
    for (int b = 0; b < 2; ++b) {
      mbar_init(&ctl.acc_full[b], 1);
      mbar_init(&ctl.acc_empty[b], epi_warps);
    }
    mbar_init(&ctl.drain_bar, 1);
    ctl.abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 5) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&ctl.tmem_base)),
                 "r"(TC_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  return ctl.tmem_base;
}

// Warps 0-5: the decode, TMA and MMA roles over this CTA's tiles.
__device__ __forceinline__ void tc_main_roles(const TcParams& P, TcCtl& ctl, const TcLut& lut, uint8_t* smem,
                                              uint32_t tmem, uint32_t my_tiles, const CUtensorMap& map_b,
                                              const CUtensorMap& map_g)
{
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t nk = P.k_chunks, S = P.stages, SA = P.a_stages;
  uint64_t* full_bar = ctl.full_bar;
  uint64_t* aready_bar = ctl.aready_bar;
  uint64_t* empty_bar = ctl.empty_bar;
  if (warp == 4) {
    if (lane == 0) {
      // TMA producer: packed genotype rows and the B rows of each stage
      uint32_t issued = 0;
      for (uint32_t i = 0; i < my_tiles && !ctl.abort_flag; ++i) {
        const uint32_t tile = blockIdx.x + i * gridDim.x;
        const uint32_t snp0 = (tile % P.m_tiles) * P.snps_per_tile;
        const uint32_t brow0 = (tile / P.m_tiles) * P.b_rows_per_tile;
        for (uint32_t k = 0; k < nk; ++k) {
          const uint32_t g = i * nk + k, st = g % S;
          if (g >= S && !mbar_wait(&empty_bar[st], ((g / S) - 1) & 1)) { ctl.abort_flag = 1; break; }
          uint8_t* sp = smem + st * P.stage_bytes;
          mbar_arrive_tx(&full_bar[st], P.b_bytes + P.pk_bytes);
          tma_load_2d(sp, &map_b, &full_bar[st], (int)(k * TC_BK), (int)brow0);
          tma_load_2d(sp + P.b_bytes + P.a_bytes, &map_g, &full_bar[st], (int)(k * (TC_BK / 4)), (int)snp0);
          ++issued;
        }
      }
      // no load may still be landing in shared memory when the CTA exits:
      // wait (bounded) for the last load of every stage
      for (uint32_t g = issued > S ? issued - S : 0; g < issued; ++g) mbar_wait(&full_bar[g % S], (g / S) & 1);
    }
  } else if (warp == 5) {
    if (lane == 0) {
      // MMA issuer: tile i accumulates into buffer i & 1
      const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((P.n_mma >> 3) << 17) | ((uint32_t)(TC_BM >> 4) << 24);
      for (uint32_t i = 0; i < my_tiles && !ctl.abort_flag; ++i) {
        const uint32_t b = i & 1, u = i >> 1;
        if (u >= 1 && !mbar_wait(&ctl.acc_empty[b], (u - 1) & 1)) { ctl.abort_flag = 1; break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t d = tmem + b * P.acc_cols;
        bool ok = true;
        for (uint32_t k = 0; k < nk; ++k) {
          const uint32_t g = i * nk + k, st = g % S, par = (g / S) & 1, ta = g % SA;
          if (!mbar_wait(&full_bar[st], par) || !mbar_wait(&aready_bar[ta], (g / SA) & 1)) { ok = false; break; }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          uint8_t* sp = smem + st * P.stage_bytes;
          const uint64_t bdesc = smem_desc(sp);
          if (P.a_tmem) {
            const uint32_t at = tmem + 2 * P.acc_cols + ta * TC_A_COLS;
#pragma unroll
            for (int kk = 0; kk < TC_BK / 16; ++kk)  // 16 bf16: 8 TMEM columns of A, 2 descriptor units of B
              mma_bf16_tmem_a(d, at + 8 * kk, bdesc + 2 * kk, idesc, (k | kk) != 0);
          } else {
            const uint64_t adesc = smem_desc(sp + P.b_bytes);
#pragma unroll
            for (int kk = 0; kk < TC_BK / 16; ++kk)  // 16 bf16 = 32 bytes = 2 descriptor units
              mma_bf16(d, adesc + 2 * kk, bdesc + 2 * kk, idesc, (k | kk) != 0);
          }
          mma_commit(&empty_bar[st]);
        }
        if (!ok) { ctl.abort_flag = 1; break; }
        mma_commit(&ctl.acc_full[b]);
      }
      // every MMA issued has completed before tensor memory is freed
      mma_commit(&ctl.drain_bar);
      if (!mbar_wait(&ctl.drain_bar, 0)) ctl.abort_flag = 1;
    }
  } else if (warp < 4) {
    // decode warps: packed 2-bit codes -> bf16 rows of A; thread = row = TMEM lane
    const uint32_t row = tid;  // 0..127
    const uint32_t sl = row / P.tpad, u = row % P.tpad;
    const uint32_t* tl = lut[P.term_of_row[u] >= 0 ? P.term_of_row[u] : TC_LUT_ZERO];
    const uint32_t total = my_tiles * nk;
    const uint32_t a_lane = tmem + ((uint32_t)(warp * 32) << 16) + 2 * P.acc_cols;
    for (uint32_t g = 0; g < total; ++g) {
      const uint32_t st = g % S, par = (g / S) & 1, ta = g % SA;
      // A in shared memory: the TMA of this stage was issued after the MMA of
      // its previous round completed (empty_bar), so that MMA no longer reads
      // the stage's A.  A in TMEM: slot ta is free after the MMA of stage
      // g - SA.  The verdict is warp-uniform: the TMEM store is .sync.aligned.
      const uint32_t gp = g - SA;
      const bool ok = !ctl.abort_flag && mbar_wait(&full_bar[st], par) &&
                      (!P.a_tmem || g < SA || mbar_wait(&empty_bar[gp % S], (gp / S) & 1));
      if (!__all_sync(0xffffffffu, ok)) { ctl.abort_flag = 1; break; }
      uint8_t* sp = smem + st * P.stage_bytes;
      const uint8_t* pk = sp + P.b_bytes + P.a_bytes + sl * 16;
      const uint4 bytes = *reinterpret_cast<const uint4*>(pk);
      const uint32_t w[4] = {bytes.x, bytes.y, bytes.z, bytes.w};
      if (P.a_tmem) {
        // 64 individuals = 32 columns, column q = individuals 2q, 2q + 1
        uint32_t v[32];
#pragma unroll
        for (int q = 0; q < 32; ++q) v[q] = tl[(w[q >> 3] >> (4 * (q & 7))) & 15];
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        tmem_st32(a_lane + ta * TC_A_COLS, v);
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      } else {
        uint8_t* a = sp + P.b_bytes;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          // 16-byte chunk c of the row: individuals 8c .. 8c + 7, 16 bits of codes
          const uint32_t h = w[c >> 1] >> ((c & 1) * 16);
          const uint4 v = make_uint4(tl[h & 15], tl[(h >> 4) & 15], tl[(h >> 8) & 15], tl[(h >> 12) & 15]);
          *reinterpret_cast<uint4*>(a + row * 128 + ((c ^ (row & 7)) << 4)) = v;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&aready_bar[ta]);
    }
  }
}

// All threads at the end: tensor memory freed once every role has drained.
// Returns true when a bounded wait gave up.
__device__ __forceinline__ bool tc_teardown(TcCtl& ctl, uint32_t tmem)
{
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  const bool aborted = ctl.abort_flag != 0;
  if ((threadIdx.x >> 5) == 5) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS));
  }
  return aborted;
}

}  // namespace

#endif
