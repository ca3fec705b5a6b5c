// The main loop shared by the tensor-core scans: D = A . B' on tcgen05 with
// A the 0/1/2 codings of 128 (SNP, term) rows, decoded from the packed 2-bit
// codes, and B any bf16 matrix of n_pad columns (the residual digits of the
// RB scan, the model columns of the Schur scan).
//
// A persistent CTA walks the tiles (tile = blockIdx.x + i gridDim.x, m tile =
// tile % m_tiles).  Warps 0-3 decode A, warp 4 issues the TMA loads of the
// packed rows and of B, warp 5 owns 512 TMEM columns and issues the MMAs of
// tile i into accumulator i % n_acc; the kernel's own epilogue warps (from
// warp 6 on) copy a finished accumulator out of TMEM and hand it back through
// acc_empty.  Every wait is bounded; a timeout sets abort_flag and every role
// leaves its loop after draining its own asynchronous work.
//
// Rings.  Stage g (128 individuals: chunk g of the CTA's walk over its tiles'
// K ranges) uses shared-memory slot
// g % stages (B and the packed codes, loaded by TMA, full_bar) and A slot
// g % a_stages (aready_bar).  The MMA of stage g commits to done_bar[g % ring],
// ring = max(stages, a_stages): the TMA waits for the MMA of stage g - stages
// before refilling a shared-memory slot, the decode for that of stage
// g - a_stages before rewriting an A slot in TMEM.  Neither phase can have
// moved on by then (a later phase of the same barrier needs the MMA of a
// stage >= g, which needs this stage first), so parity waits are exact.
//
// A is staged in one of two places:
//  - tensor memory (a_tmem): each stage's 128 x 128 bf16 block goes into 64
//    TMEM columns after the accumulators, and the MMA reads A from there.
//    Shared memory then carries only B and the packed codes (the main loop is
//    bound by shared-memory bandwidth and by latency).  With one accumulator
//    (n_acc = 1) five A slots fit; the epilogue copies the accumulator to
//    shared memory within microseconds and does its arithmetic from there
//    while the next tile accumulates, so one accumulator costs little overlap;
//  - shared memory, two 128-byte-swizzled sub-tiles of 64 individuals, when
//    the accumulators leave no room (the Schur scan of large models).
// B likewise arrives as two TMA boxes of 64 individuals per stage.
#ifndef BMG_TC_MAINLOOP_CUH_
#define BMG_TC_MAINLOOP_CUH_

#include "common.cuh"
#include "decode_bf16.h"
#include "tc_common.cuh"

namespace {

constexpr int TC_MAX_STAGES = 8;     // shared-memory ring (B and packed codes)
constexpr int TC_MAX_A_STAGES = 10;  // TMEM ring of A when A is in tensor memory
constexpr int TC_MAX_RING = 10;      // done_bar ring: max(stages, a_stages)
constexpr int TC_BM = 128;           // rows of D per tile
constexpr int TC_BK = 128;           // individuals per stage
constexpr int TC_BK_SUB = 64;        // individuals per 128-byte swizzle atom (one TMA box of B)
constexpr uint32_t TC_ACC_COLS = 256;   // widest accumulator
constexpr uint32_t TC_TMEM_COLS = 512;  // accumulators + the A slots
constexpr uint32_t TC_A_COLS = TC_BK / 2;  // TMEM columns of one A slot (two bf16 per column)
constexpr uint32_t TC_A_SUB_BYTES = TC_BM * 128;  // one swizzled A sub-tile in shared memory

struct TcParams {
  uint32_t tpad;           // rows per SNP (terms rounded up to 1, 2 or 4)
  uint32_t snps_per_tile;  // TC_BM / tpad
  uint32_t chains_tile;    // chains per N tile
  uint32_t n_mma;          // N of the MMA (chains_tile * L rounded up to 16)
  uint32_t k_chunks;       // n_pad / TC_BK
  uint32_t stages;         // shared-memory ring depth (2..TC_MAX_STAGES)
  uint32_t a_stages;       // A ring depth: TMEM slots (a_tmem), else = stages
  uint32_t ring;           // done_bar ring depth, max(stages, a_stages)
  uint32_t m_tiles, n_tiles, tiles;
  uint32_t xr_bytes;       // epilogue shared memory after the stages
  uint32_t b_rows_per_tile;  // B rows between consecutive N tiles
  uint32_t stage_bytes;
  uint32_t b_bytes, a_bytes, pk_bytes;  // a_bytes = 0 when A is in TMEM; B and A in two sub-tiles
  uint32_t n_acc;          // accumulators (1 or 2)
  uint32_t acc_cols;       // TMEM column stride of the accumulators
  uint32_t a_tmem;         // 1: A slot t at TMEM column n_acc acc_cols + t TC_A_COLS
  int32_t term_of_row[4];  // term of row u of a SNP (-1: unused)
  uint32_t wait_limit = 0;  // polls of a main-loop mbarrier wait (0: WAIT_LIMIT)
  // K segments of a tile: each closes its own accumulator (a job), so that
  // no FP32 partial sum runs over more than seg_chunks stages; the epilogue
  // adds the segments' exact integers.  0: one segment of all k_chunks.
  uint32_t seg_chunks = 0;
  // decode warps: 4 (warps 0-3, a row of 128 individuals each) or 8 (warps
  // 0-3 and 6-9, each row's two halves of 64 individuals; the epilogue then
  // starts at warp 10)
  uint32_t dec_warps = 4;
};

// stages of a tile's K segment s and the number of segments
__host__ __device__ inline uint32_t tc_seg_len(const TcParams& P)
{
  return (P.seg_chunks && P.seg_chunks < P.k_chunks) ? P.seg_chunks : P.k_chunks;
}
__host__ __device__ inline uint32_t tc_n_seg(const TcParams& P)
{
  const uint32_t sl = tc_seg_len(P);
  return (P.k_chunks + sl - 1) / sl;
}

// Where the accumulators and A go: A in TMEM when n_acc accumulators of n_mma
// columns (rounded up to 32) leave room for at least two A slots; else A in
// shared memory with two accumulators of TC_ACC_COLS.
__host__ __device__ inline void tc_place_a(TcParams& P, uint32_t n_acc)
{
  const uint32_t acc = ((P.n_mma + 31) / 32) * 32;
  const uint32_t used = n_acc * acc;
  const uint32_t room = TC_TMEM_COLS > used ? (TC_TMEM_COLS - used) / TC_A_COLS : 0;
  const uint32_t st = room < (uint32_t)TC_MAX_A_STAGES ? room : (uint32_t)TC_MAX_A_STAGES;
  if (st >= 2) {
    P.a_tmem = 1;
    P.a_stages = st;
    P.n_acc = n_acc;
    P.acc_cols = acc;
    P.a_bytes = 0;
  } else {
    P.a_tmem = 0;
    P.a_stages = 0;
    P.n_acc = 2;
    P.acc_cols = TC_ACC_COLS;
    P.a_bytes = 2 * TC_A_SUB_BYTES;
  }
}

// Once the shared-memory ring depth is known: A slots and the done ring.
__host__ __device__ inline void tc_set_rings(TcParams& P, uint32_t stages)
{
  P.stages = stages;
  if (!P.a_tmem) P.a_stages = stages;
  P.ring = P.stages > P.a_stages ? P.stages : P.a_stages;
}

// position in a ring of n slots: slot index and phase parity, advanced
// without divisions
struct TcRing {
  uint32_t i = 0, ph = 0;
  __device__ __forceinline__ void next(uint32_t n)
  {
    if (++i == n) {
      i = 0;
      ph ^= 1;
    }
  }
};

// barriers and flags of one CTA
struct TcCtl {
  uint64_t full_bar[TC_MAX_STAGES], aready_bar[TC_MAX_RING], done_bar[TC_MAX_RING];
  uint64_t acc_full[2], acc_empty[2], drain_bar;
  uint32_t tmem_base;
  volatile int abort_flag;
};

// All threads: barriers, tensor memory.  Returns the TMEM base.
__device__ __forceinline__ uint32_t tc_setup(const TcParams& P, TcCtl& ctl, int epi_warps)
{
  const int tid = threadIdx.x, warp = tid >> 5;
  if (tid == 0) {
    for (uint32_t st = 0; st < P.stages; ++st) mbar_init(&ctl.full_bar[st], 1);
    for (uint32_t t = 0; t < P.a_stages; ++t) mbar_init(&ctl.aready_bar[t], P.dec_warps);
    for (uint32_t r = 0; r < P.ring; ++r) mbar_init(&ctl.done_bar[r], 1);
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
__device__ __forceinline__ void tc_main_roles(const TcParams& P, TcCtl& ctl, uint8_t* smem,
                                              uint32_t tmem, uint32_t my_tiles, const CUtensorMap& map_b,
                                              const CUtensorMap& map_g)
{
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t nk = P.k_chunks, S = P.stages, SA = P.a_stages, R = P.ring;
  uint64_t* full_bar = ctl.full_bar;
  uint64_t* aready_bar = ctl.aready_bar;
  uint64_t* done_bar = ctl.done_bar;
  if (warp == 4) {
    if (lane == 0) {
      // TMA producer: packed genotype rows and the B rows of each stage
      uint32_t issued = 0;
      TcRing slot, done;  // this stage's shared-memory slot; the done phase of stage g - S
      const uint32_t b_half = P.b_bytes / 2;
      for (uint32_t i = 0; i < my_tiles && !ctl.abort_flag; ++i) {
        const uint32_t tile = blockIdx.x + i * gridDim.x;
        const uint32_t snp0 = (tile % P.m_tiles) * P.snps_per_tile;
        const uint32_t brow0 = (tile / P.m_tiles) * P.b_rows_per_tile;
        bool ok = true;
        for (uint32_t k = 0; k < nk; ++k) {
          if (issued >= S) {  // the slot's last reader is the MMA of stage g - S
            if (!mbar_wait(&done_bar[done.i], done.ph, P.wait_limit)) { ok = false; break; }
            done.next(R);
          }
          uint8_t* sp = smem + slot.i * P.stage_bytes;
          uint64_t* fb = &full_bar[slot.i];
          mbar_arrive_tx(fb, P.b_bytes + P.pk_bytes);
          tma_load_2d(sp, &map_b, fb, (int)(k * TC_BK), (int)brow0);
          tma_load_2d(sp + b_half, &map_b, fb, (int)(k * TC_BK + TC_BK_SUB), (int)brow0);
          tma_load_2d(sp + P.b_bytes + P.a_bytes, &map_g, fb, (int)(k * (TC_BK / 4)), (int)snp0);
          slot.next(S);
          ++issued;
        }
        if (!ok) { ctl.abort_flag = 1; break; }
      }
      // no load may still be landing in shared memory when the CTA exits:
      // wait (bounded) for the last load of every slot
      for (uint32_t g = issued > S ? issued - S : 0; g < issued; ++g) mbar_wait(&full_bar[g % S], (g / S) & 1);
    }
  } else if (warp == 5) {
    if (lane == 0) {
      // MMA issuer: tile i accumulates into buffer i % n_acc
      const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((P.n_mma >> 3) << 17) | ((uint32_t)(TC_BM >> 4) << 24);
      const uint32_t a_base = tmem + P.n_acc * P.acc_cols;
      const uint64_t d_base = smem_desc(smem);
      const uint32_t st16 = P.stage_bytes >> 4, bh16 = (P.b_bytes / 2) >> 4, a16 = (P.b_bytes + 0u) >> 4;
      const uint32_t asub16 = TC_A_SUB_BYTES >> 4;
      TcRing full, aslot;  // this stage's shared-memory slot and A slot
      uint32_t dn = 0;     // done_bar slot of this stage
      const uint32_t seg_len = tc_seg_len(P), n_seg = tc_n_seg(P);
      // job = (tile, K segment): one accumulator each, in walk order
      for (uint32_t job = 0; job < my_tiles * n_seg && !ctl.abort_flag; ++job) {
        const uint32_t b = job % P.n_acc, u = job / P.n_acc;
        const uint32_t k0 = (job % n_seg) * seg_len, k1 = min(nk, k0 + seg_len);
        if (u >= 1 && !mbar_wait(&ctl.acc_empty[b], (u - 1) & 1, P.wait_limit)) { ctl.abort_flag = 1; break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t d = tmem + b * P.acc_cols;
        bool ok = true;
        for (uint32_t k = k0; k < k1; ++k) {
          if (!mbar_wait(&full_bar[full.i], full.ph, P.wait_limit) ||
              !mbar_wait(&aready_bar[aslot.i], aslot.ph, P.wait_limit)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          // descriptors by addition: the start-address field (address / 16,
          // 14 bits) of the ring base plus the slot's offset / 16 (shared
          // memory addresses are below 2^18, so the field does not carry)
          const uint64_t bd = d_base + full.i * st16;
          const uint32_t acc0 = (k - k0) != 0;
          if (P.a_tmem) {
            const uint32_t at = a_base + aslot.i * TC_A_COLS;
            mma_bf16_tmem_a(d, at, bd, idesc, acc0);
#pragma unroll
            for (int kk = 1; kk < TC_BK / 16; ++kk)  // 16 bf16: 8 TMEM columns of A, 2 descriptor units of B
              mma_bf16_tmem_a(d, at + 8 * kk, bd + (kk >> 2) * bh16 + 2 * (kk & 3), idesc, 1u);
          } else {
            const uint64_t ad = bd + a16;
            mma_bf16(d, ad, bd, idesc, acc0);
#pragma unroll
            for (int kk = 1; kk < TC_BK / 16; ++kk)  // 16 bf16 = 32 bytes = 2 descriptor units
              mma_bf16(d, ad + (kk >> 2) * asub16 + 2 * (kk & 3), bd + (kk >> 2) * bh16 + 2 * (kk & 3), idesc, 1u);
          }
          mma_commit(&done_bar[dn]);
          if (++dn == R) dn = 0;
          full.next(S);
          aslot.next(SA);
        }
        if (!ok) { ctl.abort_flag = 1; break; }
        mma_commit(&ctl.acc_full[b]);
      }
      // every MMA issued has completed before tensor memory is freed
      mma_commit(&ctl.drain_bar);
      if (!mbar_wait(&ctl.drain_bar, 0)) ctl.abort_flag = 1;
    }
  } else if (warp < 4 || (warp >= 6 && warp < 6 + (int)P.dec_warps - 4)) {
    // decode warps: packed 2-bit codes -> bf16 rows of A; thread = row = TMEM
    // lane of the warp's lane quarter; with 8 decode warps a warp takes one
    // half (64 individuals) of its rows
    const uint32_t row = (warp & 3) * 32 + lane;  // 0..127
    const int h0 = (P.dec_warps == 8 && warp >= 6) ? 1 : 0, nh = (P.dec_warps == 8) ? 1 : 2;
    const uint32_t sl = row / P.tpad, u = row % P.tpad;
    int value[4];  // this row's coding of the four codes (-1: a padding row, zeros)
    for (int c = 0; c < 4; ++c) value[c] = P.term_of_row[u] >= 0 ? term_value(c, P.term_of_row[u]) : -1;
    const DecTab tab = dec_tab(value);
    const uint32_t total = my_tiles * nk;
    const uint32_t a_lane = tmem + ((uint32_t)((warp & 3) * 32) << 16) + P.n_acc * P.acc_cols;
    TcRing full, aslot, done;  // this stage's slots; the done phase of stage g - SA
    for (uint32_t g = 0; g < total; ++g) {
      // A in shared memory: the TMA of this stage waited for the MMA of stage
      // g - S, the last reader of the slot.  A in TMEM: slot aslot is free
      // after the MMA of stage g - SA.  One lane waits (mbarrier polls from
      // the 32 lanes of a warp are served one lane at a time) and the warp
      // barrier after the broadcast orders the other lanes' reads after its
      // acquire.  The outcome is warp-uniform: the TMEM store is .sync.aligned.
      const bool need_slot = P.a_tmem && g >= SA;
      bool ok = false;
      if (lane == 0)
        ok = !ctl.abort_flag && mbar_wait(&full_bar[full.i], full.ph, P.wait_limit) &&
             (!need_slot || mbar_wait(&done_bar[done.i], done.ph, P.wait_limit));
      ok = __shfl_sync(0xffffffffu, ok, 0);
      __syncwarp();
      if (!ok) {
        if (lane == 0) ctl.abort_flag = 1;
        break;
      }
      if (need_slot) done.next(R);
      uint8_t* sp = smem + full.i * P.stage_bytes;
      const uint4* pk = reinterpret_cast<const uint4*>(sp + P.b_bytes + P.a_bytes + sl * (TC_BK / 4));
      const uint4 c0 = pk[0], c1 = pk[1];
      const uint32_t w[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
      if (P.a_tmem) {
        // 128 individuals = 64 columns, column q = individuals 2q, 2q + 1
        // (code byte k gives columns 2k and 2k + 1).  Decoding all of a row
        // before waiting for the A slot measured slower than this order
        // (2.24 against 1.89 ms per scan at n = 10,000, p = 500,000, 32
        // chains).
        uint32_t v[32];
        const uint32_t col = a_lane + aslot.i * TC_A_COLS;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
        for (int half = 0; half < 2; ++half) {
          if (nh == 1 && half != h0) continue;  // the other decode warp's half
#pragma unroll
          for (int kb = 0; kb < 16; ++kb) {
            const int k = 16 * half + kb;
            dec_byte((w[k >> 2] >> (8 * (k & 3))) & 0xFFu, tab, v[2 * kb], v[2 * kb + 1]);
          }
          tmem_st32(col + 32 * half, v);
        }
        tmem_wait_st();  // one wait for both halves, before the MMA is told
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      } else {
        uint8_t* a = sp + P.b_bytes;
#pragma unroll
        for (int c = 0; c < 16; ++c) {
          if (nh == 1 && (c >> 3) != h0) continue;  // the other decode warp's half
          // 16-byte chunk c of the row: individuals 8c .. 8c + 7 (code bytes
          // 2c, 2c + 1), in sub-tile c / 8 of 64 individuals
          const uint32_t h = w[c >> 1] >> ((c & 1) * 16);
          uint4 v;
          dec_byte(h & 0xFFu, tab, v.x, v.y);
          dec_byte((h >> 8) & 0xFFu, tab, v.z, v.w);
          *reinterpret_cast<uint4*>(a + (c >> 3) * TC_A_SUB_BYTES + row * 128 + (((c & 7) ^ (row & 7)) << 4)) = v;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&aready_bar[aslot.i]);
      full.next(S);
      aslot.next(SA);
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
