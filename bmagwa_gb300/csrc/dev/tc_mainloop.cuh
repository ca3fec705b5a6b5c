// The main loop shared by the tensor-core scans: D = A . B' on tcgen05 with
// A the 0/1/2 codings of 128 (SNP, term) rows, decoded in shared memory from
// the packed 2-bit codes, and B any bf16 matrix of n_pad columns (the
// residual digits of the RB scan, the model columns of the Schur scan).
//
// A persistent CTA walks the tiles (tile = blockIdx.x + i gridDim.x, m tile =
// tile % m_tiles).  Warps 0-3 decode A into the 128-byte-swizzled stage
// buffers, warp 4 issues the TMA loads of the packed rows and of B, warp 5
// owns 512 TMEM columns and issues the MMAs of tile i into accumulator i & 1;
// the kernel's own epilogue warps (from warp 6 on) drain the other one and
// hand it back through acc_empty.  Every wait is bounded; a timeout sets
// abort_flag and every role leaves its loop after draining its own
// asynchronous work.
#ifndef BMG_TC_MAINLOOP_CUH_
#define BMG_TC_MAINLOOP_CUH_

#include "common.cuh"
#include "tc_common.cuh"

namespace {

constexpr int TC_MAX_STAGES = 4;
constexpr int TC_BM = 128;          // rows of D per tile
constexpr int TC_BK = 64;           // individuals per stage (128 bytes of bf16)
constexpr uint32_t TC_ACC_COLS = 256;  // columns of one accumulator
constexpr uint32_t TC_TMEM_COLS = 512; // two accumulators

struct TcParams {
  uint32_t tpad;           // rows per SNP (terms rounded up to 1, 2 or 4)
  uint32_t snps_per_tile;  // TC_BM / tpad
  uint32_t chains_tile;    // chains per N tile
  uint32_t n_mma;          // N of the MMA (chains_tile * L rounded up to 16)
  uint32_t k_chunks;       // n_pad / TC_BK
  uint32_t stages;         // pipeline depth (2..TC_MAX_STAGES)
  uint32_t m_tiles, n_tiles, tiles;
  uint32_t xr_bytes;       // epilogue shared memory after the stages
  uint32_t b_rows_per_tile;  // B rows between consecutive N tiles
  uint32_t stage_bytes;
  uint32_t b_bytes, a_bytes, pk_bytes;
  int32_t term_of_row[4];  // term of row u of a SNP (-1: unused)
};


// barriers and flags of one CTA
struct TcCtl {
  uint64_t full_bar[TC_MAX_STAGES], aready_bar[TC_MAX_STAGES], empty_bar[TC_MAX_STAGES];
  uint64_t acc_full[2], acc_empty[2], drain_bar;
  uint32_t tmem_base;
  volatile int abort_flag;
};

// All threads: decode tables, barriers, tensor memory.  Returns the TMEM base.
__device__ __forceinline__ uint32_t tc_setup(const TcParams& P, TcCtl& ctl, uint2 (*lut)[256], int threads,
                                             int epi_warps)
{
  const int tid = threadIdx.x, warp = tid >> 5;
  // decode tables: bf16 bit patterns of 0, 1, 2 are 0x0000, 0x3F80, 0x4000
  for (int e = tid; e < 4 * 256; e += threads) {
    int term = e >> 8, byte = e & 255;
    uint16_t h[4];
    for (int q = 0; q < 4; ++q) {
      int code = (byte >> (2 * q)) & 3;
      int v = term_value(code, term);
      h[q] = v == 0 ? 0 : (v == 1 ? 0x3F80 : 0x4000);
    }
    lut[term][byte] = make_uint2((uint32_t)h[0] | ((uint32_t)h[1] << 16), (uint32_t)h[2] | ((uint32_t)h[3] << 16));
  }
  if (tid == 0) {
    for (uint32_t st = 0; st < P.stages; ++st) {
      mbar_init(&ctl.full_bar[st], 1);
      mbar_init(&ctl.aready_bar[st], 4);
      mbar_init(&ctl.empty_bar[st], 1);
    }
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
__device__ __forceinline__ void tc_main_roles(const TcParams& P, TcCtl& ctl, uint2 (*lut)[256], uint8_t* smem,
                                              uint32_t tmem, uint32_t my_tiles, const CUtensorMap& map_b,
                                              const CUtensorMap& map_g)
{
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t nk = P.k_chunks, S = P.stages;
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
        const uint32_t d = tmem + b * TC_ACC_COLS;
        bool ok = true;
        for (uint32_t k = 0; k < nk; ++k) {
          const uint32_t g = i * nk + k, st = g % S, par = (g / S) & 1;
          if (!mbar_wait(&full_bar[st], par) || !mbar_wait(&aready_bar[st], par)) { ok = false; break; }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          uint8_t* sp = smem + st * P.stage_bytes;
          uint64_t bdesc = smem_desc(sp), adesc = smem_desc(sp + P.b_bytes);
#pragma unroll
          for (int kk = 0; kk < TC_BK / 16; ++kk)  // 16 bf16 = 32 bytes = 2 descriptor units
            mma_bf16(d, adesc + 2 * kk, bdesc + 2 * kk, idesc, (k | kk) != 0);
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
    // decode warps: packed 2-bit codes -> bf16 rows of the swizzled A tile
    const uint32_t row = tid;  // 0..127
    const uint32_t sl = row / P.tpad, u = row % P.tpad;
    const int term = P.term_of_row[u];
    const uint32_t total = my_tiles * nk;
    for (uint32_t g = 0; g < total; ++g) {
      if (ctl.abort_flag) break;
      const uint32_t st = g % S, par = (g / S) & 1;
      if (!mbar_wait(&full_bar[st], par)) { ctl.abort_flag = 1; break; }
      uint8_t* sp = smem + st * P.stage_bytes;
      uint8_t* a = sp + P.b_bytes;
      const uint8_t* pk = sp + P.b_bytes + P.a_bytes + sl * 16;
      uint4 bytes = *reinterpret_cast<const uint4*>(pk);
      uint32_t w[4] = {bytes.x, bytes.y, bytes.z, bytes.w};
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        uint32_t two = (w[c >> 1] >> ((c & 1) * 16)) & 0xFFFF;
        uint2 lo = (term >= 0) ? lut[term][two & 255] : make_uint2(0, 0);
        uint2 hi = (term >= 0) ? lut[term][two >> 8] : make_uint2(0, 0);
        uint4 v = make_uint4(lo.x, lo.y, hi.x, hi.y);
        *reinterpret_cast<uint4*>(a + row * 128 + ((c ^ (row & 7)) << 4)) = v;
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&aready_bar[st]);
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
