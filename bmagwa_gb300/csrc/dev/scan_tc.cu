// Tensor-core scan on sm_103a: D = A . B' with tcgen05.
//
//   A  (M x K): one row per (SNP, term) of the genotype coding, K = individuals;
//      values 0/1/2 as bf16, decoded in shared memory from the 2-bit PLINK codes
//   B  (N x K): the residual of every chain as L balanced base-256 digits
//      (bf16, exact), N = chains x L
//   D  (M x N): FP32 in tensor memory.  Every product is an integer of
//      magnitude <= 2 * 128 and every partial sum stays below 2^24 for n below
//      65,536, so D holds exact integers and x' r = sum_l D[., c L + l] 256^l
//      is exact: the same int64 the SIMT scan produces.
//
// Persistent, warp-specialised: one CTA per SM walks the tiles
// (tile = blockIdx.x + i gridDim.x).  Warps 0-3 decode A into the swizzled
// stage buffers, warp 4 issues the TMA loads of the packed genotype rows and
// of the residual digits, warp 5 owns tensor memory and issues the MMAs into
// one of two accumulators (2 x 256 columns), and TC_EPI_WARPS epilogue warps
// drain the other accumulator: tensor memory -> exact int64 sums in shared
// memory -> the FP64 Rao-Blackwell epilogue.  The epilogue of tile i thus
// overlaps the main loop of tile i + 1.  Every mbarrier wait is bounded; a
// timeout sets the chain error word and every role leaves its loop.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdio>

#include "rb_epilogue.cuh"

namespace {

// epilogue warps: a multiple of 4 (each TMEM lane quarter gets the same
// number); the kernel is instantiated for 8 and 12 and the host picks
template <int EPI>
struct TcShape {
  static constexpr int threads = 192 + 32 * EPI;
};
constexpr int TC_MAX_STAGES = 4;
constexpr int TC_BM = 128;          // rows of D per tile
constexpr int TC_BK = 64;           // individuals per stage (128 bytes of bf16)
constexpr uint32_t TC_ACC_COLS = 256;  // columns of one accumulator
constexpr uint32_t TC_TMEM_COLS = 512; // two accumulators
constexpr uint32_t WAIT_LIMIT = 1u << 24;

struct TcParams {
  uint32_t tpad;           // rows per SNP (terms rounded up to 1, 2 or 4)
  uint32_t snps_per_tile;  // TC_BM / tpad
  uint32_t chains_tile;    // chains per N tile
  uint32_t n_mma;          // N of the MMA (chains_tile * L rounded up to 16)
  uint32_t k_chunks;       // n_pad / TC_BK
  uint32_t stages;         // pipeline depth (2..TC_MAX_STAGES)
  uint32_t m_tiles, n_tiles, tiles;
  uint32_t xr_bytes;       // TC_BM x chains_tile int64 sums
  uint32_t stage_bytes;
  uint32_t b_bytes, a_bytes, pk_bytes;
  int32_t term_of_row[4];  // term of row u of a SNP (-1: unused)
};

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_tx(uint64_t* bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity)
{
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait: false after WAIT_LIMIT polls
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity)
{
  for (uint32_t it = 0; it < WAIT_LIMIT; ++it)
    if (mbar_try(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y)
{
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// shared-memory matrix descriptor, K-major, 128-byte swizzle, 8-row atoms of 1024 B
__device__ __forceinline__ uint64_t smem_desc(const void* p)
{
  uint64_t addr = smem_u32(p);
  uint64_t d = 0;
  d |= (addr >> 4) & 0x3FFFull;            // start address
  d |= (uint64_t)1 << 16;                  // leading byte offset (unused for this layout)
  d |= (uint64_t)(1024 >> 4) << 32;        // stride byte offset: next 8-row atom
  d |= (uint64_t)1 << 46;                  // descriptor version
  d |= (uint64_t)2 << 61;                  // 128-byte swizzle
  return d;
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void named_bar_sync(uint32_t id, uint32_t threads)
{
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v)
{
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
        "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
        "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
        "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace

template <int TC_EPI_WARPS>
__global__ void __launch_bounds__(TcShape<TC_EPI_WARPS>::threads, 1)
bmg_scan_tc_kernel(DevConst K, TcParams P, const __grid_constant__ CUtensorMap map_b,
                   const __grid_constant__ CUtensorMap map_g)
{
  constexpr int TC_THREADS = TcShape<TC_EPI_WARPS>::threads;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  // 1024-byte aligned base for the swizzled tiles; the int64 sums follow the stages
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  long long* xr_s = reinterpret_cast<long long*>(smem + P.stages * P.stage_bytes);
  __shared__ uint64_t full_bar[TC_MAX_STAGES], aready_bar[TC_MAX_STAGES], empty_bar[TC_MAX_STAGES];
  __shared__ uint64_t acc_full[2], acc_empty[2], drain_bar;
  __shared__ uint32_t tmem_base_sh;
  __shared__ volatile int abort_flag;
  __shared__ int epi_ok;
  __shared__ uint2 lut[4][256];  // per term: byte -> 4 bf16 values

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t L = K.limbs_n;
  const uint32_t nk = P.k_chunks, S = P.stages;
  const uint32_t ct = P.chains_tile;
  const uint32_t my_tiles = (P.tiles > blockIdx.x) ? (P.tiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;

  // decode tables: bf16 bit patterns of 0, 1, 2 are 0x0000, 0x3F80, 0x4000
  for (int e = tid; e < 4 * 256; e += TC_THREADS) {
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
    for (uint32_t st = 0; st < S; ++st) {
      mbar_init(&full_bar[st], 1);
      mbar_init(&aready_bar[st], 4);
      mbar_init(&empty_bar[st], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], TC_EPI_WARPS);
    }
    mbar_init(&drain_bar, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 5) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)),
                 "r"(TC_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base_sh;

  if (warp == 4) {
    if (lane == 0) {
      // TMA producer: packed genotype rows and residual digits of each stage
      uint32_t issued = 0;
      for (uint32_t i = 0; i < my_tiles && !abort_flag; ++i) {
        const uint32_t tile = blockIdx.x + i * gridDim.x;
        const uint32_t snp0 = (tile % P.m_tiles) * P.snps_per_tile;
        const uint32_t chain0 = (tile / P.m_tiles) * ct;
        for (uint32_t k = 0; k < nk; ++k) {
          const uint32_t g = i * nk + k, st = g % S;
          if (g >= S && !mbar_wait(&empty_bar[st], ((g / S) - 1) & 1)) { abort_flag = 1; break; }
          uint8_t* sp = smem + st * P.stage_bytes;
          mbar_arrive_tx(&full_bar[st], P.b_bytes + P.pk_bytes);
          tma_load_2d(sp, &map_b, &full_bar[st], (int)(k * TC_BK), (int)(chain0 * L));
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
      for (uint32_t i = 0; i < my_tiles && !abort_flag; ++i) {
        const uint32_t b = i & 1, u = i >> 1;
        if (u >= 1 && !mbar_wait(&acc_empty[b], (u - 1) & 1)) { abort_flag = 1; break; }
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
        if (!ok) { abort_flag = 1; break; }
        mma_commit(&acc_full[b]);
      }
      // every MMA issued has completed before tensor memory is freed
      mma_commit(&drain_bar);
      if (!mbar_wait(&drain_bar, 0)) abort_flag = 1;
    }
  } else if (warp < 4) {
    // decode warps: packed 2-bit codes -> bf16 rows of the swizzled A tile
    const uint32_t row = tid;  // 0..127
    const uint32_t sl = row / P.tpad, u = row % P.tpad;
    const int term = P.term_of_row[u];
    const uint32_t total = my_tiles * nk;
    for (uint32_t g = 0; g < total; ++g) {
      if (abort_flag) break;
      const uint32_t st = g % S, par = (g / S) & 1;
      if (!mbar_wait(&full_bar[st], par)) { abort_flag = 1; break; }
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
  } else {
    // epilogue warps: warp w reads TMEM lanes 32 (w % 4) .. +31 (the rows of
    // the tile); the TC_EPI_WARPS / 4 warps of a quarter split the chains
    const uint32_t e = warp - 6;
    const uint32_t quarter = warp & 3, part = e >> 2, nparts = TC_EPI_WARPS / 4;
    const uint32_t row = quarter * 32 + lane;
    const uint32_t c_lo = part * ct / nparts, c_hi = (part + 1) * ct / nparts;
    const uint32_t col_lo = c_lo * L, col_hi = c_hi * L;
    const uint32_t ethreads = 32 * TC_EPI_WARPS;
    for (uint32_t i = 0; i < my_tiles; ++i) {
      const uint32_t tile = blockIdx.x + i * gridDim.x;
      const uint32_t snp0 = (tile % P.m_tiles) * P.snps_per_tile;
      const uint32_t chain0 = (tile / P.m_tiles) * ct;
      const uint32_t chains_here = min(ct, K.n_chains - chain0);
      const uint32_t b = i & 1, u = i >> 1;
      // one warp waits; the verdict is shared so that all epilogue warps take
      // the same number of named-barrier steps
      if (e == 0) {
        bool ok = false;
        if (lane == 0) ok = !abort_flag && mbar_wait(&acc_full[b], u & 1);
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (lane == 0) {
          epi_ok = ok;
          if (!ok) abort_flag = 1;
        }
      }
      named_bar_sync(1, ethreads);
      if (!epi_ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // exact int64 sums: x' r of chain c = sum_l D[row, c L + l] 256^l
      {
        uint32_t chain = c_lo, limb = 0;
        long long acc = 0;
        for (uint32_t chunk = col_lo & ~31u; chunk < col_hi; chunk += 32) {
          float v[32];
          tmem_ld32(tmem + ((quarter * 32) << 16) + b * TC_ACC_COLS + chunk, v);
#pragma unroll
          for (uint32_t q = 0; q < 32; ++q) {
            const uint32_t col = chunk + q;
            if (col < col_lo || col >= col_hi) continue;
            // |D| < 2^24: an exact float integer, converted through int32
            acc += (long long)__float2int_rn(v[q]) * (1ll << (8 * limb));
            if (++limb == L) {
              xr_s[row * ct + chain] = acc;
              acc = 0;
              limb = 0;
              ++chain;
            }
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&acc_empty[b]);
      named_bar_sync(1, ethreads);
      // one unit per (SNP, chain), SNPs fastest so that a warp's stores to
      // the chain-major running means are contiguous; two units per step
      const uint32_t units = P.snps_per_tile * chains_here;
      const bool fast = rb_fast_ok(K);
      for (uint32_t ua = e * 32 + lane; ua < units; ua += 2 * ethreads) {
        uint64_t j[2];
        uint32_t c[2], sl[2], cl[2];
        bool live[2];
        for (int h = 0; h < 2; ++h) {
          const uint32_t uu = ua + h * ethreads;
          const bool in_tile = uu < units;
          sl[h] = in_tile ? uu % P.snps_per_tile : 0;
          cl[h] = in_tile ? uu / P.snps_per_tile : 0;
          j[h] = (uint64_t)snp0 + sl[h];
          c[h] = chain0 + cl[h];
          live[h] = in_tile && j[h] < K.p && K.rb[c[h]].do_scan;
          if (j[h] >= K.p) j[h] = snp0;  // a valid address for the unused half
        }
        if (fast) {
          const long long xa = xr_s[sl[0] * ct + cl[0]], xb = xr_s[sl[1] * ct + cl[1]];
          const double pa = rb_fast_pr(K, (int)c[0], j[0], xa);
          const double pb = rb_fast_pr(K, (int)c[1], j[1], xb);
          const double pr[2] = {pa, pb};
          const long long xi[2] = {xa, xb};
          for (int h = 0; h < 2; ++h) {
            if (!live[h]) continue;
            if (!in_model(K, (int)c[h], j[h])) {
              rb_store1(K, (int)c[h], j[h], pr[h]);
            } else {
              long long xr[4] = {0, 0, 0, 0};
              xr[K.types[0]] = xi[h];
              rb_epilogue(K, (int)c[h], j[h], xr);
            }
          }
        } else {
          for (int h = 0; h < 2; ++h) {
            if (!live[h]) continue;
            long long xr[4] = {0, 0, 0, 0};
            for (uint32_t q = 0; q < P.tpad; ++q) {
              const int term = P.term_of_row[q];
              if (term >= 0) xr[term] = xr_s[(sl[h] * P.tpad + q) * ct + cl[h]];
            }
            rb_epilogue(K, (int)c[h], j[h], xr);
          }
        }
      }
      named_bar_sync(1, ethreads);
    }
  }

  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (tid == 0 && abort_flag) atomicExch(&K.ch[0].error, BMG_DERR_TIMEOUT);
  if (warp == 5) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS));
  }
}

// ----------------------------------------------------------------- host side

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// dynamic shared memory of a plan: the stage ring, the int64 sums, alignment slack
static size_t tc_smem_bytes(const TcParams& P)
{
  return (size_t)P.stages * P.stage_bytes + P.xr_bytes + 1024;
}

// static shared memory of the kernel (decode tables and barriers) is below 9 KB
constexpr size_t TC_SMEM_LIMIT = 227 * 1024 - 9 * 1024;

static bool tc_plan(const DevConst* K, TcParams* P, uint32_t ct_cap)
{
  uint32_t T = K->n_terms;
  P->tpad = T <= 1 ? 1 : (T <= 2 ? 2 : 4);
  P->snps_per_tile = TC_BM / P->tpad;
  for (uint32_t u = 0; u < 4; ++u) P->term_of_row[u] = (u < T) ? K->term_of[u] : -1;
  const uint32_t L = K->limbs_n;
  if (K->n_pad % TC_BK != 0 || K->n >= 65536) return false;  // exact FP32 sums need n < 2^16
  P->k_chunks = K->n_pad / TC_BK;
  P->a_bytes = TC_BM * 128;
  P->pk_bytes = P->snps_per_tile * 16;
  // widest chain tile whose accumulator fits one TMEM buffer and whose stages
  // (at least two) and sums fit shared memory
  for (uint32_t ct = std::min(std::min(K->n_chains, TC_ACC_COLS / L), std::max(1u, ct_cap)); ct >= 1; --ct) {
    P->chains_tile = ct;
    P->n_mma = ((ct * L + 15) / 16) * 16;
    if (P->n_mma > TC_ACC_COLS || P->n_mma < 16) continue;
    P->b_bytes = P->n_mma * 128;
    P->stage_bytes = ((P->b_bytes + P->a_bytes + P->pk_bytes + 1023) / 1024) * 1024;
    P->xr_bytes = TC_BM * ct * 8;
    for (uint32_t st = TC_MAX_STAGES; st >= 2; --st) {
      P->stages = st;
      if (tc_smem_bytes(*P) <= TC_SMEM_LIMIT) {
        P->m_tiles = (uint32_t)((K->p + P->snps_per_tile - 1) / P->snps_per_tile);
        P->n_tiles = (K->n_chains + ct - 1) / ct;
        P->tiles = P->m_tiles * P->n_tiles;
        return true;
      }
    }
  }
  return false;
}

// Launch shapes the autotuner chooses between: epilogue warps and a cap on
// the chains of one N tile (0: as many as one accumulator holds).  All of
// them compute the same exact sums and the same posterior, bit for bit.
struct TcVariant {
  int epi;
  int ct_div;  // chains per tile = ceil(chains / ct_div)
};
static const TcVariant kTcVariants[] = {{12, 1}, {8, 1}, {12, 2}, {8, 2}};
constexpr int kTcVariantCount = sizeof(kTcVariants) / sizeof(kTcVariants[0]);

extern "C" int bmg_scan_tc_variants() { return kTcVariantCount; }

extern "C" void bmg_scan_tc_variant_name(int v, char* buf, size_t len)
{
  if (v < 0 || v >= kTcVariantCount) v = 0;
  snprintf(buf, len, "epilogue_warps=%d chains_per_tile=1/%d", kTcVariants[v].epi, kTcVariants[v].ct_div);
}

static uint32_t tc_cap(const DevConst* K, int v)
{
  const int d = kTcVariants[v].ct_div;
  return (K->n_chains + d - 1) / d;
}

extern "C" int bmg_scan_tc_supported(const DevConst* K)
{
  TcParams P;
  if (!tc_plan(K, &P, K->n_chains) || !encode_fn()) return 0;
  int dev = 0, major = 0, minor = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  return (major == 10 && minor == 3) ? 1 : 0;
}

template <int EPI>
static int tc_launch_shape(const DevConst* K, const TcParams& P, const CUtensorMap& mb, const CUtensorMap& mg,
                           cudaStream_t stream)
{
  const size_t smem = tc_smem_bytes(P);
  static size_t configured = 0;
  if (configured < smem) {
    if (cudaFuncSetAttribute(bmg_scan_tc_kernel<EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return 6;
    configured = smem;
  }
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  const unsigned grid = (unsigned)std::min<uint32_t>(P.tiles, (uint32_t)sms);
  bmg_scan_tc_kernel<EPI><<<grid, TcShape<EPI>::threads, smem, stream>>>(*K, P, mb, mg);
  return cudaGetLastError() == cudaSuccess ? 0 : 7;
}

extern "C" int bmg_scan_tc_launch(const DevConst* K, cudaStream_t stream, int variant)
{
  if (variant < 0 || variant >= kTcVariantCount) variant = 0;
  TcParams P;
  if (!tc_plan(K, &P, tc_cap(K, variant))) return 1;
  auto enc = encode_fn();
  if (!enc) return 2;
  CUtensorMap mb, mg;
  {
    cuuint64_t dims[2] = {K->n_pad, (cuuint64_t)K->n_chains * K->limbs_n};
    cuuint64_t strides[1] = {(cuuint64_t)K->n_pad * 2};
    cuuint32_t box[2] = {TC_BK, P.n_mma};
    cuuint32_t es[2] = {1, 1};
    if (enc(&mb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)K->limbs, dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return 3;
  }
  {
    cuuint64_t dims[2] = {K->gs, K->p};
    cuuint64_t strides[1] = {K->gs};
    cuuint32_t box[2] = {16, P.snps_per_tile};
    cuuint32_t es[2] = {1, 1};
    if (enc(&mg, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, (void*)K->geno, dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return 4;
  }
  return kTcVariants[variant].epi == 8 ? tc_launch_shape<8>(K, P, mb, mg, stream)
                                       : tc_launch_shape<12>(K, P, mb, mg, stream);
}
