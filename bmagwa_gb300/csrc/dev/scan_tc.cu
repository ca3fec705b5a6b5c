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
#include "tc_mainloop.cuh"

namespace {

// epilogue warps: a multiple of 4 (each TMEM lane quarter gets the same
// number); decode warps 4 or 8; the kernel is instantiated for (8, 4),
// (12, 4) and (8, 8) and the host picks
template <int EPI, int DEC>
struct TcShape {
  static constexpr int main_warps = 6 + DEC - 4;
  static constexpr int threads = 32 * (main_warps + EPI);
};
}  // namespace

template <int TC_EPI_WARPS, int TC_DEC_WARPS>
__global__ void __launch_bounds__(TcShape<TC_EPI_WARPS, TC_DEC_WARPS>::threads, 1)
bmg_scan_tc_kernel(DevConst K, TcParams P, const __grid_constant__ CUtensorMap map_b,
                   const __grid_constant__ CUtensorMap map_g)
{
  constexpr int MAIN = TcShape<TC_EPI_WARPS, TC_DEC_WARPS>::main_warps;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  // 1024-byte aligned base for the swizzled tiles; the int64 sums follow the stages
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  long long* xr_s = reinterpret_cast<long long*>(smem + P.stages * P.stage_bytes);
  __shared__ TcCtl ctl;
  __shared__ int epi_ok;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t L = K.limbs_n;
  const uint32_t ct = P.chains_tile;
  const uint32_t xs = ct + 1;  // row stride of the sums: odd, so rows fall in distinct banks
  const uint32_t my_tiles = (P.tiles > blockIdx.x) ? (P.tiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;
  const uint32_t tmem = tc_setup(P, ctl, TC_EPI_WARPS);

  if (warp < MAIN) {
    tc_main_roles(P, ctl, smem, tmem, my_tiles, map_b, map_g);
  } else {
    // epilogue warps: warp w reads TMEM lanes 32 (w % 4) .. +31 (the rows of
    // the tile); the TC_EPI_WARPS / 4 warps of a quarter split the chains
    const uint32_t e = warp - MAIN;
    const uint32_t quarter = warp & 3, part = e >> 2, nparts = TC_EPI_WARPS / 4;
    const uint32_t row = quarter * 32 + lane;
    const uint32_t c_lo = part * ct / nparts, c_hi = (part + 1) * ct / nparts;
    const uint32_t col_lo = c_lo * L, col_hi = c_hi * L;
    const uint32_t ethreads = 32 * TC_EPI_WARPS;
    const uint32_t n_seg = tc_n_seg(P);
    for (uint32_t job = 0; job < my_tiles * n_seg; ++job) {
      const uint32_t i = job / n_seg, seg = job % n_seg;
      const uint32_t tile = blockIdx.x + i * gridDim.x;
      const uint32_t snp0 = (tile % P.m_tiles) * P.snps_per_tile;
      const uint32_t chain0 = (tile / P.m_tiles) * ct;
      const uint32_t chains_here = min(ct, K.n_chains - chain0);
      const uint32_t b = job % P.n_acc, u = job / P.n_acc;
      // one warp waits; the outcome is shared so that all epilogue warps take
      // the same number of named-barrier steps
      if (e == 0) {
        bool ok = false;
        if (lane == 0) ok = !ctl.abort_flag && mbar_wait(&ctl.acc_full[b], u & 1, P.wait_limit);
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (lane == 0) {
          epi_ok = ok;
          if (!ok) ctl.abort_flag = 1;
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
          tmem_ld32(tmem + ((quarter * 32) << 16) + b * P.acc_cols + chunk, v);
#pragma unroll
          for (uint32_t q = 0; q < 32; ++q) {
            const uint32_t col = chunk + q;
            if (col < col_lo || col >= col_hi) continue;
            // |D| < 2^24: an exact float integer, converted through int32
            acc += (long long)__float2int_rn(v[q]) * (1ll << (8 * limb));
            if (++limb == L) {
              // the first K segment sets the exact sum, later ones add to it
              if (seg == 0) xr_s[row * xs + chain] = acc;
              else xr_s[row * xs + chain] += acc;
              acc = 0;
              limb = 0;
              ++chain;
            }
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&ctl.acc_empty[b]);
      named_bar_sync(1, ethreads);
      if (seg + 1 < n_seg) continue;  // the posterior waits for the tile's last segment
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
          const long long xa = xr_s[sl[0] * xs + cl[0]], xb = xr_s[sl[1] * xs + cl[1]];
          double la, lb;
          const double pa = rb_fast_pr(K, (int)c[0], j[0], xa, &la);
          const double pb = rb_fast_pr(K, (int)c[1], j[1], xb, &lb);
          const double pr[2] = {pa, pb}, lo[2] = {la, lb};
          const long long xi[2] = {xa, xb};
          for (int h = 0; h < 2; ++h) {
            if (!live[h]) continue;
            if (rb_plain(K, (int)c[h], j[h])) {
              rb_store1(K, (int)c[h], j[h], pr[h], lo[h]);
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
              if (term >= 0) xr[term] = xr_s[(sl[h] * P.tpad + q) * xs + cl[h]];
            }
            rb_epilogue(K, (int)c[h], j[h], xr);
          }
        }
      }
      named_bar_sync(1, ethreads);
    }
  }

  if (tc_teardown(ctl, tmem) && tid == 0) atomicExch(&K.ch[0].error, BMG_DERR_TIMEOUT);
}

// ----------------------------------------------------------------- host side


// dynamic shared memory of a plan: the stage ring, the int64 sums, alignment slack
static size_t tc_smem_bytes(const TcParams& P)
{
  return (size_t)P.stages * P.stage_bytes + P.xr_bytes + 1024;
}

// static shared memory of the kernel (decode tables and barriers) is below 2 KB
constexpr size_t TC_SMEM_LIMIT = 227 * 1024 - 2 * 1024;

static bool tc_plan(const DevConst* K, TcParams* P, uint32_t ct_cap, uint32_t n_acc)
{
  uint32_t T = K->n_terms;
  P->tpad = T <= 1 ? 1 : (T <= 2 ? 2 : 4);
  P->snps_per_tile = TC_BM / P->tpad;
  for (uint32_t u = 0; u < 4; ++u) P->term_of_row[u] = (u < T) ? K->term_of[u] : -1;
  const uint32_t L = K->limbs_n;
  if (K->n_pad % TC_BK != 0) return false;
  P->wait_limit = K->wait_limit;
  P->k_chunks = K->n_pad / TC_BK;
  // an FP32 accumulator of products of magnitude <= 256 stays exact over at
  // most 2^24 / 256 = 65,536 individuals: longer K ranges are closed in
  // segments of 510 stages (65,280 individuals) and added in int64
  P->seg_chunks = 65280 / TC_BK;
  P->pk_bytes = P->snps_per_tile * (TC_BK / 4);
  // widest chain tile whose accumulator fits one TMEM buffer and whose stages
  // (at least two) and sums fit shared memory
  for (uint32_t ct = std::min(std::min(K->n_chains, TC_ACC_COLS / L), std::max(1u, ct_cap)); ct >= 1; --ct) {
    P->chains_tile = ct;
    P->n_mma = ((ct * L + 15) / 16) * 16;
    if (P->n_mma > TC_ACC_COLS || P->n_mma < 16) continue;
    P->b_bytes = P->n_mma * TC_BK * 2;  // two 128-byte-swizzled boxes of 64 individuals
    tc_place_a(*P, n_acc);
    P->stage_bytes = ((P->b_bytes + P->a_bytes + P->pk_bytes + 1023) / 1024) * 1024;
    P->xr_bytes = TC_BM * (ct + 1) * 8;
    P->b_rows_per_tile = ct * L;
    for (uint32_t st = TC_MAX_STAGES; st >= 2; --st) {
      tc_set_rings(*P, st);
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

// Launch shapes the autotuner chooses between: epilogue warps, a cap on the
// chains of one N tile, and the number of TMEM accumulators (two overlap the
// epilogue's copy-out with the next tile's MMAs; one leaves ten A slots
// instead of four, a deeper decode ring).  All of them compute the same exact
// sums and the same posterior, bit for bit.
struct TcVariant {
  int epi;
  int ct_div;  // chains per tile = ceil(chains / ct_div); 0: the widest tile whose
               // accumulators (two of 192 columns) leave A room in tensor memory
  int n_acc;   // TMEM accumulators
  int dec;     // decode warps
};
static const TcVariant kTcVariants[] = {{12, 1, 2, 4}, {8, 1, 2, 4}, {12, 2, 2, 4}, {8, 2, 2, 4},
                                        {12, 1, 1, 4}, {8, 1, 1, 4}, {12, 0, 2, 4}, {8, 0, 2, 4},
                                        {8, 1, 2, 8},  {8, 1, 1, 8},  {8, 0, 2, 8}};
constexpr int kTcVariantCount = sizeof(kTcVariants) / sizeof(kTcVariants[0]);

extern "C" int bmg_scan_tc_variants() { return kTcVariantCount; }

extern "C" void bmg_scan_tc_variant_name(int v, char* buf, size_t len)
{
  if (v < 0 || v >= kTcVariantCount) v = 0;
  const char* dec = kTcVariants[v].dec == 8 ? " decode_warps=8" : "";
  if (kTcVariants[v].ct_div == 0)
    snprintf(buf, len, "epilogue_warps=%d chains_per_tile=A-in-TMEM accumulators=%d%s", kTcVariants[v].epi,
             kTcVariants[v].n_acc, dec);
  else
    snprintf(buf, len, "epilogue_warps=%d chains_per_tile=1/%d accumulators=%d%s", kTcVariants[v].epi,
             kTcVariants[v].ct_div, kTcVariants[v].n_acc, dec);
}

static uint32_t tc_cap(const DevConst* K, int v)
{
  const int d = kTcVariants[v].ct_div;
  // two accumulators and two A slots: each accumulator at most (512 - 2 x 64) / 2 columns
  if (d == 0) return std::max(1u, (TC_TMEM_COLS - 2 * TC_A_COLS) / 2 / K->limbs_n);
  return (K->n_chains + d - 1) / d;
}

// 1 when shape v would run the same plan as an earlier shape (the tuner
// skips it): the same epilogue warps, chains per tile and accumulators
extern "C" int bmg_scan_tc_variant_redundant(const DevConst* K, int v)
{
  if (v <= 0 || v >= kTcVariantCount) return 0;
  TcParams P;
  if (!tc_plan(K, &P, tc_cap(K, v), (uint32_t)kTcVariants[v].n_acc)) return 1;
  for (int u = 0; u < v; ++u) {
    TcParams Q;
    if (kTcVariants[u].epi != kTcVariants[v].epi || kTcVariants[u].dec != kTcVariants[v].dec ||
        !tc_plan(K, &Q, tc_cap(K, u), (uint32_t)kTcVariants[u].n_acc))
      continue;
    if (Q.chains_tile == P.chains_tile && Q.n_acc == P.n_acc && Q.a_tmem == P.a_tmem) return 1;
  }
  return 0;
}

extern "C" int bmg_scan_tc_supported(const DevConst* K)
{
  TcParams P;
  if (!tc_plan(K, &P, K->n_chains, 2) || !encode_fn()) return 0;
  int dev = 0, major = 0, minor = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  return (major == 10 && minor == 3) ? 1 : 0;
}

template <int EPI, int DEC>
static int tc_launch_shape(const DevConst* K, TcParams P, const CUtensorMap& mb, const CUtensorMap& mg,
                           cudaStream_t stream)
{
  P.dec_warps = DEC;
  const size_t smem = tc_smem_bytes(P);
  static size_t configured = 0;
  if (configured < smem) {
    if (cudaFuncSetAttribute(bmg_scan_tc_kernel<EPI, DEC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
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
  bmg_scan_tc_kernel<EPI, DEC><<<grid, TcShape<EPI, DEC>::threads, smem, stream>>>(*K, P, mb, mg);
  return cudaGetLastError() == cudaSuccess ? 0 : 7;
}

extern "C" int bmg_scan_tc_launch(const DevConst* K, cudaStream_t stream, int variant)
{
  if (variant < 0 || variant >= kTcVariantCount) variant = 0;
  TcParams P;
  if (!tc_plan(K, &P, tc_cap(K, variant), (uint32_t)kTcVariants[variant].n_acc)) return 1;
  auto enc = encode_fn();
  if (!enc) return 2;
  CUtensorMap mb, mg;
  {
    cuuint64_t dims[2] = {K->n_pad, (cuuint64_t)K->n_chains * K->limbs_n};
    cuuint64_t strides[1] = {(cuuint64_t)K->n_pad * 2};
    cuuint32_t box[2] = {TC_BK_SUB, P.n_mma};
    cuuint32_t es[2] = {1, 1};
    if (enc(&mb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)K->limbs, dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return 3;
  }
  {
    cuuint64_t dims[2] = {K->gs, K->p};
    cuuint64_t strides[1] = {K->gs};
    cuuint32_t box[2] = {TC_BK / 4, P.snps_per_tile};
    cuuint32_t es[2] = {1, 1};
    if (enc(&mg, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, (void*)K->geno, dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return 4;
  }
  if (kTcVariants[variant].dec == 8) return tc_launch_shape<8, 8>(K, P, mb, mg, stream);
  return kTcVariants[variant].epi == 8 ? tc_launch_shape<8, 4>(K, P, mb, mg, stream)
                                       : tc_launch_shape<12, 4>(K, P, mb, mg, stream);
}
