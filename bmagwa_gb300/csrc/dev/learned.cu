// The learned part of the add proposal (no reference counterpart).
//
// A 16 -> 128 -> 128 -> 1 MLP (ReLU) maps per-SNP features of a chain's
// state to a logit of inclusion:
//   f0  RB log posterior odds of the last scan / 16 (clamped to +-4)
//   f1  SNP in the model
//   f2  max |corr| to the model's SNPs within +-LD_WINDOW positions
//   f3  minor allele frequency, f4 heterozygote fraction
//   f5  f0^2, f6 = 1, f7..f15 = 0
// It is trained during burn-in on the chains' adaptive proposal p_proposal
// (the running mean of the RB probabilities, src/sampler.cpp:739-810) with a
// binary cross-entropy loss, and each chain's candidate table holds the
// topk SNPs of highest logit with weight sigmoid(logit).  The move kernel
// mixes it into the add proposal with weight `mix` and evaluates both the
// forward and the backward probabilities as the mixture, so MH stays exact;
// after burn-in nothing here runs and the proposal is fixed.
//
// Kernels: the windowed LD feature (popcounts of the packed codes), the
// forward pass over every (chain, SNP) on tcgen05 (both layers as MMAs with
// the weights resident in shared memory and the accumulators in TMEM), the
// candidate tables (deterministic top-k by histogram and ordered
// compaction), and training on the CUDA cores: forward and backward of a
// minibatch in FP32 with the gradient accumulated in global memory, then Adam.
#include <cuda_bf16.h>

#include <algorithm>

#include "common.cuh"
#include "tc_common.cuh"

namespace {

constexpr int LD_WINDOW = 32;
constexpr int TRAIN_ROWS = 128;  // rows per training CTA (one per thread)
constexpr int LDP = MLP_H + 1;   // padded row stride of the training buffers
constexpr int TOPK_BINS = 4096;  // logit histogram over [-32, 32)

__device__ __forceinline__ void mlp_features(const DevConst& K, uint32_t c, uint64_t j, float* f)
{
  const size_t cj = (size_t)c * K.p + j;
  const double lo = K.p_lml ? K.p_lml[cj] : 0.0;
  float l = (float)(lo * (1.0 / 16.0));
  l = fminf(fmaxf(l, -4.0f), 4.0f);
  const bool in = (K.inbits[(size_t)c * ((K.p + 31) / 32) + (j >> 5)] >> (j & 31)) & 1u;
  const DevPheno& P = K.ph[K.pheno_of[c]];
  const float n = (float)P.n;
  const float n1 = (float)P.cnt[2 * j], n2 = (float)P.cnt[2 * j + 1];
  const float af = (n1 + 2.0f * n2) / (2.0f * n);
  f[0] = l;
  f[1] = in ? 1.0f : 0.0f;
  f[2] = K.lrn.maxcorr[cj];
  f[3] = fminf(af, 1.0f - af);
  f[4] = n1 / n;
  f[5] = l * l;
  f[6] = 1.0f;
#pragma unroll
  for (int k = 7; k < MLP_F; ++k) f[k] = 0.0f;
}

__device__ __forceinline__ uint32_t bf16x2(float lo, float hi)
{
  return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(lo)) |
         ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(hi)) << 16);
}

// deterministic SNP index of a random training row
__device__ __forceinline__ uint64_t mix64(uint64_t a, uint64_t b, uint64_t d)
{
  uint64_t x = a * 0x9E3779B97F4A7C15ull ^ (b + 0x632BE59BD9B4E019ull) * 0xBF58476D1CE4E5B9ull ^
               d * 0x94D049BB133111EBull;
  x ^= x >> 31;
  x *= 0xD6E8FEB86659FD93ull;
  x ^= x >> 32;
  return x;
}

__device__ __forceinline__ int logit_bin(float x)
{
  int b = (int)floorf((x + 32.0f) * (TOPK_BINS / 64.0f));
  return b < 0 ? 0 : (b >= TOPK_BINS ? TOPK_BINS - 1 : b);
}

}  // namespace

// Parameters: He-normal weights from the Philox stream (key 0x6d6c70), zero
// biases, zero optimiser state, bf16 copies; the Adam step counter at 0.
extern "C" __global__ void bmg_mlp_init_kernel(DevConst K, int32_t* adam_t)
{
  const DevLearned& L = K.lrn;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < MLP_NPAR; i += gridDim.x * blockDim.x) {
    double w = 0;
    if (i < MLP_OB1) w = bmg_normal_at(0x6d6c70u, 1u, (uint64_t)i) * sqrt(2.0 / MLP_F);
    else if (i >= MLP_OW2 && i < MLP_OB2) w = bmg_normal_at(0x6d6c70u, 2u, (uint64_t)i) * sqrt(2.0 / MLP_H);
    else if (i >= MLP_OW3 && i < MLP_OB3) w = bmg_normal_at(0x6d6c70u, 3u, (uint64_t)i) * sqrt(1.0 / MLP_H);
    L.theta[i] = (float)w;
    L.grad[i] = 0.0f;
    L.adam_m[i] = 0.0f;
    L.adam_v[i] = 0.0f;
    if (i < MLP_OB1) L.w1b[i] = __bfloat16_as_ushort(__float2bfloat16_rn((float)w));
    if (i >= MLP_OW2 && i < MLP_OB2) L.w2b[i - MLP_OW2] = __bfloat16_as_ushort(__float2bfloat16_rn((float)w));
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *adam_t = 0;
}

// f2: for each model SNP m of chain c and each SNP s within +-LD_WINDOW
// positions, |corr| of their additive codings from popcounts of the codes;
// maxcorr[c][s] keeps the largest (non-negative floats order as their bits).
extern "C" __global__ void __launch_bounds__(128) bmg_mlp_ld_kernel(DevConst K)
{
  const uint32_t mi = blockIdx.x, c = blockIdx.y;
  const DevModel& M = K.cur[c];
  if ((int)mi >= M.k) return;
  const uint64_t m = M.loci[mi];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const DevPheno& P = K.ph[K.pheno_of[c]];
  const int32_t* cnt = P.cnt;
  const double n = P.n;
  const double sm = cnt[2 * m] + 2.0 * cnt[2 * m + 1], qm = cnt[2 * m] + 4.0 * cnt[2 * m + 1];
  const double vm = qm / n - (sm / n) * (sm / n);
  const uint64_t* rm = reinterpret_cast<const uint64_t*>(K.geno + m * K.gs);
  const unsigned nw64 = K.gs / 8;
  const uint64_t m5 = 0x5555555555555555ull;
  for (int d = -LD_WINDOW + warp; d <= LD_WINDOW; d += 4) {
    const long long s = (long long)m + d;
    if (d == 0 || s < 0 || s >= (long long)K.p) continue;
    const uint64_t* rs = reinterpret_cast<const uint64_t*>(K.geno + (uint64_t)s * K.gs);
    long long xy = 0;
    for (unsigned w = lane; w < nw64; w += 32) {
      const uint64_t x = rm[w], y = rs[w];
      const uint64_t mk = P.mask2 ? P.mask2[w] : m5;
      const uint64_t xh = (x >> 1) & mk, xl = x & m5, yh = (y >> 1) & mk, yl = y & m5;
      const uint64_t Hx = xh & ~xl, Rx = xh & xl, Hy = yh & ~yl, Ry = yh & yl;
      xy += __popcll(Hx & Hy) + 2 * __popcll(Hx & Ry) + 2 * __popcll(Rx & Hy) + 4 * __popcll(Rx & Ry);
    }
    xy = warp_sum_ll(xy);
    if (lane == 0) {
      const double ss = cnt[2 * s] + 2.0 * cnt[2 * s + 1], qs = cnt[2 * s] + 4.0 * cnt[2 * s + 1];
      const double vs = qs / n - (ss / n) * (ss / n);
      const double cov = (double)xy / n - (sm / n) * (ss / n);
      const float r = (vm > 0 && vs > 0) ? (float)fabs(cov / sqrt(vm * vs)) : 0.0f;
      atomicMax(reinterpret_cast<int*>(&K.lrn.maxcorr[(size_t)c * K.p + s]), __float_as_int(fminf(r, 1.0f)));
    }
  }
}

// Forward pass over every (chain, SNP) row on tcgen05.  One CTA of 128
// threads (one per row of a 128-row tile): the threads write their row's
// features as bf16 into a 128-byte-swizzled A tile, one MMA (K = 16) gives
// layer 1 in TMEM columns 0-127, the threads apply bias and ReLU and write
// the activations as the next A operand (two 64-wide K blocks), eight MMAs
// give layer 2 in columns 128-255, and the threads finish with the output
// unit.  W1 and W2 stay in shared memory for the whole launch.
extern "C" __global__ void __launch_bounds__(128, 1) bmg_mlp_infer_kernel(DevConst K)
{
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* a1 = sm;           // 128 rows x 128 B: features (K = 64, zero beyond 16)
  uint8_t* w1 = sm + 16384;   // 128 rows x 128 B: W1 rows (K = 64, zero beyond 16)
  uint8_t* h1 = sm + 32768;   // 2 K blocks x 128 rows x 128 B: layer-1 activations
  uint8_t* w2 = sm + 65536;   // 2 K blocks x 128 rows x 128 B: W2 rows
  __shared__ uint64_t bar, drain;
  __shared__ uint32_t tmem_sh;
  __shared__ int ok_sh;
  __shared__ float b1[MLP_H], b2[MLP_H], w3[MLP_H];
  const DevLearned& L = K.lrn;
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int i = tid; i < 16384 / 16; i += 128) {
    reinterpret_cast<uint4*>(a1)[i] = make_uint4(0, 0, 0, 0);
    reinterpret_cast<uint4*>(w1)[i] = make_uint4(0, 0, 0, 0);
  }
  __syncthreads();
  {
    const int u = tid;  // unit u = row u of W1 and W2 (the B operands are N x K, K-major)
    const uint4* s1 = reinterpret_cast<const uint4*>(L.w1b + u * MLP_F);
    for (int c16 = 0; c16 < 2; ++c16) *reinterpret_cast<uint4*>(w1 + u * 128 + ((c16 ^ (u & 7)) << 4)) = s1[c16];
    const uint4* s2 = reinterpret_cast<const uint4*>(L.w2b + u * MLP_H);
    for (int kb = 0; kb < 2; ++kb)
      for (int c16 = 0; c16 < 8; ++c16)
        *reinterpret_cast<uint4*>(w2 + kb * 16384 + u * 128 + ((c16 ^ (u & 7)) << 4)) = s2[kb * 8 + c16];
    b1[u] = L.theta[MLP_OB1 + u];
    b2[u] = L.theta[MLP_OB2 + u];
    w3[u] = L.theta[MLP_OW3 + u];
  }
  const float b3 = L.theta[MLP_OB3];
  if (tid == 0) {
    mbar_init(&bar, 1);
    mbar_init(&drain, 1);
    ok_sh = 1;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_sh)),
                 "r"(256u));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_sh;
  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(MLP_H >> 3) << 17) | ((128u >> 4) << 24);
  const uint64_t rows = (uint64_t)K.n_chains * K.p;
  const uint64_t tiles = (rows + 127) / 128;
  uint32_t phase = 0;
  bool issued = false;
  for (uint64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const uint64_t row = tile * 128 + tid;
    const bool valid = row < rows;
    float f[MLP_F];
    if (valid) mlp_features(K, (uint32_t)(row / K.p), row % K.p, f);
    else
      for (int k = 0; k < MLP_F; ++k) f[k] = 0.0f;
    for (int c16 = 0; c16 < 2; ++c16)
      *reinterpret_cast<uint4*>(a1 + tid * 128 + ((c16 ^ (tid & 7)) << 4)) =
          make_uint4(bf16x2(f[8 * c16], f[8 * c16 + 1]), bf16x2(f[8 * c16 + 2], f[8 * c16 + 3]),
                     bf16x2(f[8 * c16 + 4], f[8 * c16 + 5]), bf16x2(f[8 * c16 + 6], f[8 * c16 + 7]));
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      mma_bf16(tmem, smem_desc(a1), smem_desc(w1), idesc, 0);
      mma_commit(&bar);
      issued = true;
      if (!mbar_wait(&bar, phase)) ok_sh = 0;
    }
    phase ^= 1;
    __syncthreads();
    if (!ok_sh) break;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // layer 1: bias, ReLU, bf16 into the swizzled A operand of layer 2
    for (int cb = 0; cb < MLP_H; cb += 32) {
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + cb, v);
      const int kb = cb >> 6;
      for (int c16 = 0; c16 < 4; ++c16) {
        const int k0 = cb + 8 * c16;
        float h[8];
        for (int q = 0; q < 8; ++q) h[q] = fmaxf(v[8 * c16 + q] + b1[k0 + q], 0.0f);
        const int chunk = (k0 & 63) >> 3;
        *reinterpret_cast<uint4*>(h1 + kb * 16384 + tid * 128 + ((chunk ^ (tid & 7)) << 4)) =
            make_uint4(bf16x2(h[0], h[1]), bf16x2(h[2], h[3]), bf16x2(h[4], h[5]), bf16x2(h[6], h[7]));
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int kb = 0; kb < 2; ++kb)
        for (int kk = 0; kk < 4; ++kk)
          mma_bf16(tmem + MLP_H, smem_desc(h1 + kb * 16384) + 2 * kk, smem_desc(w2 + kb * 16384) + 2 * kk, idesc,
                   (kb | kk) != 0);
      mma_commit(&bar);
      if (!mbar_wait(&bar, phase)) ok_sh = 0;
    }
    phase ^= 1;
    __syncthreads();
    if (!ok_sh) break;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // layer 2: bias, ReLU, the output unit
    float acc = b3;
    for (int cb = 0; cb < MLP_H; cb += 32) {
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + MLP_H + cb, v);
      for (int q = 0; q < 32; ++q) acc += w3[cb + q] * fmaxf(v[q] + b2[cb + q], 0.0f);
    }
    if (valid) L.logit[row] = acc;
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
  }
  if (tid == 0 && issued) {
    // every MMA issued has completed before tensor memory is freed
    mma_commit(&drain);
    if (!mbar_wait(&drain, 0)) ok_sh = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (tid == 0 && !ok_sh) atomicExch(&K.ch[0].error, BMG_DERR_TIMEOUT);
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256u));
  }
}

// Candidate table of chain blockIdx.x: the topk SNPs of highest logit (ties
// of the threshold bin broken by SNP order), in ascending SNP order, with
// weight sigmoid(logit).
extern "C" __global__ void __launch_bounds__(1024) bmg_mlp_topk_kernel(DevConst K)
{
  __shared__ uint32_t hist[TOPK_BINS];
  __shared__ uint32_t scan_a[1024], scan_b[1024];
  __shared__ double red[32];
  __shared__ int thr_sh;
  __shared__ uint32_t above_sh;
  const DevLearned& L = K.lrn;
  const uint32_t c = blockIdx.x, T = L.topk;
  const int tid = threadIdx.x, nth = blockDim.x;
  const uint64_t p = K.p;
  const float* lg = L.logit + (size_t)c * p;
  for (int b = tid; b < TOPK_BINS; b += nth) hist[b] = 0;
  __syncthreads();
  for (uint64_t j = tid; j < p; j += nth) atomicAdd(&hist[logit_bin(lg[j])], 1u);
  __syncthreads();
  if (tid == 0) {
    uint32_t cum = 0;
    int b = TOPK_BINS - 1;
    for (; b >= 0; --b) {
      if (cum + hist[b] >= T) break;
      cum += hist[b];
    }
    thr_sh = b;  // -1: fewer than T SNPs in all
    above_sh = cum;
  }
  __syncthreads();
  const int thr = thr_sh;
  const uint32_t take_eq = (thr >= 0) ? T - above_sh : 0;
  const uint64_t per = (p + nth - 1) / nth;
  const uint64_t j0 = min(p, (uint64_t)tid * per), j1 = min(p, j0 + per);
  uint32_t n_hi = 0, n_eq = 0;
  for (uint64_t j = j0; j < j1; ++j) {
    const int b = logit_bin(lg[j]);
    n_hi += (b > thr);
    n_eq += (b == thr);
  }
  // exclusive prefix of the threshold-bin counts, in SNP order
  scan_a[tid] = n_eq;
  __syncthreads();
  for (int o = 1; o < nth; o <<= 1) {
    const uint32_t v = tid >= o ? scan_a[tid - o] : 0;
    __syncthreads();
    scan_a[tid] += v;
    __syncthreads();
  }
  const uint32_t eq_before = scan_a[tid] - n_eq;
  const uint32_t eq_take = (eq_before >= take_eq) ? 0 : min(n_eq, take_eq - eq_before);
  const uint32_t sel = n_hi + eq_take;
  scan_b[tid] = sel;
  __syncthreads();
  for (int o = 1; o < nth; o <<= 1) {
    const uint32_t v = tid >= o ? scan_b[tid - o] : 0;
    __syncthreads();
    scan_b[tid] += v;
    __syncthreads();
  }
  uint32_t slot = scan_b[tid] - sel;
  const uint32_t total = scan_b[nth - 1];
  uint32_t eq_seen = 0;
  double s_sum = 0;
  for (uint64_t j = j0; j < j1; ++j) {
    const int b = logit_bin(lg[j]);
    bool take = b > thr;
    if (b == thr) take = (eq_seen++ < eq_take);
    if (take) {
      const double w = 1.0 / (1.0 + exp(-(double)lg[j]));
      L.t_snp[(size_t)c * T + slot] = (uint32_t)j;
      L.t_s[(size_t)c * T + slot] = w;
      s_sum += w;
      ++slot;
    }
  }
  for (uint32_t q = total + tid; q < T; q += nth) {
    L.t_snp[(size_t)c * T + q] = 0xFFFFFFFFu;
    L.t_s[(size_t)c * T + q] = 0.0;
  }
  s_sum = warp_sum_d(s_sum);
  if ((tid & 31) == 0) red[tid >> 5] = s_sum;
  __syncthreads();
  if (tid == 0) {
    double t = 0;
    for (int w = 0; w < nth / 32; ++w) t += red[w];
    L.t_sum[c] = t;
    L.t_n[c] = total;
  }
}

// One minibatch of the MLP's training: rows (chain blockIdx.y) are the
// chain's candidates and random SNPs; target p_proposal; loss the mean
// binary cross-entropy over all rows of all chains.  Forward and backward in
// FP32 on the CUDA cores, one row per thread, the layer products through
// shared memory; the gradient goes to L.grad (atomic adds).
extern "C" __global__ void __launch_bounds__(TRAIN_ROWS, 1)
bmg_mlp_train_kernel(DevConst K, const int32_t* adam_t, const uint32_t* rows, uint32_t n_rows)
{
  extern __shared__ __align__(16) float tsm[];
  float* W2 = tsm;                    // [128][LDP]   W2[u][v]
  float* H1 = W2 + MLP_H * LDP;       // [row][LDP]   layer-1 activations
  float* B2 = H1 + TRAIN_ROWS * LDP;  // [row][LDP]   layer-2 activations, then dZ2, then dZ1
  float* W1 = B2 + TRAIN_ROWS * LDP;  // [128][16]
  float* F = W1 + MLP_H * MLP_F;      // [row][16]
  float* misc = F + TRAIN_ROWS * MLP_F;
  float* b1 = misc;                   // [128]
  float* b2 = b1 + MLP_H;             // [128]
  float* w3 = b2 + MLP_H;             // [128]
  float* dlg = w3 + MLP_H;            // [row]
  const DevLearned& L = K.lrn;
  const int tid = threadIdx.x;
  const uint32_t c = blockIdx.y, T = L.topk;
  for (int i = tid; i < MLP_H * MLP_H; i += TRAIN_ROWS) W2[(i / MLP_H) * LDP + (i % MLP_H)] = L.theta[MLP_OW2 + i];
  for (int i = tid; i < MLP_H * MLP_F; i += TRAIN_ROWS) W1[i] = L.theta[MLP_OW1 + i];
  b1[tid] = L.theta[MLP_OB1 + tid];
  b2[tid] = L.theta[MLP_OB2 + tid];
  w3[tid] = L.theta[MLP_OW3 + tid];
  const float b3 = L.theta[MLP_OB3];
  // this thread's row: candidate r of the chain's table, else a random SNP;
  // or row r of an explicit (chain, SNP) list
  const uint32_t r = blockIdx.x * TRAIN_ROWS + tid;
  uint32_t cr = c;
  uint64_t j;
  bool active = true;
  if (rows) {
    active = r < n_rows;
    cr = active ? rows[2 * r] : 0;
    j = active ? rows[2 * r + 1] : 0;
  } else {
    const uint32_t nt = L.t_n[c];
    j = (r < nt && r < T) ? L.t_snp[(size_t)c * T + r] : mix64(c, r, (uint64_t)*adam_t) % K.p;
  }
  float f[MLP_F];
  mlp_features(K, cr, j, f);
  for (int k = 0; k < MLP_F; ++k) F[tid * MLP_F + k] = f[k];
  const float t = (float)K.p_prop[(size_t)cr * K.p + K.pos[j]];
  __syncthreads();
  // forward
  for (int u = 0; u < MLP_H; ++u) {
    float z = b1[u];
    for (int k = 0; k < MLP_F; ++k) z += W1[u * MLP_F + k] * f[k];
    H1[tid * LDP + u] = fmaxf(z, 0.0f);
  }
  float lg = b3;
  for (int u = 0; u < MLP_H; ++u) {
    float z = b2[u];
    for (int v = 0; v < MLP_H; ++v) z += W2[u * LDP + v] * H1[tid * LDP + v];
    const float h = fmaxf(z, 0.0f);
    B2[tid * LDP + u] = h;
    lg += w3[u] * h;
  }
  const float rows_total = rows ? (float)n_rows : (float)(gridDim.x * TRAIN_ROWS) * (float)gridDim.y;
  const float sg = 1.0f / (1.0f + expf(-lg));
  const float d = active ? (sg - t) / rows_total : 0.0f;  // d loss / d logit
  dlg[tid] = d;
  __syncthreads();
  // output unit: thread u sums over the rows; dZ2 = d * w3 * [h2 > 0]
  {
    const int u = tid;
    float gw3 = 0, gb3 = 0;
    for (int q = 0; q < TRAIN_ROWS; ++q) {
      gw3 += dlg[q] * B2[q * LDP + u];
      gb3 += dlg[q];
    }
    atomicAdd(&L.grad[MLP_OW3 + u], gw3);
    if (u == 0) atomicAdd(&L.grad[MLP_OB3], gb3);
  }
  __syncthreads();
  for (int u = 0; u < MLP_H; ++u) {
    const float h = B2[tid * LDP + u];
    B2[tid * LDP + u] = h > 0.0f ? d * w3[u] : 0.0f;
  }
  __syncthreads();
  // layer 2: dW2[u][v] = sum_q dZ2[q][u] H1[q][v], db2[u] = sum_q dZ2[q][u]
  {
    const int u = tid;
    float gb = 0;
    for (int q = 0; q < TRAIN_ROWS; ++q) gb += B2[q * LDP + u];
    atomicAdd(&L.grad[MLP_OB2 + u], gb);
    for (int v = 0; v < MLP_H; ++v) {
      float g = 0;
      for (int q = 0; q < TRAIN_ROWS; ++q) g += B2[q * LDP + u] * H1[q * LDP + v];
      atomicAdd(&L.grad[MLP_OW2 + u * MLP_H + v], g);
    }
  }
  // dH1[q][v] = sum_u dZ2[q][u] W2[u][v]; dZ1 = dH1 * [h1 > 0] (this thread's row)
  float dz1[MLP_H];
  for (int v = 0; v < MLP_H; ++v) {
    float g = 0;
    for (int u = 0; u < MLP_H; ++u) g += B2[tid * LDP + u] * W2[u * LDP + v];
    dz1[v] = H1[tid * LDP + v] > 0.0f ? g : 0.0f;
  }
  __syncthreads();
  for (int v = 0; v < MLP_H; ++v) B2[tid * LDP + v] = dz1[v];
  __syncthreads();
  // layer 1: dW1[v][k] = sum_q dZ1[q][v] F[q][k], db1[v] = sum_q dZ1[q][v]
  {
    const int v = tid;
    float gb = 0;
    float g[MLP_F];
    for (int k = 0; k < MLP_F; ++k) g[k] = 0;
    for (int q = 0; q < TRAIN_ROWS; ++q) {
      const float dz = B2[q * LDP + v];
      gb += dz;
      for (int k = 0; k < MLP_F; ++k) g[k] += dz * F[q * MLP_F + k];
    }
    atomicAdd(&L.grad[MLP_OB1 + v], gb);
    for (int k = 0; k < MLP_F; ++k) atomicAdd(&L.grad[MLP_OW1 + v * MLP_F + k], g[k]);
  }
}

// Adam step on the accumulated gradient (which it clears), bf16 copies for
// the forward kernel, the step counter advanced.
extern "C" __global__ void bmg_mlp_adam_kernel(DevConst K, int32_t* adam_t, float lr)
{
  const DevLearned& L = K.lrn;
  const float b1 = 0.9f, b2 = 0.999f;
  const int t = *adam_t + 1;
  const float c1 = 1.0f - powf(b1, (float)t), c2 = 1.0f - powf(b2, (float)t);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < MLP_NPAR; i += gridDim.x * blockDim.x) {
    const float g = L.grad[i];
    const float m = b1 * L.adam_m[i] + (1.0f - b1) * g;
    const float v = b2 * L.adam_v[i] + (1.0f - b2) * g * g;
    L.adam_m[i] = m;
    L.adam_v[i] = v;
    const float w = L.theta[i] - lr * (m / c1) / (sqrtf(v / c2) + 1e-8f);
    L.theta[i] = w;
    L.grad[i] = 0.0f;
    if (i < MLP_OB1) L.w1b[i] = __bfloat16_as_ushort(__float2bfloat16_rn(w));
    if (i >= MLP_OW2 && i < MLP_OB2) L.w2b[i - MLP_OW2] = __bfloat16_as_ushort(__float2bfloat16_rn(w));
  }
}

extern "C" __global__ void bmg_mlp_step_kernel(int32_t* adam_t)
{
  if (threadIdx.x == 0) *adam_t += 1;
}

// ----------------------------------------------------------------- host side

extern "C" size_t bmg_mlp_train_smem()
{
  return sizeof(float) * ((size_t)MLP_H * LDP + 2 * (size_t)TRAIN_ROWS * LDP + MLP_H * MLP_F +
                          TRAIN_ROWS * MLP_F + 3 * MLP_H + TRAIN_ROWS);
}

extern "C" cudaError_t bmg_mlp_init(const DevConst* K, int32_t* adam_t, cudaStream_t s)
{
  bmg_mlp_init_kernel<<<(MLP_NPAR + 255) / 256, 256, 0, s>>>(*K, adam_t);
  return cudaGetLastError();
}

// The refresh of the learned proposal: LD feature, `steps` optimiser steps,
// forward pass over every (chain, SNP), candidate tables.
extern "C" cudaError_t bmg_mlp_refresh(const DevConst* K, uint32_t km, int steps, float lr, int32_t* adam_t,
                                       cudaStream_t s)
{
  cudaError_t e = cudaMemsetAsync(K->lrn.maxcorr, 0, sizeof(float) * K->n_chains * K->p, s);
  if (e != cudaSuccess) return e;
  bmg_mlp_ld_kernel<<<dim3(km, K->n_chains), 128, 0, s>>>(*K);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  static bool configured = false;
  if (!configured) {
    e = cudaFuncSetAttribute(bmg_mlp_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)bmg_mlp_train_smem());
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(bmg_mlp_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 98304 + 1024);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  const uint32_t blocks = (2 * K->lrn.topk + TRAIN_ROWS - 1) / TRAIN_ROWS;
  for (int st = 0; st < steps; ++st) {
    bmg_mlp_train_kernel<<<dim3(blocks, K->n_chains), TRAIN_ROWS, bmg_mlp_train_smem(), s>>>(*K, adam_t, nullptr, 0);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    bmg_mlp_adam_kernel<<<(MLP_NPAR + 255) / 256, 256, 0, s>>>(*K, adam_t, lr);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    bmg_mlp_step_kernel<<<1, 32, 0, s>>>(adam_t);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const uint64_t tiles = ((uint64_t)K->n_chains * K->p + 127) / 128;
  const unsigned grid = (unsigned)std::min<uint64_t>(tiles, (uint64_t)std::max(1, sms) * 2);
  bmg_mlp_infer_kernel<<<grid, 128, 98304 + 1024, s>>>(*K);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  bmg_mlp_topk_kernel<<<K->n_chains, 1024, 0, s>>>(*K);
  return cudaGetLastError();
}

// features of every (chain, SNP) row, for inspection
extern "C" __global__ void bmg_mlp_features_kernel(DevConst K, float* out)
{
  const uint64_t rows = (uint64_t)K.n_chains * K.p;
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < rows; r += (uint64_t)gridDim.x * blockDim.x) {
    float f[MLP_F];
    mlp_features(K, (uint32_t)(r / K.p), r % K.p, f);
    for (int k = 0; k < MLP_F; ++k) out[r * MLP_F + k] = f[k];
  }
}

extern "C" cudaError_t bmg_mlp_features(const DevConst* K, float* out, cudaStream_t s)
{
  bmg_mlp_features_kernel<<<1024, 256, 0, s>>>(*K, out);
  return cudaGetLastError();
}

// The gradient of the mean BCE over an explicit list of (chain, SNP) rows
// (device array of n pairs) into K->lrn.grad (cleared first), no step.
extern "C" cudaError_t bmg_mlp_grad(const DevConst* K, const int32_t* adam_t, const uint32_t* rows, uint32_t n,
                                    cudaStream_t s)
{
  cudaError_t e = cudaMemsetAsync(K->lrn.grad, 0, sizeof(float) * MLP_NPAR, s);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(bmg_mlp_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)bmg_mlp_train_smem());
  if (e != cudaSuccess) return e;
  bmg_mlp_train_kernel<<<dim3((n + TRAIN_ROWS - 1) / TRAIN_ROWS, 1), TRAIN_ROWS, bmg_mlp_train_smem(), s>>>(
      *K, adam_t, rows, n);
  return cudaGetLastError();
}

// forward pass of the current parameters over the current state (logits only)
extern "C" cudaError_t bmg_mlp_forward(const DevConst* K, cudaStream_t s)
{
  cudaError_t e = cudaFuncSetAttribute(bmg_mlp_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 98304 + 1024);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const uint64_t tiles = ((uint64_t)K->n_chains * K->p + 127) / 128;
  const unsigned grid = (unsigned)std::min<uint64_t>(tiles, (uint64_t)std::max(1, sms) * 2);
  bmg_mlp_infer_kernel<<<grid, 128, 98304 + 1024, s>>>(*K);
  return cudaGetLastError();
}
