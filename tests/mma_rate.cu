// Issue rate of tcgen05.mma kind::f16 (M = 128, K = 16, bf16 x bf16 -> FP32
// in tensor memory) with the instruction forms of the scan kernels: A from
// tensor memory or from 128-byte-swizzled shared memory, B from shared
// memory, N from 64 to 256, issued back to back into one accumulator by one
// thread of one CTA per SM.  Prints one JSON line per case with the SM
// cycles per instruction (clock64 around the issue loop and the final
// commit).  The operands are zeros; only the timing is of interest.
#include <cstdio>

#include "tc_common.cuh"

__global__ void __launch_bounds__(128, 1) mma_rate_kernel(int a_tmem, int n_mma, int iters, unsigned long long* out)
{
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ uint64_t bar;
  __shared__ uint32_t tbase;
  const int tid = threadIdx.x, warp = tid >> 5;
  // B: two 64-individual sub-tiles of up to 256 rows (64 KB); A: two sub-tiles of 128 rows (32 KB)
  for (int i = tid; i < 96 * 1024 / 16; i += blockDim.x) reinterpret_cast<uint4*>(smem)[i] = make_uint4(0, 0, 0, 0);
  if (tid == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tbase)), "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tm = tbase;
  if (tid == 0) {
    const uint32_t idesc =
        (1u << 4) | (1u << 7) | (1u << 10) | (((uint32_t)n_mma >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
    uint8_t* b_s = smem;
    uint8_t* a_s = smem + 65536;
    const uint32_t b_half = (uint32_t)n_mma * 128;
    const uint32_t a_t = tm + 256;  // A in TMEM after the accumulator's 256 columns
    const long long t0 = clock64();
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int kk = 0; kk < 8; ++kk) {
        if (a_tmem)
          mma_bf16_tmem_a(tm, a_t + 8 * kk, smem_desc(b_s + (kk >> 2) * b_half) + 2 * (kk & 3), idesc, (i | kk) != 0);
        else
          mma_bf16(tm, smem_desc(a_s + (kk >> 2) * 16384) + 2 * (kk & 3),
                   smem_desc(b_s + (kk >> 2) * b_half) + 2 * (kk & 3), idesc, (i | kk) != 0);
      }
    }
    mma_commit(&bar);
    const bool ok = mbar_wait(&bar, 0);
    const long long t1 = clock64();
    out[2 * blockIdx.x] = (unsigned long long)(t1 - t0);
    out[2 * blockIdx.x + 1] = ok ? 1 : 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"(512));
  }
}

int main()
{
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = 140 * 1024;  // one CTA per SM
  cudaFuncSetAttribute(mma_rate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  unsigned long long* d = nullptr;
  cudaMalloc(&d, 2 * sizeof(unsigned long long) * sms);
  unsigned long long* h = new unsigned long long[2 * sms];
  const int iters = 2000;
  for (int a_tmem : {1, 0})
    for (int n : {64, 128, 192, 256}) {
      cudaMemset(d, 0, 2 * sizeof(unsigned long long) * sms);
      mma_rate_kernel<<<sms, 128, smem>>>(a_tmem, n, iters, d);
      const cudaError_t e = cudaDeviceSynchronize();
      if (e != cudaSuccess) {
        printf("{\"error\": \"%s\"}\n", cudaGetErrorString(e));
        return 1;
      }
      cudaMemcpy(h, d, 2 * sizeof(unsigned long long) * sms, cudaMemcpyDeviceToHost);
      double cyc = 0;
      int ok = 1;
      for (int b = 0; b < sms; ++b) {
        cyc += (double)h[2 * b];
        ok &= (int)h[2 * b + 1];
      }
      cyc /= sms;
      printf("{\"a_tmem\": %d, \"n\": %d, \"cycles_per_mma\": %.1f, \"ok\": %d}\n", a_tmem, n, cyc / (iters * 8.0), ok);
    }
  delete[] h;
  cudaFree(d);
  return 0;
}
