// Per-SNP precomputed sums without any allocation.
//
// bmg_precompute_noalloc() serves callers that cannot call cudaMalloc: code
// that runs inside another framework's memory pool, a host that hands out
// only pre-registered buffers, or a stream that is being captured.  It
// computes what bmg_get_precomputed() returns for a context (the per-SNP sums
// and centred second moments of every allowed term), from genotypes the
// caller already holds on the device, into a device buffer the caller owns.
//
// Its only working memory is the file-scope array below.  The array exists
// once per device that loads the library and stays allocated until the
// process exits.  Every call shares it, so two calls that overlap on the GPU
// (different streams, or different host threads on one device) race on it;
// calls on one stream, one after another, are safe.
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>

#include <cuda_runtime.h>

#include "bmg.h"
#include "bmg_internal.h"

// per SNP: #heterozygous, #homozygous-alternate, #missing after the recode
#define BMG_NOALLOC_MAX_SNPS (1u << 20)

static __device__ __align__(256) int32_t g_noalloc_counts[3 * BMG_NOALLOC_MAX_SNPS];

namespace {

constexpr int kMaxDevices = 64;
// device address of the working array, per device; host threads that make
// their first call at the same time look it up twice and store the same value
std::atomic<int32_t*> g_counts_addr[kMaxDevices];

bmg_status fail(bmg_status st, const char* msg)
{
  bmg_host::set_thread_error(std::string("bmg_precompute_noalloc: ") + msg);
  return st;
}

// one warp per SNP; rows have the PLINK stride ceil(n/4) and need no padding
__global__ void noalloc_count_kernel(const uint8_t* packed, uint64_t n, uint64_t p, int recode,
                                     int32_t* counts)
{
  const int lane = threadIdx.x & 31;
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  const uint64_t stride = (n + 3) / 4;
  for (uint64_t j = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); j < p; j += warps) {
    const uint8_t* row = packed + j * stride;
    unsigned c0 = 0, c1 = 0, c2 = 0, c3 = 0;
    for (uint64_t i = lane; i < n; i += 32) {
      int code = (row[i >> 2] >> ((i & 3) * 2)) & 3;
      c0 += code == 0;
      c1 += code == 2;
      c2 += code == 3;
      c3 += code == 1;
    }
    for (int o = 16; o > 0; o >>= 1) {
      c0 += __shfl_xor_sync(0xffffffffu, c0, o);
      c1 += __shfl_xor_sync(0xffffffffu, c1, o);
      c2 += __shfl_xor_sync(0xffffffffu, c2, o);
      c3 += __shfl_xor_sync(0xffffffffu, c3, o);
    }
    if (lane == 0) {
      // minor-allele recode (src/data.cpp:324-339): swap homozygote counts
      long long ngenos = (long long)n - c3, macount = (long long)c1 + 2ll * c2;
      bool swap = recode && macount > ngenos;
      counts[3 * j] = (int32_t)c1;
      counts[3 * j + 1] = (int32_t)(swap ? c0 : c2);
      counts[3 * j + 2] = (int32_t)c3;
    }
  }
}

// the reference's layout (src/precomputed_snp_covariances.hpp:95-131)
__global__ void noalloc_pre_kernel(const int32_t* counts, uint64_t n, uint64_t p, int allow_mask, int ah,
                                   int offset, double* out, int* missing_flag)
{
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < p; j += (uint64_t)gridDim.x * blockDim.x) {
    double n1 = counts[3 * j], n2 = counts[3 * j + 1];
    if (counts[3 * j + 2] != 0) atomicExch(missing_flag, 1);
    double* loc = out + j * (uint64_t)offset;
    for (int t = 0; t < 4; ++t) {
      if (!((allow_mask >> t) & 1)) continue;
      double ch = (t == 3) ? 0 : 1, cr = (t == 0) ? 2 : (t == 1 ? 0 : 1);
      double xs = ch * n1 + cr * n2;
      double xx = ch * ch * n1 + cr * cr * n2;
      *loc++ = xs;
      *loc++ = xx - xs * xs / (double)n;
    }
    if (ah) {
      double as = n1 + 2 * n2;
      *loc = n1 - as * n1 / (double)n;
    }
  }
}

}  // namespace

extern "C" bmg_status bmg_precompute_noalloc(const uint8_t* d_packed, uint64_t n, uint64_t p, int32_t recode,
                                             const int32_t* types, uint32_t n_types, double* d_out,
                                             uint32_t* offset_out, int32_t* d_flag, void* stream)
{
  if (!d_packed || !types || !d_out || !d_flag) return fail(BMG_EINVAL, "null argument");
  if (n == 0 || p == 0 || n_types == 0 || n_types > 5) return fail(BMG_EINVAL, "n, p and n_types (1..5) must be positive");
  // more SNPs than the fixed working array holds
  if (p > BMG_NOALLOC_MAX_SNPS) return fail(BMG_EINVAL, "p above 2^20 SNPs, the size of the working array");
  // the per-SNP counts are 32-bit
  if (n > 0x7FFFFFFFull) return fail(BMG_EINVAL, "n above 2^31 - 1 individuals");
  int allow_types[5] = {0, 0, 0, 0, 0};
  int allow_mask = 0;
  for (uint32_t t = 0; t < n_types; ++t) {
    if (types[t] < 0 || types[t] > 4) return fail(BMG_EINVAL, "effect type outside 0..4");
    allow_types[types[t]] = 1;
    if (types[t] == BMG_TYPE_AH) allow_mask |= 3;
    else allow_mask |= 1 << types[t];
  }
  const int ah = allow_types[4], a = allow_types[0], h = allow_types[1];
  const int offset = 2 * (int)n_types + (ah ? 1 : 0) * (1 + ((a && h) ? -2 : 0) + ((a || h) ? 0 : 2));
  if (offset_out) *offset_out = (uint32_t)offset;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return fail(BMG_ECUDA, "no current device");
  int32_t* counts = g_counts_addr[dev].load(std::memory_order_acquire);
  if (!counts) {
    // once per device, with that device current: the device address of the
    // working array (its host-side name is not a device address)
    void* addr = nullptr;
    if (cudaGetSymbolAddress(&addr, g_noalloc_counts) != cudaSuccess)
      return fail(BMG_ECUDA, "cudaGetSymbolAddress of the working array failed");
    counts = static_cast<int32_t*>(addr);
    g_counts_addr[dev].store(counts, std::memory_order_release);
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (cudaMemsetAsync(d_flag, 0, sizeof(int32_t), s) != cudaSuccess) return fail(BMG_ECUDA, "cudaMemsetAsync failed");
  unsigned blocks = (unsigned)((p + 7) / 8 < 152 * 16 ? (p + 7) / 8 : 152 * 16);
  noalloc_count_kernel<<<blocks, 256, 0, s>>>(d_packed, n, p, recode, counts);
  noalloc_pre_kernel<<<blocks, 256, 0, s>>>(counts, n, p, allow_mask, ah, offset, d_out, d_flag);
  return cudaGetLastError() == cudaSuccess ? BMG_OK : fail(BMG_ECUDA, "kernel launch failed");
}
