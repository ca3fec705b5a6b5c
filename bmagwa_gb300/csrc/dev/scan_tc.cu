// Tensor-core scan: placeholder until the tcgen05 GEMM lands; the SIMT scan
// runs meanwhile.
#include "common.cuh"

extern "C" int bmg_scan_tc_supported(const DevConst* K)
{
  (void)K;
  return 0;
}

extern "C" int bmg_scan_tc_launch(const DevConst* K, cudaStream_t stream)
{
  (void)K;
  (void)stream;
  return 1;
}
