// Failure-detection self test: a kernel whose bounded mbarrier wait cannot complete
// (no thread ever arrives on the barrier, no copy is in flight), so the wait runs out,
// the kernel records TP3_ERR_TIMEOUT in the context's error flag and returns.  The host
// sees the status at its next synchronising call and the context stays usable.  This
// exercises the same bounded-wait path the tensor-core kernels use around their TMA and
// MMA barriers, without faulting or hanging the device.
#include <cuda_runtime.h>

#include "ctx_internal.h"
#include "tc_prims.cuh"

namespace {

__global__ void k_wait_selftest(int* err, long long limit) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    tp3::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) tp3::mbar_wait_limit(&bar, 0u, limit, err);
}

}  // namespace

extern "C" {

int tp3_selftest_timeout(tp3_ctx* c, long long cycles) {
  if (int r = tp3::ctx_check(c)) return r;
  if (cycles < 1000 || cycles > 4000000000LL) return tp3::ctx_fail(c, TP3_ERR_ARG, "cycles out of range");
  k_wait_selftest<<<1, 32, 0, c->stream>>>(c->d_err, cycles);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "self test");
  return TP3_OK;
}

}  // extern "C"
