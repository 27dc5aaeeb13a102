// ew_diag.cu -- the give-up path of the bounded mbarrier waits, exercised
// without a GPU fault: one block waits on an mbarrier that nothing arrives
// at, with a short poll limit; the wait gives up, the block raises the
// time-out flag and returns.  Nothing is in flight, so the context stays
// usable and the next call runs normally.
#include "ew_cart.cuh"
#include "ew_internal.h"

namespace ew {
namespace {

__global__ void wait_timeout_kernel(int polls, int* err) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_barrier_init();
  }
  __syncthreads();
  // phase 0 never completes: no thread arrives and no copy is issued
  if (threadIdx.x == 0 && !mbar_wait(&bar, 0u, polls)) atomicOr(err, ERR_WAIT_TIMEOUT);
}

}  // namespace

cudaError_t launch_wait_timeout(int polls, int* err, cudaStream_t stream) {
  wait_timeout_kernel<<<1, 32, 0, stream>>>(polls, err);
  return cudaGetLastError();
}

}  // namespace ew
