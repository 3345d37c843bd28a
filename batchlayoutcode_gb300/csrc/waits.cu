// waits.cu -- self-test of the library's bounded device waits.
//
// Every spin-wait in the layout kernels is bounded: the grid barrier of the
// cooperative kernels (grid_wait, 2 s of %globaltimer) and the mbarrier wait
// for tensor-core MMA completion (tc::mbar_wait, 1 s).  When a bound runs out
// the waiting thread records the site in the context's DevStatus and the
// kernel returns; the host maps the record to BL_ERR_DEVICE_TIMEOUT.  The two
// kernels below run exactly those waits with the arrival made or withheld,
// so a caller (and the tests) can see the timeout path end in an error code
// with the context still usable.  Nothing here faults or hangs: the withheld
// arrival only lets the wait run to its limit.
#include <algorithm>

#include "../../include/batchlayout_gb300.h"
#include "bl_internal.cuh"
#include "tc05.cuh"

namespace bl {
namespace {

// `missing` blocks never arrive; the others wait at the grid barrier.
__global__ void grid_wait_selftest_kernel(DevStatus *st, int missing) {
  unsigned int epoch = 0;
  if ((int)blockIdx.x < missing) return;
  grid_arrive(st, epoch);
  grid_wait(st, epoch);
}

// One mbarrier expecting one arrival; thread 0 arrives when `arrive` is set,
// then waits for the phase as the MMA epilogues do.
__global__ void mbar_wait_selftest_kernel(DevStatus *st, int arrive) {
  __shared__ uint64_t mbar;
  if (threadIdx.x == 0) tc::mbar_init(&mbar, 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    if (arrive) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_addr(&mbar)) : "memory");
    if (!tc::mbar_wait(&mbar, 0, kMmaTimeoutNs)) dev_record_error(st, DEV_TIMEOUT_MMA);
  }
}

}  // namespace
}  // namespace bl

extern "C" int bl_wait_selftest(bl_ctx *ctx, int site, int complete) try {
  using namespace bl;
  if (!ctx) return BL_ERR_ARG;
  if (site != 0 && site != 1) return bl_fail(ctx, BL_ERR_ARG, "site must be 0 (grid barrier) or 1 (mbarrier)");
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  BL_CUDA(ctx, cudaMemsetAsync(ctx->s.status, 0, sizeof(DevStatus), ctx->stream));
  if (site == 0) {
    const int grid = std::max(2, std::min(ctx->num_sms, 8));
    DevStatus *st = ctx->s.status;
    int missing = complete ? 0 : 1;
    void *args[] = {&st, &missing};
    BL_CUDA(ctx, cudaLaunchCooperativeKernel((const void *)grid_wait_selftest_kernel, dim3(grid), dim3(64), args, 0,
                                             ctx->stream));
  } else {
    mbar_wait_selftest_kernel<<<1, 32, 0, ctx->stream>>>(ctx->s.status, complete ? 1 : 0);
    BL_CUDA(ctx, cudaGetLastError());
  }
  ctx->launches++;
  BL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return bl_check_status(ctx);
} catch (...) {
  return bl_host_exception(ctx);
}
