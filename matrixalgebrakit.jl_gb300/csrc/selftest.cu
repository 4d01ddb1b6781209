// Self-test of the library's failure path for device-side waits.
//
// Every wait in the library's kernels (the cooperative panels' grid
// barriers, the tensor-core pipeline's mbarriers) is bounded: after a fixed
// number of polls it records MAK_ERR_TIMEOUT in the device status word and
// the kernel returns, so a missing arrival can never hang the GPU.  This
// entry launches co-resident CTAs that meet at the same grid barrier the
// panels use, told to expect more arrivals than there are CTAs, with a
// short poll limit: the wait must give up, report MAK_ERR_TIMEOUT and leave
// the context usable.  It has no counterpart in the reference.
#include "internal.h"

namespace mak {

__global__ void selftest_barrier_kernel(unsigned* bar, unsigned expect, long long spin_limit,
                                        int* status) {
  grid_barrier(bar, expect, status, spin_limit);
}

}  // namespace mak

using namespace mak;

extern "C" int mak_selftest_barrier(int ctas, int missing, int64_t spin_limit, void* work,
                                    size_t work_bytes, int* status, mak_stream_t stream) {
  if (ctas < 1 || ctas > num_sms()) return -1;
  if (missing < 0 || missing > 1024) return -2;
  if (spin_limit < 1 || spin_limit > kSpinLimit) return -3;
  if (work == nullptr) return -4;
  if (work_bytes < 2 * sizeof(unsigned)) return -5;
  if (status == nullptr) return -6;
  cudaStream_t st = (cudaStream_t)stream;
  unsigned* bar = (unsigned*)work;
  MAK_CUDA_TRY(cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), st));
  MAK_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), st));
  unsigned expect = (unsigned)(ctas + missing);
  long long limit = (long long)spin_limit;
  void* args[] = {&bar, &expect, &limit, &status};
  note_launch();
  MAK_CUDA_TRY(cudaLaunchCooperativeKernel((void*)selftest_barrier_kernel, dim3(ctas), dim3(32),
                                           args, 0, st));
  return 0;
}
