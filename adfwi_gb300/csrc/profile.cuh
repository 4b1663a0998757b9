// Kernel launch accounting: every launch site of the library brackets its launch with
// prof_before / prof_after. Launches are always counted; when a timed profiling session is
// active, CUDA events recorded on the launch stream measure each launch's device time.
#pragma once
#include <cuda_runtime.h>

namespace adfwi {

enum KernelClass : int {
  kAcFwdStep = 0,
  kAcAdjStep,
  kElFwdStep,
  kElAdjStep,
  kAux,
  kNumKernelClasses
};

int prof_before(int cls, cudaStream_t st);
void prof_after(int cls, cudaStream_t st, int token);

}  // namespace adfwi
