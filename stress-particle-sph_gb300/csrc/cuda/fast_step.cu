// fast_step.cu -- FP32 compensated form of the SPS step (placeholder until implemented).
#include <cuda_runtime.h>

#include <stdexcept>

#include "ctx.cuh"

namespace sps {

int launch_fast_step(Ctx& c) {
  (void)c;
  throw std::runtime_error("the FP32 fast form is not implemented yet");
}

}  // namespace sps
