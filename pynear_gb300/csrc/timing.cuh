// timing.cuh — optional CUDA-event bracket around a search's dominant kernel.
#pragma once

#include "common.cuh"

namespace gn {

bool timing_on();
// Record the start/end events of the dominant kernel on stream st.
void timing_begin(cudaStream_t st, const char *kernel_name);
void timing_end(cudaStream_t st);

}  // namespace gn
