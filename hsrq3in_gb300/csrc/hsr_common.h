// hsr_common.h -- host helpers shared by the orchestration files.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

namespace hsr {

// 2-D FP64 tensor map (TMA descriptor): inner extent `inner` (contiguous),
// outer extent `outer`, pitch `ld` elements, box {bx, by}; reads outside the
// tensor return 0.  Encoded through the runtime's driver entry point.
bool encode_tensor_map(CUtensorMap *m, const double *base, unsigned long long inner, unsigned long long outer,
                       unsigned long long ld, unsigned bx, unsigned by);

// True while per-kernel-class timing (hsr_set_kernel_timing) is on for the
// calling thread.
bool kernel_timing_enabled();

inline long long round_up_ll(long long x, long long m) { return (x + m - 1) / m * m; }

}  // namespace hsr
