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

// Device address of a page-locked host buffer mapped into the current
// device's address space, or null (pageable memory, or pinned for another
// device without the portable flag).
void *mapped_view(const void *host);
// dst(i, j) = src(i, j), i < rows, j < cols, column-major, by SM loads and
// stores (one launch on `st`): the host<->device path for mapped host blocks.
cudaError_t copy_cols(double *dst, long long ldd, const double *src, long long lds, int rows, int cols,
                      cudaStream_t st);

// Record the status of an entry point for hsr_last_status() on the calling
// thread, and the CUDA error behind an HSR_ERR_CUDA (cudaSuccess otherwise
// leaves the recorded error as it is).  Returns `status`.
int record_status(int status, cudaError_t cuda_error);

}  // namespace hsr
