// internal.h -- declarations shared by the host planner (api.cpp) and the
// kernel translation units.  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <functional>
#include <string>

#include "../../include/genfft_gb300.h"

namespace gfft {

// thrown inside the library, converted to a status at the C boundary
struct Error {
    gfft_status status;
    std::string msg;
};
[[noreturn]] void fail(gfft_status st, const std::string &msg);
void set_last_error(const char *msg);  // the thread's gfft_last_error() text
void check_cuda(cudaError_t e, const char *what);
// GFFT_ERR_ARCH unless the current device is an sm_103 (GB300)
void check_device();

// ---- fused single-kernel C2C (c2c_fused.cu) ------------------------------
struct FusedC2CArgs {
    const void *in;
    void *out;
    long long batch;
    long long idist, odist;       // elements between transforms
    long long istride, ostride;   // elements between points
    const void *tw;               // device twiddle table for (dtype, logn)
    double scale = 1.0;           // applied to every output (norm= scaling)
};
int fused_max_logn(int dtype);
size_t fused_twiddle_count(int dtype, int logn);              // complex elements
void fused_twiddle_fill(int dtype, int logn, void *host_buf);  // writes that many
cudaError_t launch_fused_c2c(int dtype, int logn, int inverse, const FusedC2CArgs &a,
                             cudaStream_t st);

// Opts fn in to `smem` bytes of dynamic shared memory when that is above
// the 48 KB default, once per (device, function).
cudaError_t ensure_smem(const void *fn, size_t smem);

// Launches fn as a programmatic dependent of the previous kernel on the
// stream: its CTAs may start while that kernel's last wave drains, and the
// kernel (which begins with pdl_enter()) waits for that kernel's completion
// before it touches global memory.  GFFT_PDL=0: an ordinary launch.
cudaError_t launch_pdl(const void *fn, dim3 grid, dim3 block, void **args, size_t smem, cudaStream_t st);

// ---- device twiddle cache (api.cpp) --------------------------------------
// Returns a device pointer to the table made by `fill` (count complex
// elements of dtype), cached per (device, key) for the process lifetime.
const void *cached_table(const std::string &key, int dtype, size_t count,
                         const std::function<void(void *)> &fill);

}  // namespace gfft
