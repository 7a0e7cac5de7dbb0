// genfft/gb300_common.h -- helpers shared by the drop-in header
// (genfft/fft.h) and the backend for the reference's factory seam
// (genfft/gb300_backend.h): the error type, status checks, and the staging
// of host buffers through device memory.
#ifndef GENFFT_GB300_COMMON_H
#define GENFFT_GB300_COMMON_H

#include <cuda_runtime.h>

#include <cstddef>
#include <stdexcept>
#include <string>

#include "../genfft_gb300.h"

namespace genfft {

// thrown where the reference asserts (unsupported sizes, failed calls)
struct gb300_error : std::runtime_error {
    gfft_status status;
    gb300_error(gfft_status s, const std::string &what) : std::runtime_error(what), status(s) {}
};

namespace gb300 {

template <class T>
constexpr int dtype()
{
    static_assert(sizeof(T) == 4 || sizeof(T) == 8, "genfft::gb300 supports float and double");
    return sizeof(T) == 4 ? GFFT_F32 : GFFT_F64;
}

inline void check(gfft_status s)
{
    if (s != GFFT_OK) throw gb300_error(s, std::string(gfft_status_string(s)) + ": " + gfft_last_error());
}

inline void check_cuda(cudaError_t e)
{
    if (e != cudaSuccess) throw gb300_error(GFFT_ERR_CUDA, cudaGetErrorString(e));
}

inline bool on_device(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Device staging buffer owned by a transform object (grown on demand).
class Buffer {
public:
    Buffer() = default;
    Buffer(const Buffer &) = delete;
    Buffer &operator=(const Buffer &) = delete;
    Buffer(Buffer &&o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr, o.n_ = 0; }
    ~Buffer() { if (p_) cudaFree(p_); }
    void *get(size_t bytes)
    {
        if (bytes > n_) {
            if (p_) cudaFree(p_);
            p_ = nullptr;
            n_ = 0;
            check_cuda(cudaMalloc(&p_, bytes));
            n_ = bytes;
        }
        return p_;
    }

private:
    void *p_ = nullptr;
    size_t n_ = 0;
};

// Runs `op(dev_out, dev_in)` on device pointers, staging host buffers:
// in_bytes are copied in, out_bytes copied back, then synchronised.
template <class Op>
void staged(void *out, size_t out_bytes, const void *in, size_t in_bytes, Buffer &bo, Buffer &bi, Op op,
            bool out_preload = false)
{
    const bool din = on_device(in), dout = on_device(out);
    const void *dev_in = in;
    void *dev_out = out;
    if (!din) {
        void *b = bi.get(in_bytes);
        check_cuda(cudaMemcpy(b, in, in_bytes, cudaMemcpyHostToDevice));
        dev_in = b;
    }
    if (!dout) {
        dev_out = (in == out && !din) ? const_cast<void *>(dev_in) : bo.get(out_bytes);
        if (out_preload && dev_out != dev_in) check_cuda(cudaMemcpy(dev_out, out, out_bytes, cudaMemcpyHostToDevice));
    }
    op(dev_out, dev_in);
    check_cuda(cudaDeviceSynchronize());
    if (!dout) check_cuda(cudaMemcpy(out, dev_out, out_bytes, cudaMemcpyDeviceToHost));
}

}  // namespace gb300
}  // namespace genfft

#endif  // GENFFT_GB300_COMMON_H
