// tiles_host.cpp -- registry and launchers of the tile kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <set>
#include <tuple>

#include "internal.h"
#include "tiles_registry.h"

namespace gfft {

namespace {
std::map<std::tuple<int, int, int, int>, TileKernel> &registry()
{
    static std::map<std::tuple<int, int, int, int>, TileKernel> r;
    return r;
}
std::mutex &reg_mu()
{
    static std::mutex m;
    return m;
}

// large dynamic shared memory needs an opt-in per (device, function)
cudaError_t ensure_smem(const void *fn, size_t smem)
{
    if (smem <= 48 * 1024) return cudaSuccess;
    static std::mutex mu;
    static std::set<std::pair<int, const void *>> done;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    if (done.count({dev, fn})) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) done.insert({dev, fn});
    return e;
}
}  // namespace

void tile_register(int dtype, int variant, int logl, int c, const TileKernel &k)
{
    std::lock_guard<std::mutex> lk(reg_mu());
    registry()[std::make_tuple(dtype, variant, logl, c)] = k;
}

const TileKernel *tile_find(int dtype, int variant, int logl, int c)
{
    std::lock_guard<std::mutex> lk(reg_mu());
    auto it = registry().find(std::make_tuple(dtype, variant, logl, c));
    return it == registry().end() ? nullptr : &it->second;
}

int tile_widest(int dtype, int variant, int logl, int max_c)
{
    std::lock_guard<std::mutex> lk(reg_mu());
    int best = 0;
    for (auto &kv : registry()) {
        if (std::get<0>(kv.first) == dtype && std::get<1>(kv.first) == variant &&
            std::get<2>(kv.first) == logl && std::get<3>(kv.first) <= max_c)
            best = std::max(best, std::get<3>(kv.first));
    }
    return best;
}

cudaError_t launch_colpass(const TileKernel &k, int inverse, long long tiles, long long nbatch,
                           const void *in, void *out, long long ncols, long long ld_in, long long ld_out,
                           long long idist, long long odist, const void *tw, const void *tw_lo,
                           const void *tw_hi, int lo_bits, unsigned nmask, cudaStream_t st)
{
    const void *fn = inverse ? k.inv : k.fwd;
    cudaError_t e = ensure_smem(fn, k.smem);
    if (e != cudaSuccess) return e;
    void *args[] = {(void *)&in,    (void *)&out,   (void *)&ncols, (void *)&ld_in,
                    (void *)&ld_out, (void *)&idist, (void *)&odist, (void *)&tw,
                    (void *)&tw_lo, (void *)&tw_hi, (void *)&lo_bits, (void *)&nmask};
    for (long long b0 = 0; b0 < nbatch; b0 += 65535) {
        const long long nb = std::min<long long>(65535, nbatch - b0);
        const void *inp = static_cast<const char *>(in) + b0 * idist * (long long)k.elem_bytes;
        void *outp = static_cast<char *>(out) + b0 * odist * (long long)k.elem_bytes;
        args[0] = (void *)&inp;
        args[1] = (void *)&outp;
        e = cudaLaunchKernel(fn, dim3((unsigned)tiles, (unsigned)nb), dim3(k.threads), args, k.smem, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_rowpass(const TileKernel &k, int inverse, long long tiles, long long nbatch,
                           const void *in, void *out, long long nrows, long long ld_in, long long ostride,
                           long long idist, long long odist, const void *tw, cudaStream_t st)
{
    const void *fn = inverse ? k.inv : k.fwd;
    cudaError_t e = ensure_smem(fn, k.smem);
    if (e != cudaSuccess) return e;
    for (long long b0 = 0; b0 < nbatch; b0 += 65535) {
        const long long nb = std::min<long long>(65535, nbatch - b0);
        const void *inp = static_cast<const char *>(in) + b0 * idist * (long long)k.elem_bytes;
        void *outp = static_cast<char *>(out) + b0 * odist * (long long)k.elem_bytes;
        void *args[] = {(void *)&inp,   (void *)&outp,  (void *)&nrows, (void *)&ld_in,
                        (void *)&ostride, (void *)&idist, (void *)&odist, (void *)&tw};
        e = cudaLaunchKernel(fn, dim3((unsigned)tiles, (unsigned)nb), dim3(k.threads), args, k.smem, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace gfft
