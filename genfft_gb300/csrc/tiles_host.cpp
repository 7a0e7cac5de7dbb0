// tiles_host.cpp -- registry and launchers of the tile kernels.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
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

int sm_count()
{
    static std::mutex mu;
    static std::map<int, int> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(dev);
    if (it != cache.end()) return it->second;
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
    cache[dev] = n;
    return n;
}

}  // namespace

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

cudaError_t launch_pdl(const void *fn, dim3 grid, dim3 block, void **args, size_t smem, cudaStream_t st)
{
    static const bool pdl = [] {
        const char *v = std::getenv("GFFT_PDL");
        return !(v && *v == '0');
    }();
    if (!pdl) return cudaLaunchKernel(fn, grid, block, args, smem, st);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelExC(&cfg, fn, args);
}

namespace {

bool tma_disabled()
{
    static const bool off = [] {
        const char *v = std::getenv("GFFT_NO_TMA");
        return v && *v && *v != '0';
    }();
    return off;
}

// single-buffered TMA tile kernels: GFFT_TMA1 unset or 1 = used (row and
// column passes), 2 = column passes only, 0 = not used
static int tma1_mode()
{
    static const int m = [] {
        const char *v = std::getenv("GFFT_TMA1");
        return (v && *v) ? std::atoi(v) : 1;
    }();
    return m;
}

static bool use_tma(const TileKernel &k)
{
    if (!k.tma_fwd || tma_disabled()) return false;
    if (k.tma_stages != 1) return true;
    const int m = tma1_mode();
    return m == 1 || (m == 2 && !k.tma_row);
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn()
{
    static EncodeTiled fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<EncodeTiled>(p);
    }();
    return fn;
}

bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

// persistent grid: every CTA that fits on the GPU at once (cached per kernel)
long long persistent_grid(const void *fn, int threads, size_t smem, long long work)
{
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, int> occ;
    int dev = 0;
    cudaGetDevice(&dev);
    int per_sm = 1;
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = occ.find({dev, fn});
        if (it != occ.end()) {
            per_sm = it->second;
        } else {
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem) != cudaSuccess ||
                per_sm < 1)
                per_sm = 1;
            occ[{dev, fn}] = per_sm;
        }
    }
    return std::max<long long>(1, std::min<long long>(work, (long long)sm_count() * per_sm));
}

}  // namespace

bool make_tensor_map_3d(CUtensorMap *map, const void *base, unsigned long long dx, unsigned long long dy,
                        unsigned long long dz, unsigned long long sy_bytes, unsigned long long sz_bytes, unsigned bx,
                        unsigned by)
{
    if (!encode_fn() || !aligned16(base) || sy_bytes % 16 || sz_bytes % 16) return false;
    cuuint64_t gdim[3] = {(cuuint64_t)dx, (cuuint64_t)dy, (cuuint64_t)dz};
    cuuint64_t gstride[2] = {(cuuint64_t)sy_bytes, (cuuint64_t)sz_bytes};
    cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    return encode_fn()(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<void *>(base), gdim, gstride, box, estr,
                       CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                       CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

unsigned *device_error_word()
{
    static std::mutex mu;
    static std::map<int, unsigned *> words;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    auto it = words.find(dev);
    if (it != words.end()) return it->second;
    unsigned *w = nullptr;
    check_cuda(cudaMalloc(&w, sizeof(unsigned)), "cudaMalloc(error word)");
    check_cuda(cudaMemset(w, 0, sizeof(unsigned)), "cudaMemset(error word)");
    words[dev] = w;
    return w;
}

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
    int best = 0, best_tma = 0, narrowest = 0;
    for (auto &kv : registry()) {
        if (std::get<0>(kv.first) != dtype || std::get<1>(kv.first) != variant || std::get<2>(kv.first) != logl)
            continue;
        const int c = std::get<3>(kv.first);
        if (!narrowest || c < narrowest) narrowest = c;
        if (c > max_c) continue;
        best = std::max(best, c);
        if (use_tma(kv.second)) best_tma = std::max(best_tma, c);
    }
    // prefer the widest tile that has a TMA-pipelined version; else the
    // widest under the cap; else the narrowest there is
    if (best_tma) return best_tma;
    return best ? best : narrowest;
}

cudaError_t launch_colpass(const TileKernel &k, int inverse, long long tiles, long long nbatch,
                           const void *in, void *out, long long ncols, long long ld_in, long long ld_out,
                           long long idist, long long odist, const void *tw, const void *tw_lo,
                           const void *tw_hi, int lo_bits, unsigned nmask, cudaStream_t st, double scale)
{
    // the kernels take the scale as their element type
    float scale_f = (float)scale;
    void *scale_p = k.elem_bytes == 8 ? (void *)&scale_f : (void *)&scale;
    // persistent TMA path: the tensor map needs 16-byte aligned base and
    // strides; in-place runs (out == in) are fine, each tile is loaded whole
    // before it is written back
    const size_t eb = (size_t)k.elem_bytes;
    if (use_tma(k) && encode_fn() && aligned16(in) && (ld_in * eb) % 16 == 0 &&
        (nbatch == 1 || (idist * eb) % 16 == 0) && ncols * (eb / 8) < (1LL << 32) && nbatch < (1LL << 31)) {
        const int units = (int)(eb / 8);
        CUtensorMap map;
        const long long rows = k.tma_rows;
        cuuint64_t gdim[3] = {(cuuint64_t)(ncols * units), (cuuint64_t)rows, (cuuint64_t)nbatch};
        cuuint64_t gstride[2] = {(cuuint64_t)(ld_in * eb), (cuuint64_t)((nbatch > 1 ? idist : rows * ld_in) * eb)};
        cuuint32_t box[3] = {(cuuint32_t)(k.tma_c * units), (cuuint32_t)k.tma_boxr, 1};
        cuuint32_t estr[3] = {1, 1, 1};
        CUresult r = encode_fn()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<void *>(in), gdim, gstride,
                                 box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r == CUDA_SUCCESS) {
            const void *fn = inverse ? k.tma_inv : k.tma_fwd;
            cudaError_t e = ensure_smem(fn, k.tma_smem);
            if (e != cudaSuccess) return e;
            unsigned *err = device_error_word();
            const long long grid = persistent_grid(fn, k.tma_threads, k.tma_smem, tiles * nbatch);
            void *args[] = {(void *)&map, (void *)&out, (void *)&ncols, (void *)&ld_out, (void *)&odist,
                            (void *)&nbatch, (void *)&tw, (void *)&tw_lo, (void *)&tw_hi, (void *)&lo_bits,
                            (void *)&nmask, (void *)&err, scale_p};
            return launch_pdl(fn, dim3((unsigned)grid), dim3(k.tma_threads), args, k.tma_smem, st);
        }
    }
    const void *fn = inverse ? k.inv : k.fwd;
    cudaError_t e = ensure_smem(fn, k.smem);
    if (e != cudaSuccess) return e;
    void *args[] = {(void *)&in,    (void *)&out,   (void *)&ncols, (void *)&ld_in,
                    (void *)&ld_out, (void *)&idist, (void *)&odist, (void *)&tw,
                    (void *)&tw_lo, (void *)&tw_hi, (void *)&lo_bits, (void *)&nmask, scale_p};
    for (long long b0 = 0; b0 < nbatch; b0 += 65535) {
        const long long nb = std::min<long long>(65535, nbatch - b0);
        const void *inp = static_cast<const char *>(in) + b0 * idist * (long long)k.elem_bytes;
        void *outp = static_cast<char *>(out) + b0 * odist * (long long)k.elem_bytes;
        args[0] = (void *)&inp;
        args[1] = (void *)&outp;
        e = launch_pdl(fn, dim3((unsigned)tiles, (unsigned)nb), dim3(k.threads), args, k.smem, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_rowpass(const TileKernel &k, int inverse, long long tiles, long long nbatch,
                           const void *in, void *out, long long nrows, long long ld_in, long long ostride,
                           long long idist, long long odist, const void *tw, cudaStream_t st, double scale)
{
    float scale_f = (float)scale;
    void *scale_p = k.elem_bytes == 8 ? (void *)&scale_f : (void *)&scale;
    const size_t eb = (size_t)k.elem_bytes;
    if (use_tma(k) && aligned16(in) && (ld_in * eb) % 16 == 0 &&
        (nbatch == 1 || (idist * eb) % 16 == 0)) {
        const void *fn = inverse ? k.tma_inv : k.tma_fwd;
        cudaError_t e = ensure_smem(fn, k.tma_smem);
        if (e != cudaSuccess) return e;
        unsigned *err = device_error_word();
        const long long grid = persistent_grid(fn, k.tma_threads, k.tma_smem, tiles * nbatch);
        void *args[] = {(void *)&in,    (void *)&out,   (void *)&nrows, (void *)&ld_in, (void *)&ostride,
                        (void *)&idist, (void *)&odist, (void *)&nbatch, (void *)&tw, (void *)&err, scale_p};
        return launch_pdl(fn, dim3((unsigned)grid), dim3(k.tma_threads), args, k.tma_smem, st);
    }
    const void *fn = inverse ? k.inv : k.fwd;
    cudaError_t e = ensure_smem(fn, k.smem);
    if (e != cudaSuccess) return e;
    for (long long b0 = 0; b0 < nbatch; b0 += 65535) {
        const long long nb = std::min<long long>(65535, nbatch - b0);
        const void *inp = static_cast<const char *>(in) + b0 * idist * (long long)k.elem_bytes;
        void *outp = static_cast<char *>(out) + b0 * odist * (long long)k.elem_bytes;
        void *args[] = {(void *)&inp,   (void *)&outp,  (void *)&nrows, (void *)&ld_in,
                        (void *)&ostride, (void *)&idist, (void *)&odist, (void *)&tw, scale_p};
        e = launch_pdl(fn, dim3((unsigned)tiles, (unsigned)nb), dim3(k.threads), args, k.smem, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace gfft
