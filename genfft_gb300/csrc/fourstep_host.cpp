// fourstep_host.cpp -- registry, schedule and launcher of the persistent
// four-step kernels.
#include <algorithm>
#include <cstdlib>
#include <map>
#include <mutex>
#include <set>
#include <utility>
#include <vector>

#include "fourstep.h"
#include "internal.h"

namespace gfft {

namespace {
std::map<std::pair<int, int>, std::vector<FourStepKernel>> &fs_registry()
{
    static std::map<std::pair<int, int>, std::vector<FourStepKernel>> r;
    return r;
}
std::mutex &fs_mu()
{
    static std::mutex m;
    return m;
}
std::map<std::pair<int, int>, std::vector<const FourStepKernel *>> &fs_views()
{
    static std::map<std::pair<int, int>, std::vector<const FourStepKernel *>> v;
    return v;
}
long long env_ll(const char *name, long long dflt)
{
    const char *v = std::getenv(name);
    return (v && *v) ? std::atoll(v) : dflt;
}
}  // namespace

void fourstep_register(int dtype, int logn, const FourStepKernel &k)
{
    std::lock_guard<std::mutex> lk(fs_mu());
    fs_registry()[{dtype, logn}].push_back(k);
    fs_views().erase({dtype, logn});
}

const FourStepKernel *const *fourstep_variants(int dtype, int logn, int *n)
{
    std::lock_guard<std::mutex> lk(fs_mu());
    auto it = fs_registry().find({dtype, logn});
    if (it == fs_registry().end()) {
        *n = 0;
        return nullptr;
    }
    auto &view = fs_views()[{dtype, logn}];
    if (view.empty()) {
        for (auto &k : it->second) view.push_back(&k);
        std::stable_sort(view.begin(), view.end(),
                         [](const FourStepKernel *x, const FourStepKernel *y) { return x->cc > y->cc; });
    }
    *n = (int)view.size();
    return view.data();
}

void fourstep_schedule(size_t bytes, long long batch, int grid, int depth, int items_per_transform, int *slots,
                       int *lag)
{
    // LAG: enough phases between a transform's COL and ROW tiles that the
    // ROW tiles are claimed after the COL tiles are done.  Every CTA holds
    // up to `depth` claimed items (its stages plus the one its producer
    // waits to place), so grid * depth items are in flight at once.
    int lg = (int)env_ll("GFFT_FS_LAG", -1);
    if (lg < 0) lg = std::max(1, (grid * depth + items_per_transform - 1) / items_per_transform + 1);
    // slots: lag + 2, and more while the ring stays within the L2 budget
    const long long budget = env_ll("GFFT_FS_L2_MB", 80) << 20;
    int s = (int)env_ll("GFFT_FS_SLOTS", -1);
    if (s < 0) {
        s = lg + 2;
        while ((long long)(s + 1) * (long long)bytes <= budget && s < 2 * lg + 4) s++;
        // large transforms: the fewest slots the lag allows, to stay in L2
        if ((long long)s * (long long)bytes > budget) s = std::max<long long>(lg + 1, budget / (long long)bytes);
    }
    s = std::max(s, lg + 1);
    s = (int)std::max<long long>(1, std::min<long long>(s, batch + lg + 1));
    if (lg >= s) lg = s - 1;
    *slots = s;
    *lag = lg;
}

int fourstep_grid(const FourStepKernel &k, bool dit)
{
    const void *const main_fn = dit ? k.dit : k.fwd;
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, int> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find({dev, main_fn});
    if (it != cache.end()) return it->second;
    for (const void *fn : {k.fwd, k.inv, k.dit})
        if (fn && k.smem > 48 * 1024)
            check_cuda(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem),
                       "four-step shared memory opt-in");
    int per_sm = 0, sms = 0;
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, main_fn, k.threads, k.smem), "occupancy");
    check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
    const int g = std::max(1, per_sm) * sms;
    cache[{dev, main_fn}] = g;
    return g;
}

cudaError_t launch_fourstep(const FourStepKernel &k, int inverse, const CUtensorMap &map, const FourStepArgs &a,
                            int grid, cudaStream_t st, bool dit)
{
    if (dit && !k.dit) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(a.ctr, 0, (size_t)(2 + 2 * a.slots) * sizeof(int), st);
    if (e != cudaSuccess) return e;
    FourStepArgs args = a;
    CUtensorMap m = map;
    void *p[] = {&m, &args};
    const int g = std::max(1, std::min(grid, a.nitems));
    return cudaLaunchKernel(dit ? k.dit : inverse ? k.inv : k.fwd, dim3((unsigned)g), dim3(k.threads), p, k.smem, st);
}

}  // namespace gfft
