// deo_static.cu -- the batched apply for callers that cannot allocate device
// memory.
//
// deo_batch_create allocates device memory for its instance table, work-list
// and work counter.  Some callers cannot do that: a plug-in whose host
// application owns every device allocation through its own pool and forbids
// others, or a request handler in a memory-budgeted server that must not grow
// the device footprint after the request was admitted.  deo_batch_apply_noalloc runs the same persistent
// batched kernel with that scratch in one file-scope device array of
// DEO_NOALLOC_SCRATCH_BYTES bytes, which every GPU that loads libdeo holds
// until the process exits.  The plans and each instance's input and output
// buffers are still the caller's.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "../../include/deo.h"
#include "deo_internal.h"

// plan internals (deo_host.cpp)
extern "C" const deo::PlanDev* deo_plan_device_copy(const deo_plan* p);
extern "C" int64_t deo_plan_points(const deo_plan* p);
extern "C" int deo_plan_dtype_code(const deo_plan* p);
extern "C" deo_status deo_set_error(deo_status s, const char* msg);

namespace {

// Layout: [0, 256) work counter, cleared by every call; then the instance
// table (deo::InstDev[n]); then the work items (deo::WorkItem[m]).
static __device__ __align__(256) unsigned char g_noalloc_scratch[DEO_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
constexpr size_t kCounterBytes = 256;
std::mutex g_mu;
void* g_scratch_dev[kMaxDevices];                          // device address of the array, per device
alignas(256) unsigned char g_stage[DEO_NOALLOC_SCRATCH_BYTES];  // host image of the block (guarded by g_mu)

}  // namespace

extern "C" deo_status deo_batch_apply_noalloc(int n, const deo_instance* inst, int adjoint, int tile, void* stream) {
    if (n < 0 || (n > 0 && !inst)) return deo_set_error(DEO_ERR_BAD_ARG, "null or negative instance list");
    if (n == 0) return DEO_OK;
    const int64_t t = tile > 0 ? tile : 8192;
    int dtype = -1;
    int64_t items = 0;
    for (int i = 0; i < n; ++i) {
        if (!inst[i].plan || !inst[i].u || !inst[i].du)
            return deo_set_error(DEO_ERR_BAD_ARG, "an instance has a null plan or buffer");
        if (inst[i].u == inst[i].du) return deo_set_error(DEO_ERR_BAD_ARG, "an instance's input and output alias");
        const int dt = deo_plan_dtype_code(inst[i].plan);
        if (dtype >= 0 && dt != dtype) return deo_set_error(DEO_ERR_BAD_ARG, "all instances must share one dtype");
        dtype = dt;
        items += (deo_plan_points(inst[i].plan) + t - 1) / t;
    }
    const size_t inst_off = kCounterBytes;
    const size_t item_off = inst_off + (((size_t)n * sizeof(deo::InstDev) + 255) / 256) * 256;
    const size_t bytes = item_off + (size_t)items * sizeof(deo::WorkItem);
    if (items > (int64_t)1 << 31 || bytes > (size_t)DEO_NOALLOC_SCRATCH_BYTES)
        return deo_set_error(DEO_ERR_UNSUPPORTED,
                             "batch needs more than the DEO_NOALLOC_SCRATCH_BYTES (1 MiB) static scratch: use "
                             "fewer instances, a larger tile, or deo_batch_create");

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return deo_set_error(DEO_ERR_CUDA, "cudaGetDevice failed");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_dev[dev]) {
        // once per device, with that device current: the array's device address
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return deo_set_error(DEO_ERR_CUDA, cudaGetErrorString(e));
        g_scratch_dev[dev] = p;
    }
    unsigned char* base = static_cast<unsigned char*>(g_scratch_dev[dev]);
    std::memset(g_stage, 0, kCounterBytes);
    deo::InstDev* hi = reinterpret_cast<deo::InstDev*>(g_stage + inst_off);
    deo::WorkItem* hw = reinterpret_cast<deo::WorkItem*>(g_stage + item_off);
    int64_t m = 0;
    for (int i = 0; i < n; ++i) {
        hi[i] = deo::InstDev{deo_plan_device_copy(inst[i].plan), inst[i].u, inst[i].du};
        const int64_t np = deo_plan_points(inst[i].plan);
        for (int64_t s = 0; s < np; s += t) hw[m++] = deo::WorkItem{i, (int)std::min<int64_t>(t, np - s), s};
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // From pageable host memory the copy returns once the staging buffer has
    // been consumed, so g_stage may be reused as soon as the lock is released.
    cudaError_t e = cudaMemcpyAsync(base, g_stage, bytes, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return deo_set_error(DEO_ERR_CUDA, cudaGetErrorString(e));
    const int r = deo_k_batch(reinterpret_cast<const deo::InstDev*>(base + inst_off),
                              reinterpret_cast<const deo::WorkItem*>(base + item_off), m,
                              reinterpret_cast<unsigned int*>(base), dtype, adjoint ? 1 : 0, 4, 256, st);
    if (r) return deo_set_error(DEO_ERR_CUDA, cudaGetErrorString((cudaError_t)r));
    return DEO_OK;
}
