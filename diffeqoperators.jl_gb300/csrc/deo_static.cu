// deo_static.cu -- the batched apply for callers that cannot allocate device
// memory.
//
// deo_batch_create allocates device memory for its instance table, work-list
// and work counter.  Some callers cannot do that: a plug-in whose host
// application owns every device allocation through its own pool and forbids
// others, or a request handler in a memory-budgeted server that must not grow
// the device footprint after the request was admitted.  deo_batch_apply_noalloc
// runs the same persistent batched kernel with that scratch in one file-scope
// device array of DEO_NOALLOC_SCRATCH_BYTES bytes.  CUDA loads the module that
// holds the array (and the one that holds the kernel) lazily, so the array
// and the kernel's image occupy a device from the first call on it -- a call
// with n = 0 does only that set-up -- until the process exits.  The plans and
// each instance's input and output buffers are still the caller's.
#include <cuda.h>
#include <cudaTypedefs.h>
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
extern "C" int deo_plan_has_lbc(const deo_plan* p);
extern "C" deo_status deo_set_error(deo_status s, const char* msg);

namespace {

// Layout: [0, 256) work counter, cleared by every call; then the instance
// table (deo::InstDev[n]); then the work items (deo::WorkItem[m]).
static __device__ __align__(256) unsigned char g_noalloc_scratch[DEO_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
constexpr size_t kCounterBytes = 256;
std::mutex g_mu;
// Per device: the array's device address and the id of the CUDA context it
// was looked up in.  After a device reset the primary context is a new one
// with a new id, so the address is looked up (and the kernel prepared) again.
struct DevScratch {
    unsigned long long ctx_id;
    void* ptr;
};
DevScratch g_dev[kMaxDevices];
alignas(256) unsigned char g_stage[DEO_NOALLOC_SCRATCH_BYTES];  // host image of the block (guarded by g_mu)

// The current context's unique id (cuCtxGetId), through the runtime's driver
// entry points so that the library needs no link against libcuda; 0 if the
// driver does not provide it.
unsigned long long current_ctx_id() {
    static PFN_cuCtxGetCurrent_v4000 get_cur = nullptr;
    static PFN_cuCtxGetId_v12000 get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_cur = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(p);
    });
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (!get_cur || !get_id || get_cur(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Set-up for the current device, with it current (caller holds g_mu): the
// array's device address, and every operation a call issues done once (the
// host-to-device copy, the counter's memset, k_batch's launches over an empty
// work-list), so that later calls on this device change its footprint no more.
deo_status prepare(int dev, cudaStream_t st, unsigned char** base) {
    const unsigned long long id = current_ctx_id();
    DevScratch& d = g_dev[dev];
    if (!d.ptr || id == 0 || d.ctx_id != id) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return deo_set_error(DEO_ERR_CUDA, cudaGetErrorString(e));
        std::memset(g_stage, 0, kCounterBytes);
        e = cudaMemcpyAsync(p, g_stage, kCounterBytes, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(p, 0, kCounterBytes, st);
        if (e != cudaSuccess) return deo_set_error(DEO_ERR_CUDA, cudaGetErrorString(e));
        const int r = deo_k_batch_prepare(static_cast<unsigned int*>(p), st);
        if (r) return deo_set_error(DEO_ERR_CUDA, cudaGetErrorString((cudaError_t)r));
        d.ptr = p;
        d.ctx_id = id;
    }
    *base = static_cast<unsigned char*>(d.ptr);
    return DEO_OK;
}

}  // namespace

extern "C" deo_status deo_batch_apply_noalloc(int n, const deo_instance* inst, int adjoint, int tile, void* stream) {
    if (n < 0 || (n > 0 && !inst)) return deo_set_error(DEO_ERR_BAD_ARG, "null or negative instance list");
    const int64_t t = tile > 0 ? tile : 8192;
    int dtype = -1, lbc = 0;
    int64_t items = 0;
    for (int i = 0; i < n; ++i) {
        if (!inst[i].plan || !inst[i].u || !inst[i].du)
            return deo_set_error(DEO_ERR_BAD_ARG, "an instance has a null plan or buffer");
        if (inst[i].u == inst[i].du) return deo_set_error(DEO_ERR_BAD_ARG, "an instance's input and output alias");
        const int dt = deo_plan_dtype_code(inst[i].plan);
        if (dtype >= 0 && dt != dtype) return deo_set_error(DEO_ERR_BAD_ARG, "all instances must share one dtype");
        dtype = dt;
        lbc |= deo_plan_has_lbc(inst[i].plan);
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
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // its copy from the (pageable, reused) host image cannot be captured into a graph
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) != cudaSuccess)
        return deo_set_error(DEO_ERR_CUDA, "cudaStreamIsCapturing failed");
    if (cap != cudaStreamCaptureStatusNone)
        return deo_set_error(DEO_ERR_UNSUPPORTED, "deo_batch_apply_noalloc cannot run under stream capture");
    std::lock_guard<std::mutex> lk(g_mu);
    unsigned char* base = nullptr;
    const deo_status ps = prepare(dev, st, &base);
    if (ps != DEO_OK || n == 0) return ps;
    std::memset(g_stage, 0, kCounterBytes);
    deo::InstDev* hi = reinterpret_cast<deo::InstDev*>(g_stage + inst_off);
    deo::WorkItem* hw = reinterpret_cast<deo::WorkItem*>(g_stage + item_off);
    int64_t m = 0;
    for (int i = 0; i < n; ++i) {
        hi[i] = deo::InstDev{deo_plan_device_copy(inst[i].plan), inst[i].u, inst[i].du};
        const int64_t np = deo_plan_points(inst[i].plan);
        for (int64_t s = 0; s < np; s += t) hw[m++] = deo::WorkItem{i, (int)std::min<int64_t>(t, np - s), s};
    }
    // The copy is ordered after earlier work on `stream` by the stream itself.
    // From pageable host memory CUDA stages the data before cudaMemcpyAsync
    // returns, so g_stage may be refilled once the lock is released.
    cudaError_t e = cudaMemcpyAsync(base, g_stage, bytes, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return deo_set_error(DEO_ERR_CUDA, cudaGetErrorString(e));
    const int r = deo_k_batch(reinterpret_cast<const deo::InstDev*>(base + inst_off),
                              reinterpret_cast<const deo::WorkItem*>(base + item_off), m,
                              reinterpret_cast<unsigned int*>(base), dtype, adjoint ? 1 : 0, lbc, 4, 256, st);
    if (r) return deo_set_error(DEO_ERR_CUDA, cudaGetErrorString((cudaError_t)r));
    return DEO_OK;
}
