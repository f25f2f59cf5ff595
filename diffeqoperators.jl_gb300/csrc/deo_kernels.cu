// deo_kernels.cu -- sm_103a kernels of the stencil-apply path.
//
// The forward evaluator computes, for output point `idx` and each term t,
//     r_t = sum_k W_i[k] * x[p0_i + k]      (row table, see deo_internal.h)
// with the ghost values x[1], x[len+2] produced in-kernel from the boundary
// condition's affine map; then du = ((r_0 + r_1) + r_2) ... as the
// reference's `sum(op -> op*u, ops)` does.  Nothing is materialised: the
// ghost fill, the boundary rows and the interior stencil are one pass.
//
// The adjoint evaluator computes ubar = A_l^T dbar by gathering, for every
// padded column p, the rows whose window covers p (deterministic, no atomics),
// then folding the ghost columns back through the affine map.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "deo_eval.cuh"

namespace deo {

// The forward evaluator without per-line BCs is held to the registers of a
// full SM: Float64 at 32 (eight CTAs, 64 warps, against five at its natural
// 44, with a few hundred bytes of spills: its FP64 chains wait on loads and on
// the FP64 pipe, and the extra warps cover that: 0.219 -> 0.203 ms on the
// 2048^2 non-uniform sum), Float32 at 40 (six CTAs, no spills).
template <typename T, bool ADJ, bool LBC>
__global__ void __launch_bounds__(256, (!ADJ && !LBC) ? (sizeof(T) == 8 ? 8 : 6) : 0)
    k_apply(const __grid_constant__ PlanDev P, const T* __restrict__ u, T* __restrict__ du, int overwrite) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= P.total) return;
    const T r = eval_point<T, ADJ, LBC>(P, u, idx);
    du[idx] = overwrite ? r : r + du[idx];
}

// Persistent batched kernel: CTAs pull work items from a global counter until
// the list is exhausted (no waiting on other CTAs, so no spin loops).
// The instance's plan is staged into shared memory when a work item belongs to
// a different instance than the previous one (items are instance-contiguous
// within a size class, so consecutive pulls usually share it).
struct PlanCache {
    static_assert(sizeof(PlanDev) % 8 == 0, "PlanDev copied in 8-byte words");
    unsigned long long words[sizeof(PlanDev) / 8];
    const PlanDev* src;
};

__device__ __forceinline__ const PlanDev& stage_plan(PlanCache& c, const PlanDev* p) {
    if (p != c.src) {  // uniform across the CTA
        const unsigned long long* s = reinterpret_cast<const unsigned long long*>(p);
        for (int q = threadIdx.x; q < (int)(sizeof(PlanDev) / 8); q += blockDim.x) c.words[q] = s[q];
        __syncthreads();
        if (threadIdx.x == 0) c.src = p;
    }
    return *reinterpret_cast<const PlanDev*>(c.words);
}

template <typename T, bool ADJ, bool LBC>
__global__ void __launch_bounds__(256) k_batch(const InstDev* __restrict__ inst, const WorkItem* __restrict__ items,
                                               int64_t n_items, unsigned int* counter) {
    __shared__ int64_t s_item;
    __shared__ __align__(16) PlanCache cache;
    if (threadIdx.x == 0) cache.src = nullptr;
    for (;;) {
        if (threadIdx.x == 0) s_item = (int64_t)atomicAdd(counter, 1u);
        __syncthreads();
        const int64_t it = s_item;
        const bool stale = it < n_items && inst[items[it].inst].plan != cache.src;
        __syncthreads();
        if (it >= n_items) return;
        const WorkItem w = items[it];
        const InstDev in = inst[w.inst];
        const PlanDev& P = stale ? stage_plan(cache, in.plan) : *reinterpret_cast<const PlanDev*>(cache.words);
        const T* __restrict__ u = reinterpret_cast<const T*>(in.u);
        T* __restrict__ du = reinterpret_cast<T*>(in.du);
        for (int q = threadIdx.x; q < w.count; q += blockDim.x) {
            const int64_t idx = w.start + q;
            du[idx] = eval_point<T, ADJ, LBC>(P, u, idx);
        }
    }
}

// Batched Runge-Kutta stage: same work-list scheme; each instance may run
// the forward operator or its adjoint (uniform per work item).
template <typename T, bool LBC>
__global__ void __launch_bounds__(256) k_stage(const StageDev* __restrict__ st, const WorkItem* __restrict__ items,
                                               int64_t n_items, unsigned int* counter) {
    __shared__ int64_t s_item;
    __shared__ __align__(16) PlanCache cache;
    if (threadIdx.x == 0) cache.src = nullptr;
    for (;;) {
        if (threadIdx.x == 0) s_item = (int64_t)atomicAdd(counter, 1u);
        __syncthreads();
        const int64_t it = s_item;
        const bool stale = it < n_items && st[items[it].inst].plan != cache.src;
        __syncthreads();
        if (it >= n_items) return;
        const WorkItem w = items[it];
        const StageDev S = st[w.inst];
        const PlanDev& P = stale ? stage_plan(cache, S.plan) : *reinterpret_cast<const PlanDev*>(cache.words);
        const T* a = reinterpret_cast<const T*>(S.a);  // may alias out
        const T* b = reinterpret_cast<const T*>(S.b);
        const T* __restrict__ c = reinterpret_cast<const T*>(S.c);
        T* out = reinterpret_cast<T*>(S.out);
        const T al = T(S.alpha), be = T(S.beta), ga = T(S.gamma), dt = T(S.dt);
        for (int q = threadIdx.x; q < w.count; q += blockDim.x) {
            const int64_t idx = w.start + q;
            const T f = S.adjoint ? eval_point<T, true, LBC>(P, c, idx) : eval_point<T, false, LBC>(P, c, idx);
            const T t = fma(dt, f, c[idx]);
            T acc = a ? al * a[idx] : T(0);
            if (b) acc = fma(be, b[idx], acc);
            out[idx] = fma(ga, t, acc);
        }
    }
}

}  // namespace deo

using namespace deo;

// nonlinear_diffusion!{N}(du, n, m, approx, p, q, dx, len) on padded vectors
// (derivative_operator.jl:34-66): with D_k the order-k centred operator (plan
// term k-1) applied to a padded vector by the generic method,
//   du = (D_m q) .* (D_n p)            (m > 0)   or   q[2:len+1] .* (D_n p)   (m == 0)
//   du = du .+ binomial(n, l) * (D_{l+m} q) .* (D_{n-l} p),   l = 1 .. n-1
//   du = du .+ (D_{m+n} q) .* p[2:len+1]
// each broadcast in the reference's operation order, one thread per point.
template <typename T>
__global__ void __launch_bounds__(256) k_nld(const PlanDev P, int len, int n, int m, const T* __restrict__ p,
                                             const T* __restrict__ q, T* __restrict__ du) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= len) return;
    // the vectors hold their own ghosts: row i + 1 of D_k over x[0 .. len + 1]
    auto D = [&](int k, const T* x) { return eval_row_padded<T>(P.t[k - 1].tab[0], x, 1, i + 1); };
    T acc = (m > 0 ? D(m, q) : q[i + 1]) * D(n, p);
    long long b = 1;  // binomial(n, l)
    for (int l = 1; l <= n - 1; ++l) {
        b = b * (n - l + 1) / l;
        acc = acc + (T(b) * D(l + m, q)) * D(n - l, p);
    }
    acc = acc + D(m + n, q) * p[i + 1];
    du[i] = acc;
}

extern "C" int deo_k_nonlinear_diffusion(const PlanDev* plan, int len, int n, int m, int dtype, const void* p,
                                         const void* q, void* du, void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const unsigned blocks = (unsigned)((len + 255) / 256);
    if (dtype == 0)
        k_nld<double><<<blocks, 256, 0, st>>>(*plan, len, n, m, (const double*)p, (const double*)q, (double*)du);
    else
        k_nld<float><<<blocks, 256, 0, st>>>(*plan, len, n, m, (const float*)p, (const float*)q, (float*)du);
    return (int)cudaGetLastError();
}

extern "C" int deo_k_num_sms(void);

template <typename T>
__global__ void __launch_bounds__(256) k_scale(T* __restrict__ x, int64_t n, T f) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = f * x[i];
}

// x *= f over n points of the dtype (the adjoint seed 2 u(T) of ||u(T)||^2).
extern "C" int deo_k_scale(void* x, int64_t n, int dtype, double f, void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int sms = deo_k_num_sms();
    const int64_t want = (n + 255) / 256;
    const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms * 8));
    if (dtype == 0) k_scale<double><<<blocks, 256, 0, st>>>((double*)x, n, f);
    else k_scale<float><<<blocks, 256, 0, st>>>((float*)x, n, (float)f);
    return (int)cudaGetLastError();
}

extern "C" int deo_k_stage_batch(const StageDev* st, const WorkItem* items, int64_t n_items, unsigned int* counter,
                                 int lbc,
                                 int dtype, int ctas_per_sm, int threads, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int sms = deo_k_num_sms();
    int64_t grid = (int64_t)sms * (ctas_per_sm > 0 ? ctas_per_sm : 4);
    if (grid > n_items) grid = n_items;
    if (grid <= 0) return 0;
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return (int)e;
    if (dtype == 0) {
        if (lbc) k_stage<double, true><<<(unsigned)grid, threads, 0, s>>>(st, items, n_items, counter);
        else k_stage<double, false><<<(unsigned)grid, threads, 0, s>>>(st, items, n_items, counter);
    } else {
        if (lbc) k_stage<float, true><<<(unsigned)grid, threads, 0, s>>>(st, items, n_items, counter);
        else k_stage<float, false><<<(unsigned)grid, threads, 0, s>>>(st, items, n_items, counter);
    }
    return (int)cudaGetLastError();
}

extern "C" int deo_k_apply(const PlanDev* p, const void* u, void* du, int overwrite, int adjoint, void* stream) {
    const int threads = 256;
    const int64_t blocks = (p->total + threads - 1) / threads;
    if (blocks == 0) return 0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto go = [&](auto kernel, const auto* in, auto* out) {
        kernel<<<(unsigned)blocks, threads, 0, st>>>(*p, in, out, overwrite);
    };
    const double* ud = (const double*)u;
    const float* uf = (const float*)u;
    if (p->dtype == 0) {
        if (p->has_lbc) adjoint ? go(k_apply<double, true, true>, ud, (double*)du) : go(k_apply<double, false, true>, ud, (double*)du);
        else adjoint ? go(k_apply<double, true, false>, ud, (double*)du) : go(k_apply<double, false, false>, ud, (double*)du);
    } else {
        if (p->has_lbc) adjoint ? go(k_apply<float, true, true>, uf, (float*)du) : go(k_apply<float, false, true>, uf, (float*)du);
        else adjoint ? go(k_apply<float, true, false>, uf, (float*)du) : go(k_apply<float, false, false>, uf, (float*)du);
    }
    return (int)cudaGetLastError();
}

extern "C" int deo_k_num_sms(void) {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    return n;
}

// Loads the k_batch instantiations onto the current device and runs each
// once over an empty work-list (one CTA; it only bumps *counter), so that the
// module image and the resources a launch of them takes are committed now:
// with lazy module loading (the CUDA default) that would otherwise happen at
// their first real launch.
extern "C" int deo_k_batch_prepare(unsigned int* counter, void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaFuncAttributes a;
    cudaError_t e = cudaSuccess;
    auto prep = [&](auto kernel) {
        if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, kernel);
        if (e == cudaSuccess) kernel<<<1, 256, 0, st>>>(nullptr, nullptr, 0, counter);
    };
    prep(k_batch<double, false, false>);
    prep(k_batch<double, true, false>);
    prep(k_batch<float, false, false>);
    prep(k_batch<float, true, false>);
    prep(k_batch<double, false, true>);
    prep(k_batch<double, true, true>);
    prep(k_batch<float, false, true>);
    prep(k_batch<float, true, true>);
    if (e != cudaSuccess) return (int)e;
    return (int)cudaGetLastError();
}

extern "C" int deo_k_batch(const InstDev* inst, const WorkItem* items, int64_t n_items, unsigned int* counter,
                           int dtype, int adjoint, int lbc, int ctas_per_sm, int threads, void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int sms = deo_k_num_sms();
    int64_t grid = (int64_t)sms * (ctas_per_sm > 0 ? ctas_per_sm : 4);
    if (grid > n_items) grid = n_items;
    if (grid <= 0) return 0;
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return (int)e;
    auto go = [&](auto kernel) { kernel<<<(unsigned)grid, threads, 0, st>>>(inst, items, n_items, counter); };
    if (dtype == 0) {
        if (lbc) adjoint ? go(k_batch<double, true, true>) : go(k_batch<double, false, true>);
        else adjoint ? go(k_batch<double, true, false>) : go(k_batch<double, false, false>);
    } else {
        if (lbc) adjoint ? go(k_batch<float, true, true>) : go(k_batch<float, false, true>);
        else adjoint ? go(k_batch<float, true, false>) : go(k_batch<float, false, false>);
    }
    return (int)cudaGetLastError();
}
