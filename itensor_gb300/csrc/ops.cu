// Memory-bound helpers of the DMRG hot path on sm_103a:
//   * vector kernels for Davidson (axpy/axpby/scale, batched dot products, norm)
//     -- PlusEQ / dnrm2 / ddot at itensor/itdata/qdense.cc:303-311,409-417,506-664;
//   * block gather with separable offset tables -- the permute-copies of
//     QCombiner combine/uncombine (itensor/itdata/qcombiner.cc:125-300) and of
//     transform (itensor/tensor/ten_impl.h:107-160);
//   (the batched symmetric eigensolver of the density-matrix blocks is in eigh.cu)
#include "ops.h"
#include <cmath>
#include <algorithm>
#include <cstring>

namespace itg {

// ------------------------------------------------------------------ vector kernels
__global__ void fill_kernel(double* x, int64_t n, double v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] = v;
}
__global__ void scale_kernel(double* x, int64_t n, double a) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] *= a;
}
// y = a x + b y. With b == 0, y is not read: it may be fresh pool memory whose
// bits (old digit panels, integers) need not be finite doubles, and 0 * NaN = NaN.
__global__ void axpby_kernel(double* y, double const* x, int64_t n, double a, double b) {
    if (b == 0.0) {
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
            y[i] = a * x[i];
        return;
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = fma(a, x[i], b * y[i]);
}
__global__ void axpy_kernel(double* y, double const* x, int64_t n, double a) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = fma(a, x[i], y[i]);
}

static int grid_for(Ctx& ctx, int64_t n) {
    int64_t g = (n + 255) / 256;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)ctx.sm_count * 8));
}

void launch_fill(Ctx& ctx, double* x, int64_t n, double v) {
    if (n <= 0) return;
    fill_kernel<<<grid_for(ctx, n), 256, 0, ctx.stream>>>(x, n, v);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}
void launch_scale(Ctx& ctx, double* x, int64_t n, double a) {
    if (n <= 0) return;
    scale_kernel<<<grid_for(ctx, n), 256, 0, ctx.stream>>>(x, n, a);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}
void launch_axpy(Ctx& ctx, double* y, double const* x, int64_t n, double a) {
    if (n <= 0) return;
    axpy_kernel<<<grid_for(ctx, n), 256, 0, ctx.stream>>>(y, x, n, a);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}
void launch_axpby(Ctx& ctx, double* y, double const* x, int64_t n, double a, double b) {
    if (n <= 0) return;
    axpby_kernel<<<grid_for(ctx, n), 256, 0, ctx.stream>>>(y, x, n, a, b);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}

// Dot products of x with nv vectors, two-level: per-CTA partial sums in a
// fixed order, then one CTA reduces the partials (deterministic result).
constexpr int DOT_CTAS = 256;
__global__ void dots_partial_kernel(double const* const* V, int nv, double const* x, int64_t n, double* part) {
    __shared__ double sh[32];
    for (int v = 0; v < nv; ++v) {
        double const* a = V[v];
        double s = 0;
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
            s = fma(a[i], x[i], s);
        for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x < 32) {
            double t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
            for (int o = 16; o; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
            if (threadIdx.x == 0) part[(size_t)v * gridDim.x + blockIdx.x] = t;
        }
        __syncthreads();
    }
}
__global__ void dots_final_kernel(double const* part, int nparts, int nv, double* out) {
    __shared__ double sh[32];
    for (int v = 0; v < nv; ++v) {
        double s = 0;
        for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += part[(size_t)v * nparts + i];
        for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x < 32) {
            double t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
            for (int o = 16; o; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
            if (threadIdx.x == 0) out[v] = t;
        }
        __syncthreads();
    }
}

void dots(Ctx& ctx, double const* const* V, int nv, double const* x, int64_t n, double* out) {
    if (nv <= 0) return;
    // pointer list + partials + results in one pool allocation; result via mapped memory
    size_t o_ptr = 0, o_part = ((sizeof(void*) * nv + 15) / 16) * 16;
    size_t bytes = o_part + sizeof(double) * (size_t)DOT_CTAS * nv;
    DevBuf scratch(bytes, ctx.stream);
    ctx.ensure_stage(sizeof(void*) * nv);
    std::memcpy(ctx.stage, V, sizeof(void*) * nv);
    ITG_CHECK_CUDA(cudaMemcpyAsync(scratch.as<char>() + o_ptr, ctx.stage, sizeof(void*) * nv, cudaMemcpyHostToDevice, ctx.stream));
    ctx.ensure_pin(sizeof(double) * nv);
    int nb = (int)std::max<int64_t>(1, std::min<int64_t>(DOT_CTAS, (n + 255) / 256));
    dots_partial_kernel<<<nb, 256, 0, ctx.stream>>>(reinterpret_cast<double const* const*>(scratch.as<char>() + o_ptr), nv, x, n,
                                                    reinterpret_cast<double*>(scratch.as<char>() + o_part));
    dots_final_kernel<<<1, 256, 0, ctx.stream>>>(reinterpret_cast<double const*>(scratch.as<char>() + o_part), nb, nv,
                                                 static_cast<double*>(ctx.pin_dev));
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches += 2;
    ctx.sync();
    std::memcpy(out, ctx.pin, sizeof(double) * nv);
}

double dot(Ctx& ctx, double const* a, double const* b, int64_t n) {
    double r = 0;
    double const* V[1] = {a};
    dots(ctx, V, 1, b, n, &r);
    return r;
}

double norm(Ctx& ctx, double const* a, int64_t n) {
    double r = dot(ctx, a, a, n);
    return std::sqrt(std::max(r, 0.0));
}

// ------------------------------------------------------------------ gather
// dst[doff + d1[i] + d2[j]] = src[soff + s1[i] + s2[j]], i < n1 (fastest), j < n2
__global__ void gather_kernel(GatherItem const* __restrict__ items, int32_t const* __restrict__ tab,
                              double const* __restrict__ src, double* __restrict__ dst) {
    const GatherItem it = items[blockIdx.x];
    const int64_t n = (int64_t)it.n1 * it.n2;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
        int i = (int)(e % it.n1), j = (int)(e / it.n1);
        dst[it.doff + tab[it.td1 + i] + tab[it.td2 + j]] = src[it.soff + tab[it.ts1 + i] + tab[it.ts2 + j]];
    }
}

void GatherPlan::upload(Ctx& ctx) {
    size_t o_items = 0, o_tab = ((sizeof(GatherItem) * std::max<size_t>(1, items.size()) + 15) / 16) * 16;
    size_t bytes = o_tab + sizeof(int32_t) * std::max<size_t>(1, tab.size());
    ctx.ensure_stage(bytes);
    char* st = static_cast<char*>(ctx.stage);
    if (!items.empty()) std::memcpy(st + o_items, items.data(), sizeof(GatherItem) * items.size());
    if (!tab.empty()) std::memcpy(st + o_tab, tab.data(), sizeof(int32_t) * tab.size());
    dev = dev_alloc(bytes, ctx.stream);
    ITG_CHECK_CUDA(cudaMemcpyAsync(dev->as<char>(), st, bytes, cudaMemcpyHostToDevice, ctx.stream));
    ctx.sync();
    d_items = reinterpret_cast<GatherItem*>(dev->as<char>() + o_items);
    d_tab = reinterpret_cast<int32_t*>(dev->as<char>() + o_tab);
    nitems = (int)items.size();
}

void launch_gather(Ctx& ctx, GatherPlan const& g, double const* src, double* dst) {
    if (g.nitems == 0) return;
    gather_kernel<<<g.nitems, 256, 0, ctx.stream>>>(g.d_items, g.d_tab, src, dst);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}

// Deterministic pseudo-random fill in [0,1) (splitmix64 of the element index
// and a seed); used when Davidson must replace a dependent vector.
__global__ void random_kernel(double* x, int64_t n, uint64_t seed) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t z = seed + 0x9e3779b97f4a7c15ull * (uint64_t)(i + 1);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        z ^= z >> 31;
        x[i] = (double)(z >> 11) * (1.0 / 9007199254740992.0);
    }
}
void launch_random(Ctx& ctx, double* x, int64_t n, uint64_t seed) {
    if (n <= 0) return;
    random_kernel<<<grid_for(ctx, n), 256, 0, ctx.stream>>>(x, n, seed);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}
}  // namespace itg
