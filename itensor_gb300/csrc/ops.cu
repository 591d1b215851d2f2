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
    pdl_wait();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] = v;
}
__global__ void scale_kernel(double* x, int64_t n, double a) {
    pdl_wait();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] *= a;
}
// y = a x + b y. With b == 0, y is not read: it may be fresh pool memory whose
// bits (old digit panels, integers) need not be finite doubles, and 0 * NaN = NaN.
__global__ void axpby_kernel(double* y, double const* x, int64_t n, double a, double b) {
    pdl_wait();
    if (b == 0.0) {
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
            y[i] = a * x[i];
        return;
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = fma(a, x[i], b * y[i]);
}
__global__ void axpy_kernel(double* y, double const* x, int64_t n, double a) {
    pdl_wait();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = fma(a, x[i], y[i]);
}

static int grid_for(Ctx& ctx, int64_t n) {
    int64_t g = (n + 255) / 256;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)ctx.sm_count * 8));
}

void launch_fill(Ctx& ctx, double* x, int64_t n, double v) {
    if (n <= 0) return;
    launch_pdl(ctx, grid_for(ctx, n), 256, 0, fill_kernel, x, n, v);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}
// Device-to-device copy on the SMs, launched like the other small kernels
// (programmatic dependent launch): a copy-engine transfer between two kernels
// would break their launch overlap.
__global__ void copy_kernel(double* __restrict__ dst, double const* __restrict__ src, int64_t n) {
    pdl_wait();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}
void launch_copy(Ctx& ctx, double* dst, double const* src, int64_t n) {
    if (n <= 0) return;
    launch_pdl(ctx, grid_for(ctx, n), 256, 0, copy_kernel, dst, src, n);
    ctx.kernel_launches++;
}

void launch_scale(Ctx& ctx, double* x, int64_t n, double a) {
    if (n <= 0) return;
    launch_pdl(ctx, grid_for(ctx, n), 256, 0, scale_kernel, x, n, a);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}
void launch_axpy(Ctx& ctx, double* y, double const* x, int64_t n, double a) {
    if (n <= 0) return;
    launch_pdl(ctx, grid_for(ctx, n), 256, 0, axpy_kernel, y, x, n, a);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}
void launch_axpby(Ctx& ctx, double* y, double const* x, int64_t n, double a, double b) {
    if (n <= 0) return;
    launch_pdl(ctx, grid_for(ctx, n), 256, 0, axpby_kernel, y, x, n, a, b);
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

void dots_fused(Ctx& ctx, VecList const& V, double const* x, int64_t n, double* out);

void dots(Ctx& ctx, double const* const* V, int nv, double const* x, int64_t n, double* out) {
    if (nv <= 0) return;
    if (nv <= VecList::MAX) {
        VecList L;
        for (int k = 0; k < nv; ++k) L.add(V[k], 0.0);
        dots_fused(ctx, L, x, n, out);
        return;
    }
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

// Sum of the CTAs' partials by the last CTA: a loop of one thread over the
// partials when there are few of them, else one partial per thread added as
// a tree (lanes by shuffles, then the warps' sums in warp 0). Every FP64 add
// is a warp instruction that holds its SMSP's FP64 pipe for about 64 cycles,
// so a loop over 196 partials alone took about 11 us of a 17 us launch
// (n = 50,000; the tree form: 6 us). Deterministic either way (the grid size
// decides the form). The result is valid in thread 0. Called by every thread
// of the CTA.
constexpr int TREE_MIN_PARTS = 32;
__device__ double sum_partials(double const* __restrict__ part, int nparts, double* sh) {
    if (nparts <= TREE_MIN_PARTS) {
        double t = 0;
        if (threadIdx.x == 0)
            for (int b = 0; b < nparts; ++b) t += __ldcg(part + b);
        return t;
    }
    double v = 0;
    for (int b = threadIdx.x; b < nparts; b += blockDim.x) v += __ldcg(part + b);
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();  // a previous use of sh has been read
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0;
    const int nw = (int)(blockDim.x >> 5);
    if (threadIdx.x < 32) {
        t = (int)threadIdx.x < nw ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o; o >>= 1)
            if (o < nw) t += __shfl_down_sync(0xffffffffu, t, o);
    }
    return t;
}

// ------------------------------------------------------------------ fused combinations
// y = a0 y + sum_k c_k X_k (y not read when a0 == 0), the terms added in k
// order with one FMA each (the same rounding as a chain of axpy calls), and
// optionally |y|^2: per-CTA partial sums in a fixed order, reduced by the last
// CTA to finish (deterministic whichever CTA that is). Pointers and
// coefficients travel as kernel parameters: no upload, one launch.
// Coefficients may come from scalar slots `sd` (VecList::cs): c[k] * sd[cs[k]].
// |y|^2 goes to `out` (and to `out2` when given).
__global__ void combo_kernel(double* __restrict__ y, double a0, VecList X, int64_t n, int want_norm,
                             double* __restrict__ part, unsigned int* __restrict__ counter, double* __restrict__ out,
                             double* __restrict__ out2, double const* __restrict__ sd) {
    pdl_wait();
    __shared__ double sh[32];
    __shared__ double cf[VecList::MAX];
    __shared__ bool last;
    if (threadIdx.x < X.n) {
        const int k = threadIdx.x;
        cf[k] = X.cs[k] >= 0 ? X.c[k] * sd[X.cs[k]] : X.c[k];
    }
    __syncthreads();
    double s2 = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double v = (a0 == 0.0) ? 0.0 : (a0 == 1.0 ? y[i] : a0 * y[i]);
        int k = 0;
        if (a0 == 0.0 && X.n > 0) { v = cf[0] * X.p[0][i]; k = 1; }
        for (; k < X.n; ++k) v = fma(cf[k], X.p[k][i], v);
        y[i] = v;
        s2 = fma(v, v, s2);
    }
    if (!want_norm) return;
    for (int o = 16; o; o >>= 1) s2 += __shfl_down_sync(0xffffffffu, s2, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s2;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
        part[blockIdx.x] = t;
        __threadfence();
        last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    const double t = sum_partials(part, (int)gridDim.x, sh);
    if (threadIdx.x == 0) {
        *out = t;
        if (out2) *out2 = t;
        *counter = 0;  // ready for the next launch on this stream
    }
}

// Dot products of x with every vector of V in one launch: partials per CTA in
// a fixed order, the last CTA to finish reduces them in CTA order.
__global__ void dots_fused_kernel(VecList V, double const* __restrict__ x, int64_t n, double* __restrict__ part,
                                  unsigned int* __restrict__ counter, double* __restrict__ out,
                                  double* __restrict__ out2) {
    pdl_wait();
    __shared__ double sh[32];
    __shared__ bool last;
    for (int v = 0; v < V.n; ++v) {
        double const* a = V.p[v];
        double s = 0;
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
            s = fma(a[i], x[i], s);
        for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
            part[(size_t)v * gridDim.x + blockIdx.x] = t;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        __threadfence();
        last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    if ((int)gridDim.x <= TREE_MIN_PARTS) {
        // few partials: one thread per vector, in CTA order
        for (int v = threadIdx.x; v < V.n; v += blockDim.x) {
            double t = 0;
            for (int b = 0; b < (int)gridDim.x; ++b) t += __ldcg(part + (size_t)v * gridDim.x + b);
            out[v] = t;
            if (out2) out2[v] = t;
        }
    } else {
        for (int v = 0; v < V.n; ++v) {
            const double t = sum_partials(part + (size_t)v * gridDim.x, (int)gridDim.x, sh);
            if (threadIdx.x == 0) {
                out[v] = t;
                if (out2) out2[v] = t;
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) *counter = 0;  // ready for the next launch on this stream
}

namespace {
constexpr size_t REDUCE_DOUBLES = (size_t)DOT_CTAS * VecList::MAX + 4;
}

void Ctx::ensure_reduce() {
    if (reduce_buf) return;
    reduce_buf = dev_alloc(sizeof(double) * REDUCE_DOUBLES, stream);
    ITG_CHECK_CUDA(cudaMemsetAsync(reduce_buf->p, 0, sizeof(double) * REDUCE_DOUBLES, stream));
}

void dots_fused(Ctx& ctx, VecList const& V, double const* x, int64_t n, double* out) {
    ctx.ensure_reduce();
    ctx.ensure_pin(sizeof(double) * VecList::MAX);
    double* part = ctx.reduce_buf->as<double>();
    unsigned int* counter = reinterpret_cast<unsigned int*>(part + REDUCE_DOUBLES - 2);
    const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(DOT_CTAS, (n + 255) / 256));
    launch_pdl(ctx, nb, 256, 0, dots_fused_kernel, V, x, n, part, counter, static_cast<double*>(ctx.pin_dev), nullptr);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
    ctx.sync();
    std::memcpy(out, ctx.pin, sizeof(double) * V.n);
}

void Ctx::ensure_scalars() {
    if (scal_host) return;
    ITG_CHECK_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&scal_host), sizeof(double) * NSCALAR, cudaHostAllocMapped));
    ITG_CHECK_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void**>(&scal_map), scal_host, 0));
    scal_dev = dev_alloc(sizeof(double) * NSCALAR, stream);
}

void dots_async(Ctx& ctx, VecList const& V, double const* x, int64_t n, int slot) {
    ITG_REQUIRE(slot >= 0 && slot + V.n <= Ctx::NSCALAR, "dots_async: scalar slots out of range");
    if (V.n == 0) return;
    ctx.ensure_reduce();
    ctx.ensure_scalars();
    double* part = ctx.reduce_buf->as<double>();
    unsigned int* counter = reinterpret_cast<unsigned int*>(part + REDUCE_DOUBLES - 2);
    const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(DOT_CTAS, (n + 255) / 256));
    launch_pdl(ctx, nb, 256, 0, dots_fused_kernel, V, x, n, part, counter, ctx.scal_map + slot,
                                                  ctx.scal_dev->as<double>() + slot);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}

__global__ void scale_rnorm_kernel(double* x, int64_t n, double const* __restrict__ s) {
    pdl_wait();
    __shared__ double a;
    if (threadIdx.x == 0) a = 1.0 / sqrt(fmax(*s, 0.0));
    __syncthreads();
    const double f = a;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] *= f;
}

void scale_rnorm(Ctx& ctx, double* x, int64_t n, int norm_slot) {
    ITG_REQUIRE(norm_slot >= 0 && norm_slot < Ctx::NSCALAR, "scale_rnorm: scalar slot out of range");
    if (n <= 0) return;
    ctx.ensure_scalars();
    launch_pdl(ctx, grid_for(ctx, n), 256, 0, scale_rnorm_kernel, x, n, ctx.scal_dev->as<double>() + norm_slot);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}

__global__ void scale_rnorm_min_kernel(double* x, int64_t n, double const* __restrict__ s, double min_norm) {
    pdl_wait();
    __shared__ double a;
    if (threadIdx.x == 0) {
        const double nr = sqrt(fmax(*s, 0.0));
        a = nr > min_norm ? 1.0 / nr : 1.0;
    }
    __syncthreads();
    const double f = a;
    if (f == 1.0) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] *= f;
}

void normalize_async(Ctx& ctx, double* x, int64_t n, double min_norm) {
    if (n <= 0) return;
    constexpr int slot = Ctx::NSCALAR - 1;
    VecList V;
    V.add(x, 1.0);
    dots_async(ctx, V, x, n, slot);
    launch_pdl(ctx, grid_for(ctx, n), 256, 0, scale_rnorm_min_kernel, x, n, ctx.scal_dev->as<double>() + slot, min_norm);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}

static bool uses_slots(VecList const& X) {
    for (int k = 0; k < X.n; ++k)
        if (X.cs[k] >= 0) {
            ITG_REQUIRE(X.cs[k] < Ctx::NSCALAR, "combo: scalar slot out of range");
            return true;
        }
    return false;
}

double combo(Ctx& ctx, double* y, double a0, VecList const& X, int64_t n, bool want_norm) {
    ITG_REQUIRE(X.n >= 0 && X.n <= VecList::MAX, "combo: too many terms");
    if (n <= 0) return 0.0;
    ctx.ensure_reduce();
    ctx.ensure_pin(sizeof(double));
    if (uses_slots(X)) ctx.ensure_scalars();
    double* part = ctx.reduce_buf->as<double>();
    unsigned int* counter = reinterpret_cast<unsigned int*>(part + REDUCE_DOUBLES - 2);
    const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(DOT_CTAS, (n + 255) / 256));
    launch_pdl(ctx, nb, 256, 0, combo_kernel, y, a0, X, n, want_norm ? 1 : 0, part, counter,
                                             static_cast<double*>(ctx.pin_dev), nullptr,
                                             ctx.scal_dev ? ctx.scal_dev->as<double>() : nullptr);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
    if (!want_norm) return 0.0;
    ctx.sync();
    return *static_cast<double*>(ctx.pin);
}

void combo_async(Ctx& ctx, double* y, double a0, VecList const& X, int64_t n, int norm_slot) {
    ITG_REQUIRE(X.n >= 0 && X.n <= VecList::MAX, "combo: too many terms");
    ITG_REQUIRE(norm_slot < Ctx::NSCALAR, "combo: scalar slot out of range");
    if (n <= 0) return;
    ctx.ensure_reduce();
    ctx.ensure_scalars();
    uses_slots(X);
    double* part = ctx.reduce_buf->as<double>();
    unsigned int* counter = reinterpret_cast<unsigned int*>(part + REDUCE_DOUBLES - 2);
    const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(DOT_CTAS, (n + 255) / 256));
    double* sd = ctx.scal_dev->as<double>();
    launch_pdl(ctx, nb, 256, 0, combo_kernel, y, a0, X, n, norm_slot >= 0 ? 1 : 0, part, counter,
                                             norm_slot >= 0 ? ctx.scal_map + norm_slot : nullptr,
                                             norm_slot >= 0 ? sd + norm_slot : nullptr, sd);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}

// ------------------------------------------------------------------ gather
// dst[doff + d1[i] + d2[j]] = src[soff + s1[i] + s2[j]], i < n1 (fastest), j < n2
__global__ void gather_kernel(GatherItem const* __restrict__ items, int32_t const* __restrict__ tab,
                              double const* __restrict__ src, double* __restrict__ dst) {
    pdl_wait();
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
    char* st = ctx.stage_ring(bytes);
    if (!items.empty()) std::memcpy(st + o_items, items.data(), sizeof(GatherItem) * items.size());
    if (!tab.empty()) std::memcpy(st + o_tab, tab.data(), sizeof(int32_t) * tab.size());
    dev = dev_alloc(bytes, ctx.stream);
    ctx.ring_copy(dev->as<char>(), st, bytes);
    d_items = reinterpret_cast<GatherItem*>(dev->as<char>() + o_items);
    d_tab = reinterpret_cast<int32_t*>(dev->as<char>() + o_tab);
    nitems = (int)items.size();
}

void launch_gather(Ctx& ctx, GatherPlan const& g, double const* src, double* dst) {
    if (g.nitems == 0) return;
    launch_pdl(ctx, g.nitems, 256, 0, gather_kernel, g.d_items, g.d_tab, src, dst);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}

// ------------------------------------------------------------------ noisy density matrix
// rho + noise * deltaRho with deltaRho's Hermitian part (itensor/mps/localop.h:399-403):
// one CTA per diagonal block.
// rho and out may be the same buffer (a later pass accumulates in place): each
// element is read and written by the same thread.
__global__ void noisy_rho_kernel(NoiseBlock const* __restrict__ blocks, double const* rho,
                                 double const* __restrict__ d, double* out, double half_noise) {
    pdl_wait();
    const NoiseBlock bk = blocks[blockIdx.x];
    const int64_t n = bk.n;
    for (int64_t e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int64_t i = e % n, j = e / n;
        double v = bk.rho_off >= 0 ? rho[bk.rho_off + e] : 0.0;
        if (bk.d_off >= 0) v = fma(half_noise, d[bk.d_off + e] + d[bk.d_off + i * n + j], v);
        out[bk.out_off + e] = v;
    }
}

// Trace over every block's diagonal in a fixed order (one CTA, deterministic),
// then the scale 1/tr applied by all CTAs when tr > 1e-16.
constexpr int TRACE_THREADS = 256;
__global__ void block_trace_kernel(NoiseBlock const* __restrict__ blocks, int nb, double const* __restrict__ out,
                                   double* __restrict__ tr) {
    pdl_wait();
    __shared__ double part[TRACE_THREADS];
    double s = 0.0;
    for (int b = 0; b < nb; ++b) {
        const NoiseBlock bk = blocks[b];
        for (int64_t i = threadIdx.x; i < bk.n; i += blockDim.x) s += out[bk.out_off + i * (bk.n + 1)];
    }
    part[threadIdx.x] = s;
    __syncthreads();
    for (int w = TRACE_THREADS / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *tr = part[0];
}
__global__ void trace_normalise_kernel(double* __restrict__ x, int64_t n, double const* __restrict__ tr) {
    pdl_wait();
    const double t = *tr;
    if (!(t > 1e-16)) return;
    const double inv = 1.0 / t;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] *= inv;
}

void launch_noisy_rho(Ctx& ctx, std::vector<std::vector<NoiseBlock>> const& passes, double const* rho,
                      std::vector<double const*> const& ds, double* out, int64_t out_size, double noise) {
    if (passes.empty() || passes[0].empty()) return;
    const size_t nb = passes[0].size(), pbytes = sizeof(NoiseBlock) * nb;
    const size_t bytes = pbytes * passes.size();
    char* st = ctx.stage_ring(bytes);
    for (size_t k = 0; k < passes.size(); ++k) {
        ITG_REQUIRE(passes[k].size() == nb, "noisy_rho: passes over different block lists");
        std::memcpy(st + k * pbytes, passes[k].data(), pbytes);
    }
    DevBuf tab(bytes + 16, ctx.stream);
    ctx.ring_copy(tab.as<char>(), st, bytes);
    double* dtr = reinterpret_cast<double*>(tab.as<char>() + bytes);
    // pass 0: out = rho + noise (D_0 + D_0^T)/2; pass k: out += noise (D_k + D_k^T)/2 (in place)
    for (size_t k = 0; k < passes.size(); ++k) {
        NoiseBlock const* dblocks = reinterpret_cast<NoiseBlock const*>(tab.as<char>() + k * pbytes);
        launch_pdl(ctx, (int)nb, 256, 0, noisy_rho_kernel, dblocks, k == 0 ? rho : out, ds[k], out, 0.5 * noise);
        ITG_CHECK_CUDA(cudaGetLastError());
    }
    NoiseBlock const* dblocks0 = reinterpret_cast<NoiseBlock const*>(tab.as<char>());
    launch_pdl(ctx, 1, TRACE_THREADS, 0, block_trace_kernel, dblocks0, (int)nb, out, dtr);
    ITG_CHECK_CUDA(cudaGetLastError());
    launch_pdl(ctx, grid_for(ctx, out_size), 256, 0, trace_normalise_kernel, out, out_size, dtr);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches += passes.size() + 2;
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
