// Allocation-free variant of the split-precision contraction exec.
//
// Some callers cannot let a library allocate device memory during a call:
// code that runs under another framework's allocator which owns the whole
// device pool, real-time loops where an allocation's implicit synchronisation
// is not acceptable, or sandboxes that forbid cudaMalloc after start-up. For
// them, itg_contract_exec_noalloc runs a prepared plan with the
// split-precision digit panels held in a file-scope device array of fixed size
// (ITG_NOALLOC_SCRATCH_BYTES) instead of pool memory. The array exists once
// per device that loads the library, until the process exits.
//
// Set-up: the first call from a CUDA context (the device's primary context,
// or a context the caller created and made current), with that device
// current, looks up the array's device address with cudaGetSymbolAddress (the
// host-side name is only a stand-in, never a device address) and keeps it for
// that context. A later call from another context, or from a new primary
// context after cudaDeviceReset, looks it up again. That first call should
// come before any stream capture.
//
// Every call shares the array and the array keeps the last call's contents.
// Nothing in it has to start at zero: the prep kernel rewrites every digit
// (padding included) and every row exponent a call reads. Calls that overlap
// on the GPU (two streams, or two contexts on one device) race on the array.
#include "../../include/itg.h"
#include "engine.h"
#include <mutex>
#include <vector>

namespace itg {

static __device__ __align__(256) unsigned char g_noalloc_scratch[ITG_NOALLOC_SCRATCH_BYTES];

namespace {
std::mutex g_noalloc_mu;
// The array's address is a property of the CUDA context it was looked up in:
// one entry per (device, context) seen so far.
struct NoallocEntry { int device; void* context; void* ptr; };
std::vector<NoallocEntry> g_noalloc_seen;

typedef int (*CtxGetCurrentFn)(void**);
CtxGetCurrentFn ctx_get_current() {
    static CtxGetCurrentFn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<CtxGetCurrentFn>(f);
    }();
    return fn;
}

void* noalloc_scratch(int device) {
    int cur = -1;
    ITG_CHECK_CUDA(cudaGetDevice(&cur));
    if (cur != device) ITG_CHECK_CUDA(cudaSetDevice(device));
    struct Restore {
        int cur, dev;
        ~Restore() { if (cur != dev) cudaSetDevice(cur); }
    } restore{cur, device};
    CtxGetCurrentFn get = ctx_get_current();
    if (!get) throw Error(ERR_CUDA, "noalloc: cuCtxGetCurrent is not available from the driver");
    void* context = nullptr;
    if (get(&context) != 0 || !context) throw Error(ERR_CUDA, "noalloc: no current CUDA context");
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    for (auto const& e : g_noalloc_seen)
        if (e.device == device && e.context == context) return e.ptr;
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) throw Error(ERR_CUDA, std::string("noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_noalloc_seen.push_back(NoallocEntry{device, context, p});
    return p;
}
}  // namespace

void exec_plan_noalloc(Ctx& ctx, Plan const& p, double const* A, double const* B, double* C, int S) {
    ITG_REQUIRE(S >= 3 && S <= 6, "contract_exec_noalloc: slices must be 3..6");
    if (p.nitems == 0) return;
    // narrow / small-K plans run the FP64 kernels, as itg_contract_exec does; they use no scratch
    if (!plan_uses_split(p, PREC_OZAKI_BF16)) {
        exec_plan_f64_only(ctx, p, A, B, C);
        return;
    }
    const int64_t plane = (p.panel_elems + 15) / 16 * 16;
    const size_t panel_bytes = sizeof(__nv_bfloat16) * (size_t)plane * S;
    const size_t need = split_scratch_bytes(p, S);
    if (need > (size_t)ITG_NOALLOC_SCRATCH_BYTES)
        throw Error(ERR_RANGE, "contract_exec_noalloc: the plan needs " + std::to_string(need) +
                                   " bytes of scratch, the fixed array holds " +
                                   std::to_string((size_t)ITG_NOALLOC_SCRATCH_BYTES));
    unsigned char* base = static_cast<unsigned char*>(noalloc_scratch(ctx.device));
    __nv_bfloat16* panels = reinterpret_cast<__nv_bfloat16*>(base);
    int32_t* exps = reinterpret_cast<int32_t*>(base + panel_bytes);
    launch_ozaki(ctx, p, A, B, C, S, panels, exps);
    ctx.kernel_launches += 2;
    ctx.flops_done += p.flops;
}

}  // namespace itg
