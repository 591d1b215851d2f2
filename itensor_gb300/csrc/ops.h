// Gather plans and the batched eigensolver interface (kernels in ops.cu).
#pragma once
#include "engine.h"
#include <mutex>
#include <unordered_map>

namespace itg {

// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) for kernel f only when
// `bytes` exceeds what was set for it before (the attribute lasts for the
// process; it only grows, so a concurrent launch with less never sees it
// shrink). Saves a driver call on most launches of the eigensolver kernels.
inline void grow_smem_attr(void const* f, size_t bytes) {
    if (bytes <= 48 * 1024) return;
    static std::mutex mu;
    static std::unordered_map<void const*, size_t> set;
    std::lock_guard<std::mutex> g(mu);
    size_t& cur = set[f];
    if (bytes <= cur) return;
    ITG_CHECK_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    cur = bytes;
}

struct GatherItem {
    int64_t soff, doff;
    int32_t n1, n2;        // element grid n1 x n2 (n1 fastest)
    int32_t ts1, ts2;      // table positions of source offsets along 1 and 2
    int32_t td1, td2;      // table positions of destination offsets along 1 and 2
};

struct GatherPlan {
    std::vector<GatherItem> items;
    std::vector<int32_t> tab;
    DevBufPtr dev;
    GatherItem* d_items = nullptr;
    int32_t* d_tab = nullptr;
    int nitems = 0;
    int32_t add_table(std::vector<int32_t> const& t) {
        int32_t p = (int32_t)tab.size();
        tab.insert(tab.end(), t.begin(), t.end());
        return p;
    }
    void upload(Ctx& ctx);
};

// One diagonal block of the noisy density matrix (denmat_decomp with noise):
// out = rho + noise * (D + D^T) / 2 on an n x n block; rho_off or d_off < 0
// when that term has no such block.
struct NoiseBlock {
    int64_t out_off, rho_off, d_off;
    int32_t n, pad;
};
// Writes every block of `out` (blocks listed in storage order), then divides
// out by its trace when the trace exceeds 1e-16 (itensor/decomp.h:386-394).
// Device-side throughout: no host wait.
// Several noise terms (a sum of MPOs): one pass per term over the same block
// list, the first from rho, the others added in place; one trace at the end.
void launch_noisy_rho(Ctx& ctx, std::vector<std::vector<NoiseBlock>> const& passes, double const* rho,
                      std::vector<double const*> const& ds, double* out, int64_t out_size, double noise);

// One symmetric n x n matrix (column-major) to diagonalise.
struct EigItem {
    int64_t a_off;   // input matrix in the source buffer
    int64_t v_off;   // eigenvectors (columns, eigenvalues descending) in the output buffer
    int64_t w_off;   // eigenvalues (descending) in the output buffer
    int64_t s_off;   // 2 n^2 doubles of scratch
    int32_t n;
    int32_t pad;
};

// One block to decompose by singular values: X = the m x n (m >= n) matrix read
// from src at a_off with leading dimension ld (transpose != 0: X = that matrix
// transposed, i.e. element (i,j) at a_off + j + i*ld). Outputs, singular
// values descending: U (m x n) at u_off, sigma (n) at s_out, V (n x n) at v_off,
// with X = U diag(sigma) V^T. Scratch: m n + n n + n doubles at s_off.
struct SvdItem {
    int64_t a_off, u_off, v_off, s_off;
    int64_t s_out;
    int32_t rows, cols, ld, transpose;
};
int batched_svd(Ctx& ctx, std::vector<SvdItem> const& items, double const* src, double* uout, double* sout,
                double* vout, double* scratch);

// Diagonalises every item; returns the number of items that hit the sweep cap.
int batched_eigh(Ctx& ctx, std::vector<EigItem> const& items, double const* src, double* vout, double* wout,
                 double* scratch);

}  // namespace itg
