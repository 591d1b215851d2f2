// Host-side data model of the block-sparse QN tensors whose blocks live in
// device memory.
//
// Layout conventions follow ITensor's QDense storage (itensor/itdata/qdense.h:34-187):
//   * a block is identified by one sector number per index, stored only if its
//     flux sum(dir*qn) equals the tensor's divergence
//     (getBlockOffsets, itensor/itdata/qdense.cc:134-171);
//   * blocks are dense and column-major (first index fastest);
//   * blocks are ordered by reversed-lexicographic coordinates
//     (operator<, itensor/itdata/qdense.cc:60-65) and packed back to back
//     (offsets = prefix sum of block sizes).
// Two indices contract when id and prime level agree (computeLabels,
// itensor/tensor/contract.h:155-216).
#pragma once
#include "common.h"
#include <algorithm>
#include <array>
#include <cstring>
#include <functional>

namespace itg {

constexpr int QN_SLOTS = 4;

// Up to four quantum numbers. mod[k] > 1: value taken modulo mod[k]
// (Z_n); |mod| == 1: plain integer (U(1)); mod < 0 marks a fermionic U(1)
// (bookkeeping only, as in itensor/qn.h:36-60); mod == 0: unused slot.
struct QN {
    std::array<int32_t, QN_SLOTS> v{};
    std::array<int32_t, QN_SLOTS> mod{};

    static int32_t reduce(int32_t x, int32_t m) {
        int32_t am = m < 0 ? -m : m;
        if (am > 1) return ((x % am) + am) % am;
        return x;
    }
    QN operator+(QN const& o) const {
        QN r;
        for (int k = 0; k < QN_SLOTS; ++k) {
            r.mod[k] = mod[k] ? mod[k] : o.mod[k];
            r.v[k] = reduce(v[k] + o.v[k], r.mod[k]);
        }
        return r;
    }
    QN operator-() const {
        QN r;
        for (int k = 0; k < QN_SLOTS; ++k) {
            r.mod[k] = mod[k];
            r.v[k] = reduce(-v[k], mod[k]);
        }
        return r;
    }
    QN operator-(QN const& o) const { return *this + (-o); }
    QN times(int dir) const { return dir >= 0 ? *this : -*this; }
    bool operator==(QN const& o) const { return v == o.v; }
    bool operator!=(QN const& o) const { return !(*this == o); }
};

// Sector list of an index (shared between copies of the index).
struct Sectors {
    std::vector<QN> qn;
    std::vector<int32_t> dim;
    int64_t total = 0;
    std::vector<int64_t> start;  // first position of each sector within the index
    void finish() {
        total = 0;
        start.resize(dim.size());
        for (size_t i = 0; i < dim.size(); ++i) { start[i] = total; total += dim[i]; }
    }
};

uint64_t new_index_id();

constexpr int TAG_BYTES = 28;  // four tags of seven characters (TagSet, itensor/tagset.h:35)

struct Index {
    uint64_t id = 0;
    int32_t plev = 0;
    int32_t dir = 1;  // +1 Out, -1 In
    std::shared_ptr<const Sectors> sec;
    // Tags as the reference stores them (carried through unchanged; only
    // the checkpoint files read or write them). All zero: no tags.
    std::array<char, TAG_BYTES> tags{};

    Index() = default;
    Index(std::vector<QN> qn, std::vector<int32_t> dims, int dir_, uint64_t id_ = 0, int plev_ = 0) {
        auto s = std::make_shared<Sectors>();
        s->qn = std::move(qn);
        s->dim = std::move(dims);
        s->finish();
        sec = s;
        dir = dir_;
        id = id_ ? id_ : new_index_id();
        plev = plev_;
    }
    int nblock() const { return (int)sec->dim.size(); }
    int32_t bdim(int b) const { return sec->dim[b]; }
    QN const& qn(int b) const { return sec->qn[b]; }
    int64_t dim() const { return sec->total; }
    bool same(Index const& o) const { return id == o.id && plev == o.plev; }
    Index dag() const { Index r = *this; r.dir = -dir; return r; }
    Index prime(int inc = 1) const { Index r = *this; r.plev += inc; return r; }
    Index noprime() const { Index r = *this; r.plev = 0; return r; }
};

// Block structure of a tensor (no data).
struct Layout {
    std::vector<Index> inds;
    std::vector<int32_t> coords;   // nblocks * rank, sorted reversed-lexicographically
    std::vector<int64_t> offs;     // element offset of each block
    int64_t size = 0;              // total elements

    int rank() const { return (int)inds.size(); }
    int nblocks() const { return (int)offs.size(); }
    int32_t const* block(int b) const { return coords.data() + (size_t)b * rank(); }
    int64_t block_size(int b) const {
        int64_t s = 1;
        for (int k = 0; k < rank(); ++k) s *= inds[k].bdim(block(b)[k]);
        return s;
    }
    QN flux(int32_t const* c) const {
        QN q;
        for (int k = 0; k < rank(); ++k) q = q + inds[k].qn(c[k]).times(inds[k].dir);
        return q;
    }
    // Recompute offsets from coords (coords must be sorted).
    void finish() {
        int nb = rank() ? (int)(coords.size() / rank()) : 1;
        offs.resize(nb);
        int64_t tot = 0;
        for (int b = 0; b < nb; ++b) { offs[b] = tot; tot += rank() ? block_size(b) : 1; }
        size = tot;
    }
    int find_block(int32_t const* c) const;  // -1 if absent (binary search)
    int find_index(Index const& I) const {
        for (int k = 0; k < rank(); ++k) if (inds[k].same(I)) return k;
        return -1;
    }
};

bool coords_less(int32_t const* a, int32_t const* b, int rank);  // reversed-lexicographic

// All blocks with flux == div, in storage order.
Layout allowed_layout(std::vector<Index> const& inds, QN const& div);
// Layout with an explicit (unsorted) block list; sorts and computes offsets.
Layout make_layout(std::vector<Index> const& inds, std::vector<int32_t> coords);

struct Tensor {
    std::shared_ptr<Layout> lay;
    DevBufPtr buf;       // lay->size doubles
    double scalar = 0;   // value of a rank-0 result

    Tensor() = default;
    Tensor(std::shared_ptr<Layout> l, cudaStream_t s) : lay(std::move(l)) {
        buf = dev_alloc(sizeof(double) * std::max<int64_t>(lay->size, 1), s);
    }
    double* data() const { return buf ? buf->as<double>() : nullptr; }
    std::vector<Index> const& inds() const { return lay->inds; }
    int rank() const { return lay->rank(); }
    bool valid() const { return (bool)lay; }
};

// Same data, different index labels (prime / dag / noprime); block structure unchanged.
Tensor relabel(Tensor const& t, std::vector<Index> inds);

}  // namespace itg
