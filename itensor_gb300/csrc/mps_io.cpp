// MPS / MPO checkpoints in the reference's binary layout (see mps_io.h).
#include "mps_io.h"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>

namespace itg {

namespace {

constexpr int32_t TYPE_NULL = 0;         // StorageType::Null, itensor/itdata/task_types.h:456-471
constexpr int32_t TYPE_QDENSE_REAL = 6;  // StorageType::QDenseReal

// Bounds-checked reader: a truncated or malformed file is an argument error.
struct In {
    std::vector<char> buf;
    size_t p = 0;
    std::string path;
    void raw(void* dst, size_t n) {
        if (n > buf.size() - p) throw Error(ERR_ARG, "checkpoint " + path + ": file ends early (at byte " + std::to_string(p) + ")");
        std::memcpy(dst, buf.data() + p, n);
        p += n;
    }
    template <typename T> T get() {
        T v;
        raw(&v, sizeof v);
        return v;
    }
    // counts are size_t on disk; a count beyond the bytes left is malformed
    uint64_t count(size_t elem_bytes) {
        uint64_t n = get<uint64_t>();
        if (elem_bytes && n > (buf.size() - p) / elem_bytes)
            throw Error(ERR_ARG, "checkpoint " + path + ": implausible count " + std::to_string(n) + " at byte " +
                                     std::to_string(p - 8));
        return n;
    }
};

struct Out {
    std::vector<char> buf;
    void raw(void const* src, size_t n) {
        auto c = static_cast<char const*>(src);
        buf.insert(buf.end(), c, c + n);
    }
    template <typename T> void put(T v) { raw(&v, sizeof v); }
};

// The reference orders QN entries by their name read as a little-endian
// 64-bit integer (seven characters and a terminating zero; SmallString
// operator<, itensor/smallstring.h:105-109).
int64_t name_key(std::array<char, 7> const& n) {
    unsigned char b[8] = {};
    std::memcpy(b, n.data(), 7);
    uint64_t u = 0;
    for (int i = 7; i >= 0; --i) u = (u << 8) | b[i];
    return (int64_t)u;
}
bool name_empty(std::array<char, 7> const& n) { return n[0] == 0; }

FileIndex read_index(In& in) {
    FileIndex I;
    in.raw(I.tags.data(), TAG_BYTES);
    I.plev = in.get<int32_t>();
    I.id = in.get<uint64_t>();
    I.dim = in.get<int32_t>();
    I.dir = in.get<int32_t>();
    uint64_t ns = in.count(4 * (7 + 8) + 8);
    I.sectors.resize(ns);
    for (auto& s : I.sectors) {
        for (auto& q : s.qn) {
            in.raw(q.name.data(), 7);
            q.val = in.get<int32_t>();
            q.mod = in.get<int32_t>();
        }
        s.size = in.get<int64_t>();
    }
    return I;
}

void write_index(Out& o, FileIndex const& I) {
    o.raw(I.tags.data(), TAG_BYTES);
    o.put<int32_t>(I.plev);
    o.put<uint64_t>(I.id);
    o.put<int32_t>(I.dim);
    o.put<int32_t>(I.dir);
    o.put<uint64_t>(I.sectors.size());
    for (auto const& s : I.sectors) {
        for (auto const& q : s.qn) {
            o.raw(q.name.data(), 7);
            o.put<int32_t>(q.val);
            o.put<int32_t>(q.mod);
        }
        o.put<int64_t>(s.size);
    }
}

FileTensor read_tensor(In& in) {
    FileTensor T;
    uint64_t r = in.count(28 + 4 + 8 + 4 + 4 + 8 + 8);
    for (uint64_t k = 0; k < r; ++k) {
        T.inds.push_back(read_index(in));
        T.strides.push_back(in.get<uint64_t>());
    }
    T.lognum = in.get<double>();
    T.sign = in.get<int32_t>();
    T.type = in.get<int32_t>();
    if (T.type == TYPE_NULL) return T;
    if (T.type != TYPE_QDENSE_REAL)
        throw Error(ERR_ARG, "checkpoint " + in.path + ": storage type " + std::to_string(T.type) +
                                 " is not supported (only QN block-sparse real tensors)");
    uint64_t nb = in.count(8 + 8);
    T.blocks.resize(nb);
    T.offsets.resize(nb);
    for (uint64_t b = 0; b < nb; ++b) {
        uint64_t br = in.count(8);
        T.blocks[b].resize(br);
        in.raw(T.blocks[b].data(), 8 * br);
        T.offsets[b] = in.get<int64_t>();
    }
    uint64_t n = in.count(8);
    T.data.resize(n);
    in.raw(T.data.data(), 8 * n);
    return T;
}

void write_tensor(Out& o, FileTensor const& T) {
    o.put<uint64_t>(T.inds.size());
    for (size_t k = 0; k < T.inds.size(); ++k) {
        write_index(o, T.inds[k]);
        o.put<uint64_t>(T.strides[k]);
    }
    o.put<double>(T.lognum);
    o.put<int32_t>(T.sign);
    o.put<int32_t>(T.type);
    if (T.type == TYPE_NULL) return;
    o.put<uint64_t>(T.blocks.size());
    for (size_t b = 0; b < T.blocks.size(); ++b) {
        o.put<uint64_t>(T.blocks[b].size());
        o.raw(T.blocks[b].data(), 8 * T.blocks[b].size());
        o.put<int64_t>(T.offsets[b]);
    }
    o.put<uint64_t>(T.data.size());
    o.raw(T.data.data(), 8 * T.data.size());
}

// Union of the QN names of every index, ordered as the reference orders them.
std::vector<std::array<char, 7>> collect_names(MpsFile const& f) {
    std::vector<std::array<char, 7>> names;
    for (auto const& T : f.A)
        for (auto const& I : T.inds)
            for (auto const& s : I.sectors)
                for (auto const& q : s.qn) {
                    if (name_empty(q.name) && q.mod == 0) continue;
                    if (std::find(names.begin(), names.end(), q.name) == names.end()) names.push_back(q.name);
                }
    std::sort(names.begin(), names.end(),
              [](auto const& a, auto const& b) { return name_key(a) < name_key(b); });
    ITG_REQUIRE(names.size() <= (size_t)QN_SLOTS, "checkpoint: more than four quantum-number names");
    return names;
}

Index to_index(FileIndex const& fi, std::vector<std::array<char, 7>> const& names) {
    ITG_REQUIRE(fi.dir == 1 || fi.dir == -1, "checkpoint: index arrow must be In or Out");
    ITG_REQUIRE(!fi.sectors.empty(), "checkpoint: an index without QN sectors (only QN tensors are supported)");
    std::vector<QN> qs(fi.sectors.size());
    std::vector<int32_t> dims(fi.sectors.size());
    int64_t tot = 0;
    for (size_t s = 0; s < fi.sectors.size(); ++s) {
        auto const& fs = fi.sectors[s];
        ITG_REQUIRE(fs.size > 0 && fs.size < (int64_t(1) << 31), "checkpoint: bad sector size");
        dims[s] = (int32_t)fs.size;
        tot += fs.size;
        for (auto const& q : fs.qn) {
            if (name_empty(q.name) && q.mod == 0) continue;
            int k = (int)(std::find(names.begin(), names.end(), q.name) - names.begin());
            qs[s].mod[k] = q.mod;
            qs[s].v[k] = QN::reduce(q.val, q.mod);
        }
    }
    ITG_REQUIRE(tot == fi.dim, "checkpoint: index dimension differs from the sum of its sectors");
    Index I(qs, dims, fi.dir, fi.id, fi.plev);
    I.tags = fi.tags;
    return I;
}

FileIndex from_index(Index const& I, std::vector<std::array<char, 7>> const& names) {
    FileIndex fi;
    fi.tags = I.tags;
    fi.plev = I.plev;
    fi.id = I.id;
    fi.dim = (int32_t)I.dim();
    fi.dir = I.dir;
    // entries in the reference's name order, packed to the front
    std::vector<int> order;
    for (int k = 0; k < (int)names.size(); ++k) order.push_back(k);
    std::sort(order.begin(), order.end(), [&](int a, int b) { return name_key(names[a]) < name_key(names[b]); });
    for (int s = 0; s < I.nblock(); ++s) {
        FileSector fs;
        fs.size = I.bdim(s);
        int n = 0;
        for (int k : order) {
            if (I.qn(s).mod[k] == 0) continue;
            fs.qn[n].name = names[k];
            fs.qn[n].val = I.qn(s).v[k];
            fs.qn[n].mod = I.qn(s).mod[k];
            ++n;
        }
        fi.sectors.push_back(fs);
    }
    return fi;
}

}  // namespace

MpsFile read_mps_file(std::string const& path) {
    In in;
    in.path = path;
    std::ifstream s(path, std::ios::binary);
    if (!s.good()) throw Error(ERR_ARG, "checkpoint: cannot open " + path + " for reading");
    in.buf.assign(std::istreambuf_iterator<char>(s), std::istreambuf_iterator<char>());
    MpsFile f;
    f.N = in.get<int32_t>();
    ITG_REQUIRE(f.N >= 1 && f.N < (1 << 20), "checkpoint " + path + ": bad number of sites");
    for (int j = 0; j < f.N + 2; ++j) f.A.push_back(read_tensor(in));
    f.leftlim = in.get<int32_t>();
    f.rightlim = in.get<int32_t>();
    ITG_REQUIRE(in.p == in.buf.size(), "checkpoint " + path + ": trailing bytes after the MPS");
    ITG_REQUIRE(f.A[0].type == TYPE_NULL && f.A[f.N + 1].type == TYPE_NULL,
                "checkpoint " + path + ": the boundary tensors must be empty");
    for (int j = 1; j <= f.N; ++j)
        ITG_REQUIRE(f.A[j].type == TYPE_QDENSE_REAL, "checkpoint " + path + ": site tensor " + std::to_string(j) +
                                                         " is not a QN block-sparse real tensor");
    f.qn_names = collect_names(f);
    return f;
}

void write_mps_file(MpsFile const& f, std::string const& path) {
    ITG_REQUIRE((int)f.A.size() == f.N + 2, "checkpoint: an MPS holds N + 2 tensors");
    Out o;
    o.put<int32_t>(f.N);
    for (auto const& T : f.A) write_tensor(o, T);
    o.put<int32_t>(f.leftlim);
    o.put<int32_t>(f.rightlim);
    std::ofstream s(path, std::ios::binary);
    if (!s.good()) throw Error(ERR_ARG, "checkpoint: cannot open " + path + " for writing");
    s.write(o.buf.data(), (std::streamsize)o.buf.size());
    if (!s.good()) throw Error(ERR_ARG, "checkpoint: write to " + path + " failed");
}

std::vector<Tensor> load_mps(Ctx& ctx, MpsFile const& f) {
    std::vector<Tensor> out;
    for (int j = 1; j <= f.N; ++j) {
        FileTensor const& T = f.A[j];
        auto L = std::make_shared<Layout>();
        for (auto const& fi : T.inds) L->inds.push_back(to_index(fi, f.qn_names));
        const int r = L->rank();
        ITG_REQUIRE(r > 0, "checkpoint: a site tensor without indices");
        QN div;
        for (size_t b = 0; b < T.blocks.size(); ++b) {
            ITG_REQUIRE((int)T.blocks[b].size() == r, "checkpoint: block coordinates of the wrong rank");
            for (int k = 0; k < r; ++k) {
                int64_t c = T.blocks[b][k];
                ITG_REQUIRE(c >= 0 && c < L->inds[k].nblock(), "checkpoint: block coordinate out of range");
                L->coords.push_back((int32_t)c);
            }
            if (b > 0)
                ITG_REQUIRE(coords_less(L->block((int)b - 1), L->block((int)b), r),
                            "checkpoint: blocks not in storage order");
            QN q = L->flux(L->block((int)b));
            if (b == 0) div = q;
            ITG_REQUIRE(q == div, "checkpoint: blocks of different flux in one tensor");
        }
        L->finish();
        ITG_REQUIRE((int64_t)T.data.size() == L->size, "checkpoint: data size differs from the blocks'");
        for (size_t b = 0; b < T.blocks.size(); ++b)
            ITG_REQUIRE(T.offsets[b] == L->offs[b], "checkpoint: block offsets differ from the packed layout");
        std::vector<double> host = T.data;
        if (!(T.lognum == 0.0 && T.sign == 1)) {
            const double sc = T.sign == 0 ? 0.0 : T.sign * std::exp(T.lognum);
            for (auto& x : host) x *= sc;
        }
        out.push_back(upload_tensor(ctx, L, host.data()));
    }
    return out;
}

MpsFile store_mps(Ctx& ctx, std::vector<Tensor> const& sites, int leftlim, int rightlim,
                  std::vector<std::array<char, 7>> const& qn_names) {
    ITG_REQUIRE(!sites.empty(), "checkpoint: no site tensors");
    ITG_REQUIRE(qn_names.size() <= (size_t)QN_SLOTS, "checkpoint: more than four quantum-number names");
    MpsFile f;
    f.N = (int32_t)sites.size();
    f.leftlim = leftlim;
    f.rightlim = rightlim;
    f.qn_names = qn_names;
    f.A.emplace_back();
    for (auto const& S : sites) {
        ITG_REQUIRE(S.valid() && S.rank() > 0, "checkpoint: a site tensor without indices");
        for (auto const& I : S.inds())
            for (int s = 0; s < I.nblock(); ++s)
                for (int k = 0; k < QN_SLOTS; ++k)
                    ITG_REQUIRE(I.qn(s).mod[k] == 0 || k < (int)qn_names.size(),
                                "checkpoint: a quantum number in a slot that has no name");
        FileTensor T;
        T.type = TYPE_QDENSE_REAL;
        uint64_t stride = 1;
        for (auto const& I : S.inds()) {
            T.inds.push_back(from_index(I, qn_names));
            T.strides.push_back(stride);
            stride *= (uint64_t)I.dim();
        }
        Layout const& L = *S.lay;
        for (int b = 0; b < L.nblocks(); ++b) {
            T.blocks.emplace_back(L.block(b), L.block(b) + L.rank());
            T.offsets.push_back(L.offs[b]);
        }
        T.data = download(ctx, S);
        f.A.push_back(std::move(T));
    }
    f.A.emplace_back();
    return f;
}

}  // namespace itg
