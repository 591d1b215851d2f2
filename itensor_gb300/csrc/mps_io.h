// MPS / MPO checkpoints in the reference's plain binary layout, read and
// written on the host, loaded onto and stored from the device.
//
// The layout is the one writeToFile/readFromFile produce for an MPS or MPO
// (itensor/util/readwrite.h:337-370): little-endian raw values, in order
//   MPS      int N; N+2 ITensors (A_0 .. A_{N+1}); int leftLim; int rightLim
//            (MPS::write/read, itensor/mps/mps.cc:353-378; an MPO is written
//            the same way, itensor/mps/mpo.h:26-57)
//   ITensor  IndexSet; LogNum scale (double log|s|, int sign); int storage type;
//            the storage (ITensor::write, itensor/itensor.cc:769-803)
//   IndexSet size_t n; n x (Index, size_t stride)  (RangeT storage,
//            itensor/tensor/range.h:52-74,286-298)
//   Index    TagSet (4 x 7 chars, int prime level); uint64 id; int dim;
//            int arrow; size_t nsect; nsect x (QN, long size)
//            (Index::write itensor/index.cc:712-721, TagSet itensor/tagset.cc:265-271,
//            QNInt itensor/index.cc:562-573)
//   QN       4 x (7-char name, int value, int modulus)  (itensor/qn.cc:88-106,499-509)
//   QDense   size_t nblocks; nblocks x (size_t rank, rank x long, long offset);
//            size_t n; n x double  (itensor/itdata/qdense.h:236-248,
//            BlOf itensor/util/readwrite.h:319-331)
// Only QN block-sparse real storage (type 6) and empty tensors (type 0) occur
// in the MPS and MPO this path handles; other storage types are refused.
#pragma once
#include "algo.h"
#include <string>

namespace itg {

struct FileQNum {
    std::array<char, 7> name{};
    int32_t val = 0, mod = 0;
};
struct FileSector {
    std::array<FileQNum, 4> qn;
    int64_t size = 0;
};
struct FileIndex {
    std::array<char, TAG_BYTES> tags{};
    int32_t plev = 0;
    uint64_t id = 0;
    int32_t dim = 0;
    int32_t dir = 1;
    std::vector<FileSector> sectors;
};
struct FileTensor {
    std::vector<FileIndex> inds;
    std::vector<uint64_t> strides;
    double lognum = 0.0;
    int32_t sign = 1;
    int32_t type = 0;                      // 0 empty, 6 QN block-sparse real
    std::vector<std::vector<int64_t>> blocks;
    std::vector<int64_t> offsets;
    std::vector<double> data;
};
struct MpsFile {
    int32_t N = 0;
    std::vector<FileTensor> A;             // N + 2 tensors, A[0] and A[N+1] empty
    int32_t leftlim = 0, rightlim = 0;
    // QN names in slot order: slot k of the device QNs holds the quantum
    // number called qn_names[k] (names in the order the file's QNs list them)
    std::vector<std::array<char, 7>> qn_names;
};

MpsFile read_mps_file(std::string const& path);
void write_mps_file(MpsFile const& f, std::string const& path);
// Site tensors 1..N onto the device (scale folded into the data).
std::vector<Tensor> load_mps(Ctx& ctx, MpsFile const& f);
// Site tensors from the device; QN slot k is written under qn_names[k].
MpsFile store_mps(Ctx& ctx, std::vector<Tensor> const& sites, int leftlim, int rightlim,
                  std::vector<std::array<char, 7>> const& qn_names);

}  // namespace itg
