"""Writes a block-sparse tensor in the reference's binary ITensor layout, so
that the reference library (oracle/_ref, where it is built) reads the same
bytes the device path runs on. Test and baseline infrastructure only.

Layout (little-endian), as ITensor::write (itensor/itensor.cc:769-784):
IndexSet (size_t n; n x (Index, size_t stride), itensor/tensor/range.h:52-74,
286-298), LogNum scale (double 0, int 1), int storage type 6 (QDenseReal,
itensor/itdata/task_types.h:456-471), then QDense (size_t nblocks; per block
size_t rank, rank x long coordinates, long offset; size_t n; n doubles;
itensor/itdata/qdense.h:236-241). An Index is TagSet (4 x 7 chars, int prime
level), uint64 id, int dim, int arrow, size_t nsect, per sector 4 x (7-char
QN name, int value, int modulus) and long size (itensor/index.cc:712-721,
itensor/qn.cc:100-106).
"""
import struct

import numpy as np


def _name7(s):
    b = s.encode()[:7]
    return b + b"\0" * (7 - len(b))


def _index(I, qn_name):
    out = b"".join(_name7("") for _ in range(4)) + struct.pack("<i", I["plev"])
    out += struct.pack("<Qii", int(I["id"]), int(sum(I["dims"])), int(I["dir"]))
    out += struct.pack("<Q", len(I["dims"]))
    for q, d in zip(I["qn"], I["dims"]):
        out += _name7(qn_name) + struct.pack("<ii", int(q), 1)
        out += b"".join(_name7("") + struct.pack("<ii", 0, 0) for _ in range(3))
        out += struct.pack("<q", int(d))
    return out


def tensor_bytes(t, qn_name="Sz"):
    """A workload tensor (dict(inds=[dict(id, plev, dir, qn, dims)], coords, data),
    blocks in storage order) as the bytes writeToFile(path, T) gives."""
    inds = t["inds"]
    out = struct.pack("<Q", len(inds))
    stride = 1
    for I in inds:
        out += _index(I, qn_name) + struct.pack("<Q", stride)
        stride *= int(sum(I["dims"]))
    out += struct.pack("<di", 0.0, 1) + struct.pack("<i", 6)
    coords = np.asarray(t["coords"]).reshape(-1, len(inds))
    out += struct.pack("<Q", len(coords))
    off = 0
    for c in coords:
        out += struct.pack("<Q", len(c)) + struct.pack("<%dq" % len(c), *[int(x) for x in c])
        out += struct.pack("<q", off)
        n = 1
        for I, b in zip(inds, c):
            n *= int(I["dims"][int(b)])
        off += n
    data = np.ascontiguousarray(t["data"], dtype="<f8")
    assert data.size == off
    out += struct.pack("<Q", data.size) + data.tobytes()
    return out


def write(path, t, qn_name="Sz"):
    with open(path, "wb") as f:
        f.write(tensor_bytes(t, qn_name))
