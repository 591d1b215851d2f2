"""Independent reader of the reference's binary MPS/MPO layout, for tests.

The layout follows writeToFile(path, psi) of the reference
(itensor/util/readwrite.h:337-370; MPS::write itensor/mps/mps.cc:365-378;
ITensor::write itensor/itensor.cc:769-784; Index::write itensor/index.cc:712-721;
TagSet itensor/tagset.cc:265-271; QNum itensor/qn.cc:100-106; QDense
itensor/itdata/qdense.h:236-241). Tensors come back in the fixtures' JSON form
(inds with id/plev/dir/tags/sectors, blocks, offsets, data), which
oracle.blocksparse.BSTensor.from_json reads.
"""
import struct


class _Reader:
    def __init__(self, b):
        self.b, self.p = b, 0

    def get(self, fmt):
        v = struct.unpack_from("<" + fmt, self.b, self.p)
        self.p += struct.calcsize("<" + fmt)
        return v if len(v) > 1 else v[0]

    def chars(self, n):
        s = self.b[self.p:self.p + n]
        self.p += n
        return s


def _index(r):
    tags = [r.chars(7).rstrip(b"\0").decode() for _ in range(4)]
    plev = r.get("i")
    iid = r.get("Q")
    dim = r.get("i")
    dr = r.get("i")
    sectors = []
    for _ in range(r.get("Q")):
        qn = []
        for _ in range(4):
            name = r.chars(7).rstrip(b"\0").decode()
            val, mod = r.get("ii")
            if name or mod:
                qn.append([name, val, mod])
        sectors.append([qn, r.get("q")])
    assert sum(s for _, s in sectors) == dim
    return dict(id=str(iid), plev=plev, dir=dr, tags=",".join(t for t in tags if t), sectors=sectors)


def _tensor(r):
    inds = []
    for _ in range(r.get("Q")):
        inds.append(_index(r))
        r.get("Q")  # stride
    lognum, sign = r.get("d"), r.get("i")
    typ = r.get("i")
    if typ == 0:
        return None
    assert typ == 6, "only QN block-sparse real storage"
    blocks, offsets = [], []
    for _ in range(r.get("Q")):
        n = r.get("Q")
        blocks.append(list(struct.unpack_from("<%dq" % n, r.b, r.p)))
        r.p += 8 * n
        offsets.append(r.get("q"))
    n = r.get("Q")
    data = list(struct.unpack_from("<%dd" % n, r.b, r.p))
    r.p += 8 * n
    if not (lognum == 0.0 and sign == 1):
        import math
        sc = 0.0 if sign == 0 else sign * math.exp(lognum)
        data = [x * sc for x in data]
    return dict(inds=inds, blocks=blocks, offsets=offsets, data=data)


def read(path):
    """(site tensors 1..N as fixture dicts, leftLim, rightLim)."""
    r = _Reader(open(path, "rb").read())
    N = r.get("i")
    A = [_tensor(r) for _ in range(N + 2)]
    lims = r.get("ii")
    assert r.p == len(r.b), "trailing bytes"
    assert A[0] is None and A[N + 1] is None
    return A[1:N + 1], lims[0], lims[1]
