"""Block-sparse QN tensors (numpy restatement of ITensor's QDense storage).

Conventions followed from the reference:
  * QN = up to 4 named values with a modulus; |mod|>1 reduces the value
    (itensor/qn.h:36-174). A missing name equals value 0.
  * Index = (id, prime level, arrow, QN sectors); two indices contract when
    id and prime level agree (itensor/index.h:78-282, computeLabels
    itensor/tensor/contract.h:155-216).
  * A tensor stores the blocks whose flux sum(dir*qn) equals its divergence
    (getBlockOffsets itensor/itdata/qdense.cc:134-171). Blocks are dense,
    column-major (first index fastest), ordered by reversed-lexicographic
    block coordinates (operator< itensor/itdata/qdense.cc:60-65); offsets are
    the prefix sum of block sizes.
  * Contraction: output indices are A's uncontracted then B's uncontracted in
    order (contractIS itensor/indexset_impl.h:77-127); output blocks are the
    sorted unique targets of matching block pairs (getContractedOffsets
    itensor/itdata/qutil.h:93-242) -- block-deficient results keep only
    produced blocks.
"""
from __future__ import annotations

import itertools
import numpy as np

OUT, IN = 1, -1


class QN:
    """Named quantum numbers; ``vals`` maps name -> (value, mod)."""
    __slots__ = ("vals",)

    def __init__(self, *items):
        v = {}
        for name, val, mod in items:
            v[name] = (_reduce(val, mod), mod)
        self.vals = v

    @staticmethod
    def from_json(lst):
        return QN(*[(n, int(v), int(m)) for n, v, m in lst])

    def key(self):
        return tuple(sorted((n, v) for n, (v, m) in self.vals.items() if v != 0))

    def __eq__(self, other):
        return self.key() == other.key()

    def __hash__(self):
        return hash(self.key())

    def __add__(self, other):
        out = dict(self.vals)
        for n, (v, m) in other.vals.items():
            if n in out:
                v0, m0 = out[n]
                mm = m0 if m0 != 0 else m
                out[n] = (_reduce(v0 + v, mm), mm)
            else:
                out[n] = (_reduce(v, m), m)
        q = QN()
        q.vals = out
        return q

    def __neg__(self):
        q = QN()
        q.vals = {n: (_reduce(-v, m), m) for n, (v, m) in self.vals.items()}
        return q

    def __sub__(self, other):
        return self + (-other)

    def scaled(self, s):
        return self if s == 1 else -self

    def to_json(self):
        return [[n, v, m] for n, (v, m) in sorted(self.vals.items())]

    def __repr__(self):
        return "QN(%s)" % ",".join("%s=%d" % (n, v) for n, (v, m) in sorted(self.vals.items()))


def _reduce(v, m):
    am = abs(m)
    if am > 1:
        return ((v % am) + am) % am
    return v


_next_id = [1]


def new_id():
    _next_id[0] += 1
    return _next_id[0]


class Index:
    __slots__ = ("id", "plev", "dir", "sectors", "tags")

    def __init__(self, sectors, dir=OUT, tags="", id=None, plev=0):
        self.id = new_id() if id is None else id
        self.plev = plev
        self.dir = dir
        self.sectors = [(q, int(d)) for q, d in sectors]
        self.tags = tags

    @staticmethod
    def from_json(j):
        secs = [(QN.from_json(q), d) for q, d in j["sectors"]]
        return Index(secs, dir=int(j["dir"]), tags=j.get("tags", ""), id=j["id"], plev=int(j["plev"]))

    def same(self, other):
        return self.id == other.id and self.plev == other.plev

    @property
    def dim(self):
        return sum(d for _, d in self.sectors)

    @property
    def nblock(self):
        return len(self.sectors)

    def qn(self, b):
        return self.sectors[b][0]

    def bdim(self, b):
        return self.sectors[b][1]

    def dag(self):
        return Index(self.sectors, -self.dir, self.tags, self.id, self.plev)

    def prime(self, inc=1):
        return Index(self.sectors, self.dir, self.tags, self.id, self.plev + inc)

    def noprime(self):
        return Index(self.sectors, self.dir, self.tags, self.id, 0)

    def __repr__(self):
        return "Index(id=%s,p=%d,dir=%d,%s)" % (self.id, self.plev, self.dir, [(repr(q), d) for q, d in self.sectors])


def rkey(c):
    """Reversed-lexicographic order of block coordinates."""
    return tuple(reversed(c))


def flux(inds, coords):
    q = QN()
    for I, b in zip(inds, coords):
        q = q + I.qn(b).scaled(I.dir)
    return q


class BSTensor:
    """QN block-sparse tensor. ``blocks`` maps coordinate tuples to
    Fortran-ordered arrays with shape = sector sizes."""

    def __init__(self, inds, blocks=None, scalar=None):
        self.inds = list(inds)
        self.blocks = {} if blocks is None else dict(blocks)
        self.scalar = scalar  # rank-0 value

    # ---- construction
    @staticmethod
    def allowed_blocks(inds, div):
        """All blocks with flux == div, in storage order (first index fastest)."""
        out = []
        ranges = [range(I.nblock) for I in inds]
        for c in itertools.product(*reversed(ranges)):
            c = tuple(reversed(c))
            if flux(inds, c) == div:
                out.append(c)
        return out

    @staticmethod
    def zeros(inds, div):
        T = BSTensor(inds)
        for c in BSTensor.allowed_blocks(inds, div):
            T.blocks[c] = np.zeros(T.block_shape(c), order="F")
        return T

    @staticmethod
    def random(inds, div, rng):
        T = BSTensor(inds)
        for c in BSTensor.allowed_blocks(inds, div):
            T.blocks[c] = np.asfortranarray(rng.standard_normal(T.block_shape(c)))
        return T

    @staticmethod
    def from_json(j):
        inds = [Index.from_json(x) for x in j["inds"]]
        if "scalar" in j:
            return BSTensor(inds, scalar=float(j["scalar"]))
        if not inds:
            return BSTensor(inds, scalar=float(j["data"][0]) if j["data"] else 0.0)
        T = BSTensor(inds)
        data = np.asarray(j["data"], dtype=np.float64)
        for c, off in zip(j["blocks"], j["offsets"]):
            c = tuple(int(x) for x in c)
            shp = T.block_shape(c)
            n = int(np.prod(shp)) if shp else 1
            T.blocks[c] = np.reshape(data[off:off + n], shp, order="F").copy(order="F")
        return T

    # ---- layout
    def block_shape(self, c):
        return tuple(I.bdim(b) for I, b in zip(self.inds, c))

    @property
    def order(self):
        return len(self.inds)

    def sorted_coords(self):
        return sorted(self.blocks.keys(), key=rkey)

    def layout(self):
        """(coords list, offsets list, total size) in storage order."""
        cs = self.sorted_coords()
        offs, tot = [], 0
        for c in cs:
            offs.append(tot)
            tot += int(np.prod(self.block_shape(c))) if c else 1
        return cs, offs, tot

    def flat(self):
        cs, offs, tot = self.layout()
        out = np.zeros(tot)
        for c, o in zip(cs, offs):
            b = self.blocks[c]
            out[o:o + b.size] = b.reshape(-1, order="F")
        return out

    def div(self):
        if not self.blocks:
            return QN()
        c = self.sorted_coords()[0]
        return flux(self.inds, c)

    def copy(self):
        return BSTensor(self.inds, {c: b.copy(order="F") for c, b in self.blocks.items()}, self.scalar)

    # ---- index operations
    def dag(self):
        return BSTensor([I.dag() for I in self.inds], self.blocks, self.scalar)

    def prime(self, which=None, inc=1):
        """Prime all indices, or those whose id is in ``which``."""
        inds = [I.prime(inc) if (which is None or I.id in which) else I for I in self.inds]
        return BSTensor(inds, self.blocks, self.scalar)

    def noprime(self):
        return BSTensor([I.noprime() for I in self.inds], self.blocks, self.scalar)

    def find(self, I):
        for k, J in enumerate(self.inds):
            if J.same(I):
                return k
        return -1

    # ---- arithmetic
    def scale(self, a):
        return BSTensor(self.inds, {c: a * b for c, b in self.blocks.items()},
                        None if self.scalar is None else a * self.scalar)

    def norm(self):
        if self.scalar is not None:
            return abs(self.scalar)
        return float(np.sqrt(sum(float(np.vdot(b, b)) for b in self.blocks.values())))

    def permuted_to(self, inds):
        """Same tensor with its indices reordered to match ``inds`` (by id/plev)."""
        perm = [self.find(I) for I in inds]
        if perm == list(range(len(inds))):
            return self
        assert all(p >= 0 for p in perm)
        out = BSTensor([self.inds[p] for p in perm])
        for c, b in self.blocks.items():
            out.blocks[tuple(c[p] for p in perm)] = np.asfortranarray(np.transpose(b, perm))
        return out

    def __add__(self, other):
        """PlusEQ: union of blocks, other permuted to self's index order
        (itensor/itdata/qdense.cc:506-664)."""
        o = other.permuted_to(self.inds)
        out = self.copy()
        for c, b in o.blocks.items():
            if c in out.blocks:
                out.blocks[c] = out.blocks[c] + b
            else:
                out.blocks[c] = b.copy(order="F")
        return out

    def __sub__(self, other):
        return self + other.scale(-1.0)


def contract(A: BSTensor, B: BSTensor) -> BSTensor:
    """C = A*B over all indices common to both (doTask(Contract,QDense,QDense),
    itensor/itdata/qdense.cc:671-743)."""
    rA, rB = A.order, B.order
    AtoB = [-1] * rA
    BtoA = [-1] * rB
    for i in range(rA):
        for j in range(rB):
            if A.inds[i].same(B.inds[j]):
                AtoB[i] = j
                BtoA[j] = i
                break
    a_unc = [i for i in range(rA) if AtoB[i] < 0]
    b_unc = [j for j in range(rB) if BtoA[j] < 0]
    a_con = [i for i in range(rA) if AtoB[i] >= 0]
    b_con = [AtoB[i] for i in a_con]
    Cinds = [A.inds[i] for i in a_unc] + [B.inds[j] for j in b_unc]
    C = BSTensor(Cinds)
    if A.scalar is not None or B.scalar is not None:
        raise ValueError("contract: rank-0 operand")
    acc = {}
    for ca in A.sorted_coords():
        for cb in B.sorted_coords():
            if any(ca[i] != cb[AtoB[i]] for i in a_con):
                continue
            cc = tuple(ca[i] for i in a_unc) + tuple(cb[j] for j in b_unc)
            prod = np.tensordot(A.blocks[ca], B.blocks[cb], axes=(a_con, b_con))
            if cc in acc:
                acc[cc] = acc[cc] + prod
            else:
                acc[cc] = prod
    if not Cinds:
        C.scalar = float(acc.get((), 0.0)) if acc else 0.0
        return C
    C.blocks = {c: np.asfortranarray(v) for c, v in acc.items()}
    return C


def dot(A: BSTensor, B: BSTensor) -> float:
    """eltC(dag(A)*B) for real data: sum over common blocks (A, B same indices)."""
    Bp = B.permuted_to(A.inds)
    s = 0.0
    for c, b in A.blocks.items():
        if c in Bp.blocks:
            s += float(np.vdot(b, Bp.blocks[c]))
    return s
