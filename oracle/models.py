"""Site sets and MPO construction for the model Hamiltonians of the DMRG
workloads (host-side setup; the reference builds these with its SiteSet /
AutoMPO classes, itensor/mps/sites/spinhalf.h:39-56,
itensor/mps/sites/electron.h:41-60, sample/Heisenberg.h:55-116).

The MPO is an upper-triangular finite-state machine: link state 0 = "done",
1 = "not started", then one channel per (left operator, distance) pair. A term
c * A_i B_j (i<j) leaves "not started" with A at site i, travels through
channel (A, k) carrying identity (or the fermion string F), and ends with
c(j-k, j) * B at site j. Two MPOs of one Hamiltonian give the same
effective Hamiltonian, so DMRG trajectories agree with the reference's.
"""
from __future__ import annotations

import numpy as np

from .blocksparse import BSTensor, Index, QN, OUT, IN


# ---------------------------------------------------------------- sites
class SiteType:
    def __init__(self, name, qns, ops, fermionic=()):
        self.name = name
        self.qns = qns              # QN per basis state
        self.ops = ops              # name -> dense matrix <i|O|j>
        self.fermionic = set(fermionic)

    def state(self, label):
        return self.labels.index(label)


def spin_half(conserve="Sz"):
    if conserve == "Sz":
        qns = [QN(("Sz", 1, 1)), QN(("Sz", -1, 1))]
    elif conserve == "Parity":
        qns = [QN(("Parity", 1, 2)), QN(("Parity", 0, 2))]
    else:
        qns = [QN(), QN()]
    Sz = np.diag([0.5, -0.5])
    Sp = np.array([[0.0, 1.0], [0.0, 0.0]])
    Sm = Sp.T.copy()
    Sx = 0.5 * (Sp + Sm)
    st = SiteType("S=1/2", qns, {"Id": np.eye(2), "Sz": Sz, "S+": Sp, "S-": Sm, "Sx": Sx})
    st.labels = ["Up", "Dn"]
    return st


def electron():
    # basis: Emp, Up, Dn, UpDn with |UpDn> = c+_up c+_dn |0>
    qns = [QN(("Nf", 0, -1), ("Sz", 0, 1)), QN(("Nf", 1, -1), ("Sz", 1, 1)),
           QN(("Nf", 1, -1), ("Sz", -1, 1)), QN(("Nf", 2, -1), ("Sz", 0, 1))]
    adu = np.zeros((4, 4)); adu[1, 0] = 1; adu[3, 2] = 1          # a+_up
    add = np.zeros((4, 4)); add[2, 0] = 1; add[3, 1] = -1         # a+_dn (passes the up mode)
    F = np.diag([1.0, -1.0, -1.0, 1.0])
    nu = adu @ adu.T
    nd = add @ add.T
    ops = {"Id": np.eye(4), "F": F, "Adagup": adu, "Aup": adu.T.copy(), "Adagdn": add, "Adn": add.T.copy(),
           "Nup": nu, "Ndn": nd, "Nupdn": nu @ nd, "Ntot": nu + nd}
    # left-hand operators of a hop carry the string on the right: (a+ F), (F a)
    ops["AdagupF"] = adu @ F
    ops["FAup"] = F @ adu.T
    ops["AdagdnF"] = add @ F
    ops["FAdn"] = F @ add.T
    st = SiteType("Electron", qns, ops, fermionic=("AdagupF", "FAup", "AdagdnF", "FAdn"))
    st.labels = ["Emp", "Up", "Dn", "UpDn"]
    return st


def site_index(st: SiteType, n):
    return Index([(q, 1) for q in st.qns], dir=OUT, tags="Site,n=%d" % n)


def op_flux(st: SiteType, O):
    """QN carried by operator O (q(out) - q(in) of any nonzero element)."""
    nz = np.argwhere(np.abs(O) > 0)
    if len(nz) == 0:
        return QN()
    i, j = nz[0]
    return st.qns[i] - st.qns[j]


# ---------------------------------------------------------------- Hamiltonians
class Hamiltonian:
    """sum of one-site terms (c, op, i) and two-site terms (c, opA, i, opB, j), i<j, 1-based."""

    def __init__(self, st: SiteType, N):
        self.st, self.N = st, N
        self.one = []
        self.two = []

    def add1(self, c, op, i):
        self.one.append((c, op, i))

    def add2(self, c, opA, i, opB, j):
        if i > j:
            raise ValueError("add2 wants i<j")
        self.two.append((c, opA, i, opB, j))


def heisenberg(N, J=1.0, Jz=None, J2=0.0):
    Jz = J if Jz is None else Jz
    H = Hamiltonian(spin_half("Sz"), N)
    for j in range(1, N):
        H.add2(Jz, "Sz", j, "Sz", j + 1)
        H.add2(0.5 * J, "S+", j, "S-", j + 1)
        H.add2(0.5 * J, "S-", j, "S+", j + 1)
    if J2 != 0.0:
        for j in range(1, N - 1):
            H.add2(J2, "Sz", j, "Sz", j + 2)
            H.add2(0.5 * J2, "S+", j, "S-", j + 2)
            H.add2(0.5 * J2, "S-", j, "S+", j + 2)
    return H


def tfi(N, h):
    H = Hamiltonian(spin_half("Parity"), N)
    for j in range(1, N):
        H.add2(-1.0, "Sx", j, "Sx", j + 1)
    for j in range(1, N + 1):
        H.add1(-h, "Sz", j)
    return H


def square_bonds(Nx, Ny, yperiodic):
    """Bond list of ITensor's squareLattice (itensor/mps/lattice/square.h:9-37)."""
    yperiodic = yperiodic and Ny > 2
    bonds = []
    for n in range(1, Nx * Ny + 1):
        x = (n - 1) // Ny + 1
        y = (n - 1) % Ny + 1
        if x < Nx:
            bonds.append((n, n + Ny))
        if Ny > 1:
            if y < Ny:
                bonds.append((n, n + 1))
            if yperiodic and y == 1:
                bonds.append((n, n + Ny - 1))
    return bonds


def hubbard(Nx, Ny, t, U, yperiodic=False):
    N = Nx * Ny
    H = Hamiltonian(electron(), N)
    for (i, j) in square_bonds(Nx, Ny, yperiodic):
        a, b = min(i, j), max(i, j)
        H.add2(-t, "AdagupF", a, "Aup", b)
        H.add2(-t, "FAup", a, "Adagup", b)
        H.add2(-t, "AdagdnF", a, "Adn", b)
        H.add2(-t, "FAdn", a, "Adagdn", b)
    for j in range(1, N + 1):
        H.add1(U, "Nupdn", j)
    return H


# ---------------------------------------------------------------- MPO
def build_mpo(H: Hamiltonian, sites=None):
    """Returns (sites, W list) with W_n inds (dag(s_n), s_n', row=dag(link_{n-1}), col=link_n);
    the first and last tensors have their boundary link projected out."""
    st, N = H.st, H.N
    if sites is None:
        sites = [site_index(st, n) for n in range(1, N + 1)]
    lefts = []
    rng = 1
    for (c, a, i, b, j) in H.two:
        if a not in lefts:
            lefts.append(a)
        rng = max(rng, j - i)
    states = [("done", 0), ("start", 0)] + [(a, k) for a in lefts for k in range(1, rng + 1)]
    sidx = {s: n for n, s in enumerate(states)}
    sq = {("done", 0): QN(), ("start", 0): QN()}
    for a in lefts:
        fa = op_flux(st, st.ops[a])
        for k in range(1, rng + 1):
            sq[(a, k)] = -fa
    # group states into sectors by QN (first appearance order)
    sec_q, sec_of, off_in = [], {}, {}
    counts = []
    for s in states:
        q = sq[s]
        for n, qq in enumerate(sec_q):
            if qq == q:
                break
        else:
            n = len(sec_q)
            sec_q.append(q)
            counts.append(0)
        sec_of[s] = n
        off_in[s] = counts[n]
        counts[n] += 1
    links = [Index([(q, c) for q, c in zip(sec_q, counts)], dir=OUT, tags="Link,l=%d" % l) for l in range(N + 1)]
    d = len(st.qns)
    Ws = []
    for n in range(1, N + 1):
        D = len(states)
        W = np.zeros((d, d, D, D))  # (s_in, s_out, row, col) dense
        def put(r, c, O, coef=1.0):
            W[:, :, sidx[r], sidx[c]] += coef * st.ops[O].T

        put(("done", 0), ("done", 0), "Id")
        put(("start", 0), ("start", 0), "Id")
        for (c, op, i) in H.one:
            if i == n:
                put(("start", 0), ("done", 0), op, c)
        for a in lefts:
            ferm = a in st.fermionic
            # start a channel here
            if any(tt[1] == a and tt[2] == n for tt in H.two):
                put(("start", 0), (a, 1), a, _left_coef(H, a, n))
            for k in range(1, rng):
                if any(tt[1] == a and tt[2] == n - k and tt[4] > n for tt in H.two):
                    put((a, k), (a, k + 1), "F" if ferm else "Id")
        for (c, a, i, b, j) in H.two:
            if j == n:
                put((a, j - i), ("done", 0), b, c / _left_coef(H, a, i))
        T = BSTensor([sites[n - 1].dag(), sites[n - 1].prime(), links[n - 1].dag(), links[n]])
        for cs in BSTensor.allowed_blocks(T.inds, QN()):
            blk = np.zeros(T.block_shape(cs), order="F")
            any_nz = False
            rs = [s for s in states if sec_of[s] == cs[2]]
            cols = [s for s in states if sec_of[s] == cs[3]]
            for r in rs:
                for cc in cols:
                    v = W[cs[0], cs[1], sidx[r], sidx[cc]]
                    if v != 0.0:
                        blk[0, 0, off_in[r], off_in[cc]] = v
                        any_nz = True
            if any_nz:
                T.blocks[cs] = blk
        Ws.append(T)
    # boundary projections: row of W_1 = start, col of W_N = done
    Ws[0] = _project(Ws[0], 2, sec_of[("start", 0)], off_in[("start", 0)])
    Ws[-1] = _project(Ws[-1], 3, sec_of[("done", 0)], off_in[("done", 0)])
    return sites, Ws, links


def _left_coef(H: Hamiltonian, a, i):
    """Coefficient carried by the starting operator a at site i: the common
    coefficient of every two-site term that starts there, else 1 (the ending
    operators carry the rest).  For the nearest-neighbour Heisenberg chain
    this is the gauge of sample/Heisenberg.h:79-90 (J/2 and Jz on the left
    operator, 1 on the right), which the noise term (a sum over MPO link
    channels, itensor/mps/localop.h:375-406) depends on."""
    cs = [tt[0] for tt in H.two if tt[1] == a and tt[2] == i]
    if cs and all(c == cs[0] for c in cs) and cs[0] != 0.0:
        return cs[0]
    return 1.0


def _project(T: BSTensor, axis, sec, off):
    inds = [I for k, I in enumerate(T.inds) if k != axis]
    out = BSTensor(inds)
    for c, b in T.blocks.items():
        if c[axis] != sec:
            continue
        nc = tuple(x for k, x in enumerate(c) if k != axis)
        out.blocks[nc] = np.asfortranarray(np.take(b, off, axis=axis))
    return out


def product_mps(sites, st: SiteType, labels):
    """MPS of a product state with the link QNs of MPS(InitState)
    (itensor/mps/mps.cc:558-585): link i carries the QN of sites i+1..N."""
    N = len(sites)
    qs = [st.qns[st.labels.index(l)] for l in labels]
    qa = [QN() for _ in range(N + 1)]
    tot = QN()
    for q in qs:
        tot = tot + q
    qa[0] = tot
    for i in range(1, N + 1):
        qa[i] = qa[i - 1] - qs[i - 1]
    links = [None] + [Index([(qa[i], 1)], dir=OUT, tags="Link,l=%d" % i) for i in range(1, N)]
    A = []
    for i in range(1, N + 1):
        s = st.labels.index(labels[i - 1])
        if i == 1:
            T = BSTensor([sites[0], links[1]])
            T.blocks[(s, 0)] = np.ones((1, 1), order="F")
        elif i == N:
            T = BSTensor([links[N - 1].dag(), sites[N - 1]])
            T.blocks[(0, s)] = np.ones((1, 1), order="F")
        else:
            T = BSTensor([links[i - 1].dag(), sites[i - 1], links[i]])
            T.blocks[(0, s, 0)] = np.ones((1, 1, 1), order="F")
        A.append(T)
    return A
