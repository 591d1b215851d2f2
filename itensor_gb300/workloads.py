"""Seeded synthetic inputs for the isolated effective-Hamiltonian apply.

Layout (the isolated-apply workload): U(1) Sz link of total dimension m over
2K+1 sectors with q = 2(k-K) and Gaussian sizes floor(m g_k / sum g),
g_k = exp(-(k-K)^2 / (2 sigma^2)), remainder to the centre sector; local
dimension 2 (S=1/2, Sz = +-1); MPO = Heisenberg bulk tensor (bond dim 5 with
sectors Sz 0 x3, -2, +2, as sample/Heisenberg.h:55-116). psi(l,s1,s2,r),
L(l,w,l') and R(r,w',r') hold every block of divergence 0 with N(0,1)
entries from a seeded generator.

Tensors are returned as plain numpy descriptions so that both the device path
and the CPU oracle can be fed the same bytes:
    index  = dict(id, plev, dir, qn=[Sz per sector], dims=[...])
    tensor = dict(inds=[index...], coords=int32 (nblocks x rank), data=float64)
"""
from __future__ import annotations

import itertools
import numpy as np


def gauss_sectors(m, K, sigma):
    g = np.exp(-((np.arange(2 * K + 1) - K) ** 2) / (2.0 * sigma * sigma))
    sizes = np.floor(m * g / g.sum()).astype(int)
    sizes[K] += m - int(sizes.sum())
    qs = [2 * (k - K) for k in range(2 * K + 1)]
    keep = [k for k in range(2 * K + 1) if sizes[k] > 0]
    return [qs[k] for k in keep], [int(sizes[k]) for k in keep]


def _index(id_, qn, dims, dir_=1, plev=0):
    return dict(id=id_, plev=plev, dir=dir_, qn=list(qn), dims=list(dims))


def dag(I):
    J = dict(I)
    J["dir"] = -I["dir"]
    return J


def prime(I):
    J = dict(I)
    J["plev"] = I["plev"] + 1
    return J


def allowed_blocks(inds, div=0):
    ranges = [range(len(I["dims"])) for I in inds]
    out = []
    for c in itertools.product(*reversed(ranges)):
        c = tuple(reversed(c))
        if sum(I["dir"] * I["qn"][b] for I, b in zip(inds, c)) == div:
            out.append(c)
    return out


def block_size(inds, c):
    n = 1
    for I, b in zip(inds, c):
        n *= I["dims"][b]
    return n


def random_tensor(inds, rng, div=0):
    cs = allowed_blocks(inds, div)
    size = sum(block_size(inds, c) for c in cs)
    return dict(inds=inds, coords=np.asarray(cs, np.int32).reshape(len(cs), len(inds)), data=rng.standard_normal(size))


def heisenberg_w(s_in, wl, wr, J=1.0, Jz=1.0):
    """Bulk MPO tensor W(dag(s), s', dag(wl), wr) of the S=1/2 Heisenberg chain.
    Link states: 0 done, 1 start, 2 Sz channel (sector Sz 0), 3 after S+ (Sz -2), 4 after S- (Sz +2)."""
    Sz = np.diag([0.5, -0.5])
    Sp = np.array([[0.0, 1.0], [0.0, 0.0]])
    Sm = Sp.T
    Id = np.eye(2)
    D = 5
    W = np.zeros((2, 2, D, D))  # (s_in, s_out, row, col)

    def put(r, c, O, a=1.0):
        W[:, :, r, c] += a * O.T

    put(0, 0, Id); put(1, 1, Id)
    put(2, 0, Sz); put(1, 2, Sz, Jz)
    put(3, 0, Sm); put(1, 3, Sp, J / 2)
    put(4, 0, Sp); put(1, 4, Sm, J / 2)
    # link sectors: [Sz 0: states 0,1,2], [Sz -2: state 3], [Sz +2: state 4]
    sec_states = [[0, 1, 2], [3], [4]]
    inds = [dag(s_in), prime(s_in), dag(wl), wr]
    coords, data = [], []
    for c in allowed_blocks(inds):
        rs, cs = sec_states[c[2]], sec_states[c[3]]
        blk = np.zeros((1, 1, len(rs), len(cs)))
        for i, r in enumerate(rs):
            for j, cc in enumerate(cs):
                blk[0, 0, i, j] = W[c[0], c[1], r, cc]
        if np.any(blk != 0):
            coords.append(c)
            data.append(blk.reshape(-1, order="F"))
    return dict(inds=inds, coords=np.asarray(coords, np.int32).reshape(len(coords), 4), data=np.concatenate(data))


def heff_workload(m=1024, K=15, sigma=6.0, seed=0):
    """psi, L, W1, W2, R of the isolated H_eff apply (ids 1..7 for l, s1, s2, r, wl, wm, wr)."""
    rng = np.random.default_rng(seed)
    qn, dims = gauss_sectors(m, K, sigma)
    l = _index(1, qn, dims)
    r = _index(4, qn, dims)
    s1 = _index(2, [1, -1], [1, 1])
    s2 = _index(3, [1, -1], [1, 1])
    wqn, wdims = [0, -2, 2], [3, 1, 1]
    wl, wm, wr = _index(5, wqn, wdims), _index(6, wqn, wdims), _index(7, wqn, wdims)
    psi = random_tensor([dag(l), s1, s2, r], rng)
    L = random_tensor([l, wl, dag(prime(l))], rng)
    R = random_tensor([dag(r), dag(wr), prime(r)], rng)
    W1 = heisenberg_w(s1, wl, wm)
    W2 = heisenberg_w(s2, wm, wr)
    return dict(psi=psi, L=L, W1=W1, W2=W2, R=R, m=m, nsect=len(dims))


def to_device(ctx, t):
    """A workload tensor as an itensor_gb300.Tensor (Sz in QN slot 0)."""
    import itensor_gb300 as itg
    inds = [itg.Index(I["id"], I["plev"], I["dir"], [[q, 0, 0, 0] for q in I["qn"]], I["dims"], [1, 0, 0, 0])
            for I in t["inds"]]
    return ctx.tensor(inds, t["coords"].reshape(-1), t["data"])
