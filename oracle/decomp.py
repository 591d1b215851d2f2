"""Bond split: QN combiner, truncation, blockwise eigh / SVD, denmatDecomp.

Restates, in numpy:
  * combiner / combine / uncombine      itensor/itensor.cc:1469-1560,
                                         itensor/itdata/qcombiner.cc:125-300
  * truncate                             itensor/decomp.cc:305-463
  * diag_hermitian, QN branch            itensor/hermitian.cc:180-426
  * denmatDecomp                         itensor/decomp.h:316-418
  * svd (QN) via svdOrd2/svdImpl         itensor/decomp.cc:121-248, itensor/svd.cc:169-401
"""
from __future__ import annotations

import itertools
import numpy as np

from .blocksparse import BSTensor, Index, QN, OUT, IN, contract, rkey

REAL_EPSILON = np.finfo(np.float64).eps


class Combiner:
    """Fuses ``inds`` into one QN index ``ci``. ``ranges`` maps a tuple of
    sector numbers (one per fused index) to (sector n of ci, start, extent)."""

    def __init__(self, inds, cdir=None, tags="Link,CMB"):
        inds = list(inds)
        if cdir is None:
            cdir = IN if all(I.dir == IN for I in inds) else OUT
        qms = []  # [qn, m]
        ranges = {}
        # C.range(): first fused index fastest
        for c in itertools.product(*reversed([range(I.nblock) for I in inds])):
            c = tuple(reversed(c))
            q = QN()
            m = 1
            for I, b in zip(inds, c):
                q = q + I.qn(b).scaled(I.dir * cdir)
                m *= I.bdim(b)
            for n, (qq, mm) in enumerate(qms):
                if qq == q:
                    ranges[c] = (n, mm, m)
                    qms[n][1] += m
                    break
            else:
                ranges[c] = (len(qms), 0, m)
                qms.append([q, m])
        self.inds = inds
        self.ranges = ranges
        self.ci = Index([(q, m) for q, m in qms], dir=cdir, tags=tags)


def combine(T: BSTensor, C: Combiner) -> BSTensor:
    """cmb*T: fused index first, then T's other indices in order."""
    pos = [T.find(I) for I in C.inds]
    assert all(p >= 0 for p in pos)
    rest = [k for k in range(T.order) if k not in pos]
    out = BSTensor([C.ci] + [T.inds[k] for k in rest])
    for c, b in T.blocks.items():
        sub = tuple(c[p] for p in pos)
        n, start, ext = C.ranges[sub]
        nc = (n,) + tuple(c[k] for k in rest)
        if nc not in out.blocks:
            out.blocks[nc] = np.zeros(out.block_shape(nc), order="F")
        pb = np.transpose(b, pos + rest)
        shp = pb.shape
        pb = np.reshape(pb, (ext,) + shp[len(pos):], order="F")
        out.blocks[nc][start:start + ext] = pb
    return out


def uncombine(T: BSTensor, C: Combiner) -> BSTensor:
    """Replaces the fused index (wherever it sits in T) by the original ones."""
    jc = T.find(C.ci)
    assert jc >= 0
    newinds = T.inds[:jc] + C.inds + T.inds[jc + 1:]
    out = BSTensor(newinds)
    for c, b in T.blocks.items():
        n = c[jc]
        for sub, (nn, start, ext) in C.ranges.items():
            if nn != n:
                continue
            nc = c[:jc] + sub + c[jc + 1:]
            sl = np.take(b, range(start, start + ext), axis=jc)
            shp = sl.shape
            subdims = tuple(I.bdim(s) for I, s in zip(C.inds, sub))
            out.blocks[nc] = np.asfortranarray(np.reshape(sl, shp[:jc] + subdims + shp[jc + 1:], order="F"))
    return out


def truncate(P, maxdim, mindim, cutoff, absoluteCutoff=False, doRelCutoff=True, respectDegenerate=False):
    """Returns (P_kept, truncerr, docut_lower, docut_upper, ndegen_below).
    P is sorted descending (itensor/decomp.cc:305-463)."""
    P = np.array(P, dtype=np.float64)
    origm = len(P)
    n = origm - 1
    if P[0] == 0.0:
        return P[:1].copy(), 0.0, -REAL_EPSILON, REAL_EPSILON, 1
    if origm == 1:
        dc = 1e-3 * P[0]
        return P.copy(), 0.0, P[0] - dc, P[0] + dc, 1
    P0 = P[0]
    P = P / P0
    if absoluteCutoff or not doRelCutoff:
        cutoff = cutoff / P0
    for zn in range(n, -1, -1):
        if P[zn] >= 0:
            break
        P[zn] = 0
    truncerr = 0.0
    while n >= maxdim:
        truncerr += P[n]
        n -= 1
    if absoluteCutoff:
        while P[n] <= cutoff and n >= mindim:
            truncerr += P[n]
            n -= 1
    else:
        scale = 1.0
        if doRelCutoff:
            scale = 0.0
            for x in P:
                scale += float(x)
            if scale == 0.0:
                scale = 1.0
        while truncerr + P[n] <= cutoff * scale and n >= mindim:
            truncerr += P[n]
            n -= 1
        truncerr = 0 if scale == 0 else truncerr / scale
    if n < 0:
        n = 0
    m = n + 1
    degen_cutoff = 1e-3 * P[n]
    if P[n] == 0.0:
        degen_cutoff = REAL_EPSILON
    docut_lower = P[n] - degen_cutoff
    docut_upper = P[n] + degen_cutoff
    ndegen_below = 1
    if n > 0:
        while n - ndegen_below >= 0 and abs(P[n - ndegen_below] - P[n]) < degen_cutoff:
            ndegen_below += 1
    ndegen_above = 0
    if n + 1 < origm:
        while n + 1 + ndegen_above < origm and abs(P[n + 1 + ndegen_above] - P[n]) < degen_cutoff:
            ndegen_above += 1
    if respectDegenerate and (ndegen_below + ndegen_above > 1):
        if maxdim < m + ndegen_above:
            m -= ndegen_below
            ndegen_above += ndegen_below
            ndegen_below = 0
        else:
            m += ndegen_above
            ndegen_below += ndegen_above
            ndegen_above = 0
    P = P[:m] * P0
    return P, truncerr * P0, docut_lower * P0, docut_upper * P0, ndegen_below


def _block_eigh_desc(M):
    """diagHermitian: eigen-decompose -M ascending = M descending
    (itensor/tensor/algs_impl.h:91-139)."""
    w, V = np.linalg.eigh(-0.5 * (M + M.T))
    return -w, V


def diag_hermitian(rho: BSTensor, ai: Index, maxdim=None, mindim=1, cutoff=0.0, truncate_=True,
                   doRelCutoff=True, absoluteCutoff=False, respectDegenerate=False, tags="Link"):
    """QN diag_hermitian of an order-2, divergence-zero tensor rho(ai, ai').
    Returns (U, d_index, eigs_kept, truncerr, per-block kept counts)."""
    i0 = rho.find(ai)
    assert i0 >= 0
    if maxdim is None:
        maxdim = ai.dim
    blocks = []  # (sector, M) in storage order
    for c in rho.sorted_coords():
        b = rho.blocks[c]
        M = b if i0 == 0 else b.T
        blocks.append((c[i0], M))
    evs = []
    alleig = []
    for sec, M in blocks:
        d, V = _block_eigh_desc(M)
        evs.append((sec, d, V))
        alleig.extend(d.tolist())
    probs = np.array(sorted(alleig, reverse=True))
    truncerr, lo, up, ndegen = 0.0, -1.0, -1.0, 0
    m = len(probs)
    if truncate_:
        probs, truncerr, lo, up, ndegen = truncate(probs, maxdim, mindim, cutoff, absoluteCutoff,
                                                   doRelCutoff, respectDegenerate)
        m = len(probs)
    kept = []
    total_m = 0
    for sec, d, V in evs:
        this_m = 0
        if truncate_:
            while this_m < len(d) and total_m < m and d[this_m] > up:
                this_m += 1
                total_m += 1
            while ndegen > 0 and this_m < len(d) and total_m < m and d[this_m] > lo:
                this_m += 1
                total_m += 1
                ndegen -= 1
        else:
            this_m = len(d)
            total_m += this_m
        kept.append(this_m)
    secs = [(ai.qn(sec), k) for (sec, d, V), k in zip(evs, kept) if k > 0]
    if not secs:
        secs = [(ai.qn(evs[0][0]), 1)]
    dind = Index(secs, dir=-ai.dir, tags=tags)
    U = BSTensor([ai.dag(), dind.dag()])
    n = 0
    for (sec, d, V), k in zip(evs, kept):
        if k == 0:
            continue
        U.blocks[(sec, n)] = np.asfortranarray(V[:, :k])
        n += 1
    return U, dind, probs, truncerr, kept


def swap_prime01(T: BSTensor) -> BSTensor:
    """swapTags(T, "0", "1"): prime levels 0 and 1 exchanged, data unchanged."""
    inds = [I.prime(1) if I.plev == 0 else (I.prime(-1) if I.plev == 1 else I) for I in T.inds]
    return BSTensor(inds, T.blocks, T.scalar)


def block_trace(rho: BSTensor) -> float:
    """delta(dag(ci), prime(ci)) * rho for a 2-index QN tensor (ci, ci')."""
    return float(sum(np.trace(b) for c, b in rho.blocks.items() if c[0] == c[1]))


def denmat_decomp(AA: BSTensor, A: BSTensor, B: BSTensor, fromleft: bool, maxdim, mindim, cutoff,
                  respectDegenerate=True, normalize=True, noise=0.0, op=None):
    """denmatDecomp (itensor/decomp.h:316-418), with the noise term
    rho += noise * deltaRho and the trace normalisation (decomp.h:386-394)
    when noise > 0, followed by the DoNormalize step of MPS::svdBond
    (itensor/mps/mps_impl.h:73-78). Returns (A', B', probs, truncerr)."""
    to_orth, newoc = (A, B) if fromleft else (B, A)
    cinds = [I for I in to_orth.inds if newoc.find(I) < 0]
    cmb = Combiner(cinds)
    AAc = combine(AA, cmb)
    rho = contract(AAc, AAc.dag().prime(which={cmb.ci.id}))
    if noise > 0 and op is not None:
        rho = rho + op.delta_rho(AA, cmb, fromleft).scale(noise)
        tr = block_trace(rho)
        if tr > 1e-16:
            rho = rho.scale(1.0 / tr)
    U, dind, probs, te, kept = diag_hermitian(rho, cmb.ci, maxdim=maxdim, mindim=mindim, cutoff=cutoff,
                                              respectDegenerate=respectDegenerate)
    Ud = U.dag()
    new_orth = uncombine(Ud, cmb)
    new_oc = contract(U, AAc)
    if normalize:
        nrm = new_oc.norm()
        if nrm > 1e-16:
            new_oc = new_oc.scale(1.0 / nrm)
    if fromleft:
        return new_orth, new_oc, probs, te
    return new_oc, new_orth, probs, te


def svd_split(AA: BSTensor, Uinds, maxdim, mindim, cutoff, respectDegenerate=True, fromleft=True,
              normalize=True):
    """svd route of MPS::svdBond (itensor/mps/mps_impl.h:50-65): returns
    (A', B', probs, truncerr) with the singular values pushed into the new
    orthogonality centre."""
    # U's indices in the order they appear on AA (itensor/decomp.cc:185-192)
    Uinds = [I for I in AA.inds if any(I.same(J) for J in Uinds)]
    Vinds = [I for I in AA.inds if not any(I.same(J) for J in Uinds)]
    cu = Combiner(Uinds)
    cv = Combiner(Vinds)
    AAc = combine(combine(AA, cu), cv)  # inds (vi, ui)
    ui, vi = cu.ci, cv.ci
    blocks = []
    for c in AAc.sorted_coords():
        b = AAc.blocks[c]
        blocks.append((c[1], c[0], b.T))  # rows ui, cols vi
    res = []
    alleig = []
    for bu, bv, M in blocks:
        Uu, s, Vt = np.linalg.svd(M, full_matrices=False)
        res.append((bu, bv, Uu, s, Vt.T))
        alleig.extend((s * s).tolist())
    probs = np.array(sorted(alleig, reverse=True))
    probs, te, lo, up, ndegen = truncate(probs, maxdim, mindim, cutoff, False, True, respectDegenerate)
    m = len(probs)
    kept = []
    total_m = 0
    for bu, bv, Uu, s, V in res:
        this_m = 0
        while this_m < len(s) and total_m < m and s[this_m] ** 2 > up:
            this_m += 1
            total_m += 1
        while ndegen > 0 and this_m < len(s) and total_m < m and s[this_m] ** 2 > lo:
            this_m += 1
            total_m += 1
            ndegen -= 1
        kept.append(this_m)
    Lidx = Index([(ui.qn(bu), k) for (bu, bv, _, _, _), k in zip(res, kept) if k > 0], dir=ui.dir, tags="Link,U")
    Ridx = Index([(vi.qn(bv), k) for (bu, bv, _, _, _), k in zip(res, kept) if k > 0], dir=vi.dir, tags="Link,V")
    U = BSTensor([ui, Lidx.dag()])
    V = BSTensor([vi, Ridx.dag()])
    D = BSTensor([Lidx, Ridx])
    n = 0
    for (bu, bv, Uu, s, Vv), k in zip(res, kept):
        if k == 0:
            continue
        U.blocks[(bu, n)] = np.asfortranarray(Uu[:, :k])
        V.blocks[(bv, n)] = np.asfortranarray(Vv[:, :k])
        D.blocks[(n, n)] = np.asfortranarray(np.diag(s[:k]))
        n += 1
    U = uncombine(U, cu)
    V = uncombine(V, cv)
    if normalize:
        D = D.scale(1.0 / D.norm())
    if fromleft:
        return U, contract(V, D), probs, te
    return contract(U, D), V, probs, te
