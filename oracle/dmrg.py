"""Two-site DMRG in numpy: LocalOp::product, davidson, LocalMPO environments,
MPS::svdBond and the DMRGWorker sweep loop.

Restates:
  * LocalOp::product              itensor/mps/localop.h:324-365 (size :488-530)
  * davidson (block size 1)       itensor/iterativesolvers.h:99-451
  * LocalMPO position/makeL/makeR itensor/mps/localmpo.h:443-470, 542-618
  * MPS::svdBond                  itensor/mps/mps_impl.h:21-99
  * DMRGWorker / sweepnext        itensor/mps/dmrg.h:336-467, itensor/mps/sweeps.h:489-503
  * LocalMPOSet (sums of MPOs)   itensor/mps/localmposet.h:140-176
  * LocalMPO of an MPS, LocalMPO_MPS (excited states)
                                  itensor/mps/localmpo.h:340-349, 389-421, 543-594;
                                  itensor/mps/localmpo_mps.h:98-156; itensor/mps/dmrg.h:245-266
"""
from __future__ import annotations

import numpy as np

from .blocksparse import BSTensor, contract, dot
from .decomp import denmat_decomp, svd_split, combine, swap_prime01


class LocalOp:
    def __init__(self, W1, W2, L=None, R=None):
        self.W1, self.W2, self.L, self.R = W1, W2, L, R

    def product(self, phi: BSTensor) -> BSTensor:
        if self.L is None:
            p = phi
            if self.R is not None:
                p = contract(p, self.R)
            p = contract(p, self.W2)
            p = contract(p, self.W1)
        else:
            p = contract(phi, self.L)
            p = contract(p, self.W1)
            p = contract(p, self.W2)
            if self.R is not None:
                p = contract(p, self.R)
        return p.noprime()

    def delta_rho(self, AA: BSTensor, cmb, fromleft: bool) -> BSTensor:
        """LocalOp::deltaRho (itensor/mps/localop.h:375-406): the noise term
        of the density matrix, AA with the environment and MPO tensor of the
        side being orthogonalised, combined and squared, Hermitian part."""
        drho = AA
        if fromleft:
            if self.L is not None:
                drho = contract(drho, self.L)
            drho = contract(drho, self.W1)
        else:
            if self.R is not None:
                drho = contract(drho, self.R)
            drho = contract(drho, self.W2)
        drho = combine(drho.noprime(), cmb)
        drho = contract(drho, drho.dag().prime(which={cmb.ci.id}))
        return (drho + swap_prime01(drho).dag()).scale(0.5)

    def size(self, phi: BSTensor) -> int:
        n = 1
        for I in phi.inds:
            n *= I.dim
        return n


def davidson(A: LocalOp, phi: BSTensor, maxiter=2, errgoal=1e-14, miniter=1, rng=None):
    """Returns (energy, phi). Real arithmetic; the projected matrix is real
    symmetric and is diagonalised as -M ascending (diagHermitian)."""
    approx0 = 1e-12
    nrm = phi.norm()
    phi = phi.scale(1.0 / nrm)
    maxsize = A.size(phi)
    actual_maxiter = min(maxiter, maxsize - 1)
    V = [None] * (actual_maxiter + 2)
    AV = [None] * (actual_maxiter + 2)
    M = np.full((actual_maxiter + 2, actual_maxiter + 2), np.nan)
    V[0] = phi
    AV[0] = A.product(V[0])
    initEn = dot(V[0], AV[0])
    last_lambda = 1000.0
    lam = np.nan
    U = None
    qnorm = np.nan
    phi_t = phi
    for ii in range(actual_maxiter + 1):
        ni = ii + 1
        if ii == 0:
            lam = initEn
            M[0, 0] = lam
            q = AV[0] - V[0].scale(lam)
        else:
            Mref = M[:ii + 1, :ii + 1]
            # diagHermitian(-M) then negated: eigenvalues of M ascending
            D, U = np.linalg.eigh(Mref)
            lam = D[0]
            phi_t = V[0].scale(U[0, 0])
            q = AV[0].scale(U[0, 0])
            for k in range(1, ii + 1):
                phi_t = phi_t + V[k].scale(U[k, 0])
                q = q + AV[k].scale(U[k, 0])
            q = q + phi_t.scale(-lam)
            if U[0, 0] < 0:
                phi_t = phi_t.scale(-1.0)
                q = q.scale(-1.0)
        qnorm = q.norm()
        converged = (qnorm < errgoal and abs(lam - last_lambda) < errgoal) or qnorm < max(approx0, errgoal * 1e-3)
        last_lambda = lam
        if qnorm < 1e-20 or (converged and ii >= miniter) or ii == actual_maxiter:
            break
        # Gram-Schmidt, one pass
        npass = 1
        pass_ = 1
        tot_pass = 0
        done = False
        while pass_ <= npass:
            tot_pass += 1
            Vq = [dot(V[k], q) for k in range(ni)]
            for k in range(ni):
                q = q + V[k].scale(-Vq[k])
            qnrm = q.norm()
            if qnrm < 1e-10:
                if rng is None:
                    rng = np.random.default_rng(0)
                q = V[ni - 1].copy()
                for c in q.blocks:
                    q.blocks[c] = np.asfortranarray(rng.random(q.blocks[c].shape))
                qnrm = q.norm()
                pass_ -= 1
                if ni >= maxsize or tot_pass > npass * 3:
                    done = True
                    break
            q = q.scale(1.0 / qnrm)
            pass_ += 1
        if done:
            break
        V[ni] = q
        AV[ni] = A.product(V[ni])
        for k in range(ni + 1):
            M[k, ni] = dot(V[k], AV[ni])
            M[ni, k] = M[k, ni]
    if actual_maxiter == 0 or U is None:
        return lam, (phi_t if ii > 0 else V[0])
    return lam, phi_t


class LocalMPO:
    """Cached left/right environments; PH[k] for k<b holds sites 1..k, for
    k>b+1 holds sites k..N (1-based)."""

    def __init__(self, W):
        self.W = W
        self.N = len(W)
        self.PH = [None] * (self.N + 2)
        self.LHlim = 0
        self.RHlim = self.N + 1

    def makeL(self, psi, k):
        while self.LHlim < k:
            ll = self.LHlim
            A = psi[ll]  # site ll+1
            E = A if self.PH[ll] is None else contract(self.PH[ll], A)
            E = contract(E, self.W[ll])
            E = contract(E, A.dag().prime())
            self.PH[ll + 1] = E
            self.LHlim = ll + 1

    def makeR(self, psi, k):
        while self.RHlim > k:
            rl = self.RHlim
            A = psi[rl - 2]  # site rl-1
            E = A if self.PH[rl] is None else contract(self.PH[rl], A)
            E = contract(E, self.W[rl - 2])
            E = contract(E, A.dag().prime())
            self.PH[rl - 1] = E
            self.RHlim = rl - 1

    def position(self, b, psi):
        self.makeL(psi, b - 1)
        self.makeR(psi, b + 2)
        self.LHlim = b - 1
        self.RHlim = b + 2
        L = self.PH[b - 1] if b - 1 >= 1 else None
        R = self.PH[b + 2] if b + 2 <= self.N else None
        return LocalOp(self.W[b - 1], self.W[b], L, R)


class LocalMPS:
    """LocalMPO built from a previously found state psi_j: environments of
    <psi_j|psi> (makeL/makeR with dag(prime(psi_j(k), "Link"))) and, at bond b,
    the projection of phi onto psi_j's two-site tensor: phip = dag(othr) (othr * phi)."""

    def __init__(self, psij, site_ids):
        self.P = list(psij)
        self.N = len(psij)
        self.sites = set(site_ids)
        self.PH = [None] * (self.N + 2)
        self.LHlim = 0
        self.RHlim = self.N + 1
        self.b = None

    def _dagp(self, k):
        """dag(prime(psi_j(k), "Link")) for site k (1-based): every index but the site primed."""
        A = self.P[k - 1]
        return A.dag().prime(which={I.id for I in A.inds if I.id not in self.sites})

    def makeL(self, psi, k):
        while self.LHlim < k:
            ll = self.LHlim
            E = psi[ll] if self.PH[ll] is None else contract(self.PH[ll], psi[ll])
            self.PH[ll + 1] = contract(E, self._dagp(ll + 1))
            self.LHlim = ll + 1

    def makeR(self, psi, k):
        while self.RHlim > k:
            rl = self.RHlim
            E = psi[rl - 2] if self.PH[rl] is None else contract(self.PH[rl], psi[rl - 2])
            self.PH[rl - 1] = contract(E, self._dagp(rl - 1))
            self.RHlim = rl - 1

    def position(self, b, psi):
        self.makeL(psi, b - 1)
        self.makeR(psi, b + 2)
        self.LHlim, self.RHlim, self.b = b - 1, b + 2, b

    def othr(self):
        b = self.b
        L = self.PH[b - 1] if b - 1 >= 1 else None
        R = self.PH[b + 2] if b + 2 <= self.N else None
        o = self._dagp(b) if L is None else contract(L, self._dagp(b))
        return contract(o, self._dagp(b + 1) if R is None else contract(R, self._dagp(b + 1)))

    def product(self, phi):
        o = self.othr()
        z = contract(o, phi).scalar
        return o.dag().scale(z)


class OpSum:
    """LocalMPOSet::product (itensor/mps/localmposet.h:140-152): the sum of the
    local products of several MPOs on the same sites; deltaRho summed (:166-176)."""

    def __init__(self, ops):
        self.ops = ops

    def product(self, phi):
        p = self.ops[0].product(phi)
        for op in self.ops[1:]:
            p = p + op.product(phi)
        return p

    def delta_rho(self, AA, cmb, fromleft):
        d = self.ops[0].delta_rho(AA, cmb, fromleft)
        for op in self.ops[1:]:
            d = d + op.delta_rho(AA, cmb, fromleft)
        return d

    def size(self, phi):
        return self.ops[0].size(phi)


class ProjectedOp:
    """LocalMPO_MPS::product: H phi + weight * sum_j P_j phi; deltaRho and size
    from the MPO part (itensor/mps/localmpo_mps.h:65-72, 137-150)."""

    def __init__(self, op, projs, weight):
        self.op, self.projs, self.weight = op, projs, weight

    def product(self, phi):
        p = self.op.product(phi)
        for M in self.projs:
            p = p + M.product(phi).scale(self.weight)
        return p

    def delta_rho(self, AA, cmb, fromleft):
        return self.op.delta_rho(AA, cmb, fromleft)

    def size(self, phi):
        return self.op.size(phi)


def sweep_bonds(N):
    """(b, half-sweep) sequence of sweepnext: b=1..N-1 then N-1..1."""
    out = [(b, 1) for b in range(1, N)]
    out += [(b, 2) for b in range(N - 1, 0, -1)]
    return out


def dmrg(W, psi, sweeps, record=None, usesvd=None, psis=None, weight=1.0, site_ids=None):
    """sweeps: list of dicts {maxdim, mindim, cutoff, niter}. psi: list of
    site tensors (modified copy returned). Returns (energy, psi, records).
    psis: previously found states to stay orthogonal to (H + weight sum_j
    |psi_j><psi_j|, itensor/mps/dmrg.h:245-266); site_ids: ids of the site indices."""
    psi = list(psi)
    N = len(psi)
    # W: one MPO (list of site tensors) or a list of MPOs whose sum is H
    # (dmrg(psi, {H1, H2, ...}, sweeps), itensor/mps/dmrg.h:181-230)
    Wset = W if isinstance(W[0], list) else [W]
    PHs = [LocalMPO(w) for w in Wset]
    projs = [LocalMPS(p, site_ids) for p in (psis or [])]
    energy = np.nan
    recs = []
    for sw, s in enumerate(sweeps, start=1):
        for b, ha in sweep_bonds(N):
            ops = [P.position(b, psi) for P in PHs]
            op = ops[0] if len(ops) == 1 else OpSum(ops)
            if projs:
                for M in projs:
                    M.position(b, psi)
                op = ProjectedOp(op, projs, weight)
            phi = contract(psi[b - 1], psi[b])
            energy, phi = davidson(op, phi, maxiter=s["niter"])
            noise = s.get("noise", 0.0)
            # MPS::svdBond (itensor/mps/mps_impl.h:50): SVD when UseSVD or (noise == 0 and cutoff < 1e-12)
            svd_route = usesvd if usesvd is not None else (noise == 0 and s["cutoff"] < 1e-12)
            if svd_route:
                Uinds = [I for I in psi[b - 1].inds if psi[b].find(I) < 0]
                A, B, probs, te = svd_split(phi, Uinds, s["maxdim"], s["mindim"], s["cutoff"],
                                            fromleft=(ha == 1))
            else:
                A, B, probs, te = denmat_decomp(phi, psi[b - 1], psi[b], ha == 1, s["maxdim"], s["mindim"],
                                                s["cutoff"], noise=noise, op=op)
            psi[b - 1], psi[b] = A, B
            link = [I for I in A.inds if B.find(I) >= 0][0]
            recs.append((sw, ha, b, energy, te, link.dim))
            if record is not None:
                record(sw, ha, b, energy, te, link)
    return energy, psi, recs
