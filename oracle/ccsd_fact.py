"""ORACLE (test infrastructure only) -- factorised FP64 r-ccsd for any molecule size.

The same equations as the literal C restatement (``cc_literal.c``), term for
term, but every inner sum of the reference is written as one tensor
contraction (``numpy.einsum`` picks the pairwise contraction order and hands
the big ones to BLAS). That turns the reference's o^4 v^4 loop nest into
o^3 v^3 / o^2 v^4 work, so N = 160 runs on a workstation.

Term labels follow the comments of the reference:
  singles  src/methods/coupledCluster/ccsd/proj-ccsd-spat-hf-1.f90
           6 :20, 8 :22-31, 7 :33-49, 9 :51-60, 10 :62-73, 11 :75-86, 12 :88-97, 13 :99-116
  doubles  src/methods/coupledCluster/ccsd/proj-ccsd-spat-hf-2.f90
           14 :25, 25 :27-35, 26 :37-45, 17 :47-56, 18 :58-67, 19-22/27/28 :69-103,
           33/36/38 :105-132, 34/35/37 :134-161, 23/24/39 :163-206, 15 :208-216,
           16 :218-226, 29-32 :228-251; mirrored d2(j,i,b,a)=d2(i,j,a,b) :253
The reference evaluates the doubles formula only for pairs (ia) <= (jb) and
mirrors it; ``doubles`` does the same on the full tensor.

Only the integral blocks the equations touch are built, straight from the
zero-differential-overlap form (mod_cc.f90:2258-2277):
``(pq|rs) = sum_{mu,nu} C_mu,p C_mu,q G_mu,nu C_nu,r C_nu,s`` and
``R(p,q,r,s) = 2(pq|rs) - (ps|rq)``.

Step, DIIS, energy and stop rules follow mod_cc.f90:987-1017, 1390-1423,
1514-1555, 1643-1671, 1916-1952, 2133-2193 and gIterator.f90:88-210. DIIS
solves its bordered system by Gaussian elimination (``numpy.linalg.solve``);
the reference's eigen-decomposition gives the same coefficients in exact
arithmetic but stalls near 1e-10 once the Gram matrix loses its smallest
eigenvalues to rounding.
"""
from __future__ import annotations

import numpy as np

from .rhf import IteratorRules


def _e(spec, *ops):
    return np.einsum(spec, *ops, optimize=True)


class Integrals:
    """Lazily built blocks of R restricted to occupied (o) / virtual (v) ranges."""

    def __init__(self, C, G, o):
        self.C = np.asarray(C, dtype=np.float64)
        self.G = np.asarray(G, dtype=np.float64)
        self.o = o
        self._cache = {}

    def _cols(self, s):
        return self.C[:, :self.o] if s == "o" else self.C[:, self.o:]

    def coulomb(self, spec):
        """(pq|rs) with p,q,r,s ranging over the spaces named in spec (e.g. 'vovo')."""
        key = "J" + spec
        if key not in self._cache:
            P, Q, Rr, S = (self._cols(x) for x in spec)
            B1 = _e("mp,mq->mpq", P, Q)
            B2 = _e("nr,ns->nrs", Rr, S)
            Y = _e("mn,nrs->mrs", self.G, B2)
            self._cache[key] = _e("mpq,mrs->pqrs", B1, Y)
        return self._cache[key]

    def R(self, spec):
        """R(p,q,r,s) = 2(pq|rs) - (ps|rq) on the block named by spec."""
        key = "R" + spec
        if key not in self._cache:
            p, q, r, s = spec
            J = self.coulomb(spec)
            K = self.coulomb(p + s + r + q).transpose(0, 3, 2, 1)   # (ps|rq) -> [p,q,r,s]
            self._cache[key] = 2.0 * J - K
        return self._cache[key]


def singles(F, I: Integrals, t1, t2):
    """d1(i,a) of projection_ccsd_singles_spatial_hf."""
    o = t1.shape[0]
    Fov, Fvv, Foo = F[:o, o:], F[o:, o:], F[:o, :o]
    R = I.R
    d1 = Fov.copy()                                                        # 6
    d1 += _e("aijb,jb->ia", R("voov"), t1)                                 # 8
    d1 += _e("ab,ib->ia", Fvv, t1) - _e("ij,ja->ia", Foo, t1)              # 7
    d1 += _e("jb,ijab->ia", Fov, 2 * t2 - t2.transpose(1, 0, 2, 3))        # 9
    Rvvov = R("vvov")
    d1 += _e("abjc,ijbc->ia", Rvvov, t2) + _e("abjc,ib,jc->ia", Rvvov, t1, t1)   # 10
    Rovoo = R("ovoo")
    d1 -= _e("kbji,jkab->ia", Rovoo, t2) + _e("kbji,ja,kb->ia", Rovoo, t1, t1)   # 11
    d1 -= _e("jb,ib,ja->ia", Fov, t1, t1)                                  # 12
    Rovov = R("ovov")                                                      # 13
    d1 += _e("kcjb,kc,ijab->ia", Rovov, t1, 2 * t2 - t2.transpose(1, 0, 2, 3))
    d1 -= _e("kcjb,ib,jkac->ia", Rovov, t1, t2)
    d1 -= _e("kcjb,ka,jibc->ia", Rovov, t1, t2)
    d1 -= _e("kcjb,ka,jb,ic->ia", Rovov, t1, t1, t1)
    return d1


def doubles_unsym(F, I: Integrals, t1, t2):
    """The doubles formula of projection_ccsd_doubles_spatial_hf for every (i,j,a,b)."""
    o = t1.shape[0]
    R = I.R
    Fov, Fvv, Foo = F[:o, o:], F[o:, o:], F[:o, :o]
    tau = t2 + _e("ia,jb->ijab", t1, t1)            # tau(i,j,a,b) = t2 + t1(i,a) t1(j,b)
    t2T = t2.transpose(1, 0, 2, 3)                  # t2(j,i,a,b) at [i,j,a,b]
    x = _e("aibj->ijab", R("vovo")).copy()    # a fresh array: the cached block is a view  # 14
    Rvovv = R("vovv")
    x += _e("bjac,ic->ijab", Rvovv, t1) + _e("aibc,jc->ijab", Rvovv, t1)              # 25
    Roovo = R("oovo")
    x -= _e("kibj,ka->ijab", Roovo, t1) + _e("kjai,kb->ijab", Roovo, t1)              # 26
    x += _e("kilj,klab->ijab", R("oooo"), tau)                                        # 17
    x += _e("bdac,ijcd->ijab", R("vvvv"), tau)                                        # 18
    # 19, 20, 21, 22, 27, 28
    Rvoov, Rovvo, Roovv, Rvvoo = R("voov"), R("ovvo"), R("oovv"), R("vvoo")
    x += 2 * _e("ikac,bjkc->ijab", t2, Rvoov) + 2 * _e("jkbc,aikc->ijab", t2, Rvoov)
    x -= _e("ikca,kcbj->ijab", t2, Rovvo) + _e("jkcb,kcai->ijab", t2, Rovvo)
    x -= _e("jkac,kcbi->ijab", t2, Rovvo) + _e("ikbc,kcaj->ijab", t2, Rovvo)
    x -= _e("kjac,kibc->ijab", t2, Roovv) + _e("kibc,kjac->ijab", t2, Roovv)
    x -= _e("ackj,ic,kb->ijab", Rvvoo, t1, t1) + _e("bcki,jc,ka->ijab", Rvvoo, t1, t1)
    x -= _e("kcbj,ic,ka->ijab", Rovvo, t1, t1) + _e("kcai,jc,kb->ijab", Rovvo, t1, t1)
    # 33, 36, 38
    Rovvv, Rvvov = R("ovvv"), R("vvov")
    x += _e("kcbd,jd,ikac->ijab", Rovvv, t1, 2 * t2 - t2.transpose(1, 0, 2, 3))
    x -= _e("kcbd,jkac,id->ijab", Rovvv, t2, t1) + _e("kcbd,kjad,ic->ijab", Rovvv, t2, t1)
    x += _e("kcad,id,jkbc->ijab", Rovvv, t1, 2 * t2 - t2.transpose(1, 0, 2, 3))
    x -= _e("kcad,ikbc,jd->ijab", Rovvv, t2, t1) + _e("kcad,kibd,jc->ijab", Rovvv, t2, t1)
    x += _e("kd,kdbc,ijac->ijab", t1, Rovvv, 2 * t2 - t2.transpose(0, 1, 3, 2))
    x += _e("kd,kdac,jibc->ijab", t1, Rovvv, 2 * t2 - t2.transpose(0, 1, 3, 2))
    x -= _e("ackd,kb,ijcd->ijab", Rvvov, t1, tau)
    x -= _e("bckd,ka,jicd->ijab", Rvvov, t1, tau)
    # 34, 35, 37
    Rovoo, Rooov = R("ovoo"), R("ooov")
    x += _e("kclj,lb,ikac->ijab", Rovoo, t1, -2 * t2 + t2.transpose(1, 0, 2, 3))
    x += _e("kclj,ikbc,la->ijab", Rovoo, t2, t1) + _e("kclj,ilcb,ka->ijab", Rovoo, t2, t1)
    x += _e("kcli,la,jkbc->ijab", Rovoo, t1, -2 * t2 + t2.transpose(1, 0, 2, 3))
    x += _e("kcli,jkac,lb->ijab", Rovoo, t2, t1) + _e("kcli,jlca,kb->ijab", Rovoo, t2, t1)
    x += _e("lc,kjlc,ikab->ijab", t1, Rooov, -2 * t2 + t2.transpose(1, 0, 2, 3))
    x += _e("lc,kilc,jkba->ijab", t1, Rooov, -2 * t2 + t2.transpose(1, 0, 2, 3))
    x += _e("kclj,ic,klab->ijab", Rovoo, t1, tau)
    x += _e("kcli,jc,klba->ijab", Rovoo, t1, tau)
    # 23, 24, 39: sum_{kcld} R(k,c,l,d) * [...]
    W = R("ovov")
    m2 = (_e("kcld,ljdb,ic,ka->ijab", W, t2, t1, t1) + _e("kcld,lida,jc,kb->ijab", W, t2, t1, t1)
          + _e("kcld,ljab,kc,id->ijab", W, t2, t1, t1) + _e("kcld,liba,kc,jd->ijab", W, t2, t1, t1)
          + _e("kcld,ijac,kb,ld->ijab", W, t2, t1, t1) + _e("kcld,jibc,ka,ld->ijab", W, t2, t1, t1)
          + _e("kcld,kicd,ljab->ijab", W, t2, t2) + _e("kcld,kjcd,liba->ijab", W, t2, t2)
          + _e("kcld,ijac,klbd->ijab", W, t2, t2) + _e("kcld,jibc,klad->ijab", W, t2, t2)
          + _e("kcld,ikca,ljdb->ijab", W, t2, t2) + _e("kcld,jkcb,lida->ijab", W, t2, t2)
          - _e("kcld,ikac,ljdb->ijab", W, t2, t2) - _e("kcld,jkbc,lida->ijab", W, t2, t2))
    x -= 2 * m2
    x += (_e("kcld,jldb,ic,ka->ijab", W, t2, t1, t1) + _e("kcld,ilda,jc,kb->ijab", W, t2, t1, t1)
          + _e("kcld,lidb,jc,ka->ijab", W, t2, t1, t1) + _e("kcld,ljda,ic,kb->ijab", W, t2, t1, t1)
          + _e("kcld,ilcb,jd,ka->ijab", W, t2, t1, t1) + _e("kcld,jlca,id,kb->ijab", W, t2, t1, t1)
          + _e("kcld,liab,kc,jd->ijab", W, t2, t1, t1) + _e("kcld,ljba,kc,id->ijab", W, t2, t1, t1)
          + _e("kcld,ijca,kb,ld->ijab", W, t2, t1, t1) + _e("kcld,jicb,ka,ld->ijab", W, t2, t1, t1)
          + _e("kcld,klab,ic,jd->ijab", W, t2, t1, t1)
          + _e("kcld,ijcd,klab->ijab", W, t2, tau)
          + _e("kcld,ic,ka,jd,lb->ijab", W, t1, t1, t1, t1)
          + _e("kcld,kjcd,liab->ijab", W, t2, t2) + _e("kcld,kicd,ljba->ijab", W, t2, t2)
          + _e("kcld,ijbc,klad->ijab", W, t2, t2) + _e("kcld,jiac,klbd->ijab", W, t2, t2)
          - _e("kcld,lidb,jkac->ijab", W, t2, t2) + _e("kcld,lidb,jkca->ijab", W, t2, t2)
          - _e("kcld,ljda,ikbc->ijab", W, t2, t2) + _e("kcld,ljda,ikcb->ijab", W, t2, t2)
          + 0.5 * (_e("kcld,ikca,jldb->ijab", W, t2, t2) + _e("kcld,jkcb,ilda->ijab", W, t2, t2)
                   + _e("kcld,jkda,ilcb->ijab", W, t2, t2) + _e("kcld,ikdb,jlca->ijab", W, t2, t2)))
    # 15
    x += _e("ca,ijcb->ijab", Fvv, 2 * t2 - t2T) + _e("cb,jica->ijab", Fvv, 2 * t2 - t2T)
    # 16
    x -= _e("ki,kjab->ijab", Foo, 2 * t2 - t2.transpose(0, 1, 3, 2))
    x -= _e("kj,kiba->ijab", Foo, 2 * t2 - t2.transpose(0, 1, 3, 2))
    # 29, 30, 31, 32
    x += -2 * (_e("kc,kjab,ic->ijab", Fov, t2, t1) + _e("kc,kiba,jc->ijab", Fov, t2, t1)
               + _e("kc,ijac,kb->ijab", Fov, t2, t1) + _e("kc,jibc,ka->ijab", Fov, t2, t1))
    x += (_e("kc,kiab,jc->ijab", Fov, t2, t1) + _e("kc,kjba,ic->ijab", Fov, t2, t1)
          + _e("kc,jiac,kb->ijab", Fov, t2, t1) + _e("kc,ijbc,ka->ijab", Fov, t2, t1))
    return x


def pair_matrix(x):
    """[i,j,a,b] -> M[(i,a),(j,b)] with the reference excitation order (i outer, a inner)."""
    o, _, v, _ = x.shape
    return x.transpose(0, 2, 1, 3).reshape(o * v, o * v)


def from_pair_matrix(M, o, v):
    return M.reshape(o, v, o, v).transpose(0, 2, 1, 3)


def doubles(F, I, t1, t2):
    """d2 of the reference: the formula on pairs (ia)<=(jb), mirrored to (jb),(ia)."""
    o, v = t1.shape
    M = pair_matrix(doubles_unsym(F, I, t1, t2))
    M = np.triu(M) + np.triu(M, 1).T
    return from_pair_matrix(M, o, v)


def residuals(F, I, t1, t2):
    return singles(F, I, t1, t2), doubles(F, I, t1, t2)


def guess(F, I, o):
    """guessCC r-ccsd (mod_cc.f90:634-650)."""
    eo, ev = np.diag(F)[:o], np.diag(F)[o:]
    t1 = F[:o, o:] / (eo[:, None] - ev[None, :])
    Rovov = I.R("ovov")                               # R(i,a,j,b)
    den = eo[:, None, None, None] + eo[None, :, None, None] - ev[None, None, :, None] - ev[None, None, None, :]
    t2 = Rovov.transpose(0, 2, 1, 3) / den
    return t1, t2


def energy(F, I, t1, t2, eref):
    """energyCC r-ccsd: [total, Eref, 2 sum F t1, doubles part, 0]."""
    o = t1.shape[0]
    s1 = float((F[:o, o:] * t1).sum())
    tau = t2 + _e("ia,jb->ijab", t1, t1)
    s2 = float(_e("aibj,ijab->", I.R("vovo"), tau))
    return np.array([2 * s1 + s2 + eref, eref, 2 * s1, s2, 0.0])


class DIIS:
    """pushCCVectors/newCCVectors over the packed pair list (ia) <= (jb)."""

    def __init__(self, o, v, nd=20):
        self.o, self.v, self.nd = o, v, nd
        self.iu = np.triu_indices(o * v)
        self.st, self.sd = [], []
        self.B = np.zeros((nd + 1, nd + 1))

    def push(self, t1, t2, d1, sd2):
        self.st.insert(0, np.concatenate([t1.ravel(), pair_matrix(t2)[self.iu]]))
        self.sd.insert(0, np.concatenate([d1.ravel(), pair_matrix(sd2)[self.iu]]))
        del self.st[self.nd:], self.sd[self.nd:]

    def extrapolate(self, iteration):
        n = min(iteration, self.nd)
        B = self.B
        B[1:n, 1:n] = B[0:n - 1, 0:n - 1].copy()
        for k in range(n):
            B[k, 0] = B[0, k] = float(self.sd[k] @ self.sd[0])
        if n == 1:
            return None
        A = np.ones((n + 1, n + 1)); A[:n, :n] = B[:n, :n]; A[n, n] = 0.0
        rhs = np.zeros(n + 1); rhs[n] = 1.0
        with np.errstate(all="ignore"):
            try:
                c = np.linalg.solve(A, rhs)[:n]
            except np.linalg.LinAlgError:
                return None
        if not np.all(np.isfinite(c)):
            return None          # singular subspace: keep the stepped amplitudes
        x = sum(c[k] * self.st[k] for k in range(n))
        o, v = self.o, self.v
        t1 = x[:o * v].reshape(o, v)
        M = np.zeros((o * v, o * v)); M[self.iu] = x[o * v:]
        M = M + np.triu(M, 1).T
        return t1, from_pair_matrix(M, o, v)


def ccsd(F, C, G, eref, o, t1=None, t2=None, eps=1e-12, maxiter=2000, nd=20, diis=True,
         step1=1.0, step2=1.0, projtype=2, callback=None):
    """Full solve; returns dict(energy, status, iterations, t1, t2, trace)."""
    I = Integrals(C, G, o)
    if t1 is None:
        t1, t2 = guess(F, I, o)
    t1, t2 = t1.copy(), t2.copy()
    eo, ev = np.diag(F)[:o], np.diag(F)[o:]
    v = ev.shape[0]
    D1 = eo[:, None] - ev[None, :]
    D2 = eo[:, None, None, None] + eo[None, :, None, None] - ev[None, None, :, None] - ev[None, None, None, :]
    rules = IteratorRules(maxiter, eps)
    hist = DIIS(o, v, nd) if diis else None
    trace = []
    status = None
    while status is None:
        d1, d2 = residuals(F, I, t1, t2)
        sd2 = d2 if projtype == 1 else 2 * d2 + d2.transpose(0, 1, 3, 2)
        t1 = t1 + step1 * d1 / D1
        t2 = t2 + step2 * sd2 / D2
        acc = (float(np.abs(d1).max()), float(np.abs(d2).max()))
        if not max(acc) < eps and hist is not None:
            hist.push(t1, t2, d1, sd2)
            new = hist.extrapolate(rules.iteration + 1)
            if new is not None:
                t1, t2 = new
        e = energy(F, I, t1, t2, eref)
        trace.append((acc[0], acc[1], e[0]))
        if callback is not None:
            callback(rules.iteration + 1, acc, e)
        status = rules.update(max(acc))
    return {"energy": e, "status": status, "iterations": rules.iteration, "t1": t1, "t2": t2,
            "trace": np.array(trace), "ecorr": e[0] - eref}
