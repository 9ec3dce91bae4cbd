"""ORACLE (test infrastructure only) -- textbook spin-orbital CCSD, an independent pin.

Not a restatement of helios: the published spin-orbital CCSD equations with
the effective-Hamiltonian intermediates of J. F. Stanton, J. Gauss, J. D. Watts
and R. J. Bartlett, J. Chem. Phys. 94, 4334 (1991), solved by Jacobi steps
with DIIS. Given the same RHF orbitals and PPP integrals its converged
correlation energy must equal the reference's spin-adapted "2-1" r-ccsd
(the closed-shell equations are an exact spin adaptation of these).

Spin orbital 2P+s is spatial orbital P with spin s; occupied spin orbitals
come first after reordering. Antisymmetrised integrals
<pq||rs> = <pq|rs> - <pq|sr>, <pq|rs> = (PR|QS) delta_sp,sr delta_sq,ss.
Feasible for N <= 14 sites (arrays of (2N)^4).
"""
from __future__ import annotations

import numpy as np


def _e(s, *a):
    return np.einsum(s, *a, optimize=True)


def spin_integrals(C, G, h_core, nocc):
    """Fock matrix and <pq||rs> in the spin-orbital MO basis (occupied first)."""
    N = C.shape[0]
    B = _e("mp,mq->mpq", C, C)                        # ZDO pair densities
    eri = _e("mpq,mn,nrs->pqrs", B, G, B)             # (pq|rs)
    hmo = C.T @ h_core @ C
    ns = 2 * N
    # order: occupied alpha/beta pairs first, then virtual
    order = [2 * p + s for p in range(nocc) for s in (0, 1)] + [2 * p + s for p in range(nocc, N) for s in (0, 1)]
    spat = np.array([k // 2 for k in order])
    spin = np.array([k % 2 for k in order])
    phys = eri[np.ix_(spat, spat, spat, spat)].transpose(0, 2, 1, 3)  # <pq|rs> = (pr|qs)
    same = (spin[:, None] == spin[None, :]).astype(float)
    phys = phys * same[:, None, :, None] * same[None, :, None, :]
    anti = phys - phys.transpose(0, 1, 3, 2)
    h = hmo[np.ix_(spat, spat)] * same
    no = 2 * nocc
    f = h + _e("piqi->pq", anti[:, :no, :, :no])
    return f, anti, no, ns


def ccsd(C, G, h_core, nocc, eps=1e-11, maxiter=300, ndiis=8):
    f, g, no, ns = spin_integrals(C, G, h_core, nocc)
    o, v = slice(0, no), slice(no, ns)
    fo, fv = np.diag(f)[o], np.diag(f)[v]
    Dia = fo[:, None] - fv[None, :]
    Dijab = fo[:, None, None, None] + fo[None, :, None, None] - fv[None, None, :, None] - fv[None, None, None, :]
    foo, fvv, fov = f[o, o], f[v, v], f[o, v]
    t1 = fov / Dia
    t2 = g[o, o, v, v] / Dijab
    hist_t, hist_e = [], []
    for it in range(1, maxiter + 1):
        tau_t = t2 + 0.5 * (_e("ia,jb->ijab", t1, t1) - _e("ib,ja->ijab", t1, t1))
        tau = t2 + _e("ia,jb->ijab", t1, t1) - _e("ib,ja->ijab", t1, t1)
        Fae = fvv - np.diag(np.diag(fvv)) - 0.5 * _e("me,ma->ae", fov, t1) \
            + _e("mf,mafe->ae", t1, g[o, v, v, v]) - 0.5 * _e("mnaf,mnef->ae", tau_t, g[o, o, v, v])
        Fmi = foo - np.diag(np.diag(foo)) + 0.5 * _e("ie,me->mi", t1, fov) \
            + _e("ne,mnie->mi", t1, g[o, o, o, v]) + 0.5 * _e("inef,mnef->mi", tau_t, g[o, o, v, v])
        Fme = fov + _e("nf,mnef->me", t1, g[o, o, v, v])
        Wmnij = g[o, o, o, o] + _e("je,mnie->mnij", t1, g[o, o, o, v]) - _e("ie,mnje->mnij", t1, g[o, o, o, v]) \
            + 0.25 * _e("ijef,mnef->mnij", tau, g[o, o, v, v])
        Wabef = g[v, v, v, v] - _e("mb,amef->abef", t1, g[v, o, v, v]) + _e("ma,bmef->abef", t1, g[v, o, v, v]) \
            + 0.25 * _e("mnab,mnef->abef", tau, g[o, o, v, v])
        Wmbej = g[o, v, v, o] + _e("jf,mbef->mbej", t1, g[o, v, v, v]) - _e("nb,mnej->mbej", t1, g[o, o, v, o]) \
            - _e("jnfb,mnef->mbej", 0.5 * t2 + _e("jf,nb->jnfb", t1, t1), g[o, o, v, v])
        r1 = fov + _e("ie,ae->ia", t1, Fae) - _e("ma,mi->ia", t1, Fmi) + _e("imae,me->ia", t2, Fme) \
            - _e("nf,naif->ia", t1, g[o, v, o, v]) - 0.5 * _e("imef,maef->ia", t2, g[o, v, v, v]) \
            - 0.5 * _e("mnae,nmei->ia", t2, g[o, o, v, o])
        Pab = lambda x: x - x.transpose(0, 1, 3, 2)
        Pij = lambda x: x - x.transpose(1, 0, 2, 3)
        r2 = g[o, o, v, v].copy()
        r2 += Pab(_e("ijae,be->ijab", t2, Fae - 0.5 * _e("mb,me->be", t1, Fme)))
        r2 -= Pij(_e("imab,mj->ijab", t2, Fmi + 0.5 * _e("je,me->mj", t1, Fme)))
        r2 += 0.5 * _e("mnab,mnij->ijab", tau, Wmnij) + 0.5 * _e("ijef,abef->ijab", tau, Wabef)
        x = _e("imae,mbej->ijab", t2, Wmbej) - _e("ie,ma,mbej->ijab", t1, t1, g[o, v, v, o])
        r2 += Pij(Pab(x))
        r2 += Pij(_e("ie,abej->ijab", t1, g[v, v, v, o])) - Pab(_e("ma,mbij->ijab", t1, g[o, v, o, o]))
        # r1, r2 are D*t_new; residuals relative to the current amplitudes
        n1, n2 = r1 / Dia, r2 / Dijab
        err = max(np.abs(n1 - t1).max(), np.abs(n2 - t2).max())
        new = np.concatenate([n1.ravel(), n2.ravel()])
        old = np.concatenate([t1.ravel(), t2.ravel()])
        t1, t2 = n1, n2
        if err < eps:
            break
        hist_t.append(new)
        hist_e.append(new - old)
        if len(hist_t) > ndiis:
            hist_t.pop(0); hist_e.pop(0)
        if len(hist_t) >= 2:
            n = len(hist_t)
            E = np.array(hist_e)
            B = np.ones((n + 1, n + 1)); B[:n, :n] = E @ E.T; B[n, n] = 0
            rhs = np.zeros(n + 1); rhs[n] = 1
            try:
                c = np.linalg.solve(B, rhs)[:n]
            except np.linalg.LinAlgError:
                continue
            vec = c @ np.array(hist_t)
            t1 = vec[:t1.size].reshape(t1.shape); t2 = vec[t1.size:].reshape(t2.shape)
    e = _e("ia,ia->", fov, t1) + 0.25 * _e("ijab,ijab->", g[o, o, v, v], t2) \
        + 0.5 * _e("ijab,ia,jb->", g[o, o, v, v], t1, t1)
    return float(e), it
