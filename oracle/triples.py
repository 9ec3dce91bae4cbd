"""ORACLE (test infrastructure only) -- the (T) triples correction of r-ccsd(t).

``spin_triples`` restates the reference's spin-orbital energy for
'spin-r-ccsd(t)' (src/methods/coupledCluster/mod_cc.f90:2028-2111): for every
spin-conserving (i, j, k, a, b, c) the connected triples amplitude
  amp = (sum1 - sum2) / D,  D = F_aa + F_bb + F_cc - F_ii - F_jj - F_kk,
with sum1 the nine hole terms R(j,c,k,l) t2(i,l,a,b) - ... and sum2 the nine
particle terms R(b,k,c,d) t2(i,j,a,d) - ... (:2061-2085), and
  c1 = sum amp^2 D / 36,  c2 = sum amp t1(i,a) R(b,j,c,k) / 4,
  c3 = sum amp t2(i,j,a,b) F(k,c),  E(T) = c1 + c2 + c3.
R(p,q,r,s) = [pq||rs] = [pq|rs] - [ps|qr] (spin_hf_int, :2281-2307), i.e. the
physicist's <pr||qs>. Vectorised over all index tuples (the spin-forbidden
ones have zero integrals); feasible for N <= 14 sites.

``closed_shell_triples`` is the spin-adapted form the GPU evaluates, on
spatial orbitals (closed-shell amplitudes t_ij^ab = t2[i, j, a, b], the
reference's layout t2(o, o, v, v)):
  X_ijk^abc = sum_d (bd|ai) t_kj^cd - sum_l (ck|jl) t_il^ab,
  W_ijk^abc = X summed over the six simultaneous permutations of the pairs
              (ia), (jb), (kc),
  V_ijk^abc = W + (bj|ck) t_i^a + (ai|ck) t_j^b + (ai|bj) t_k^c,
  Y_ijk^abc = 4 W_abc + W_bca + W_cab - 2 W_acb - 2 W_bac - 2 W_cba,
  E(T) = sum V Y / (3 D),  D = e_i + e_j + e_k - e_a - e_b - e_c.

``textbook_triples`` is an independent pin, not a restatement of helios:
the published spin-orbital (T) (T. D. Crawford and H. F. Schaefer, Rev.
Comput. Chem. 14, 33 (2000)), connected and disconnected amplitudes
  D t_c = P(i/jk) P(a/bc) [sum_e t_jk^ae <ei||bc> - sum_m t_im^bc <ma||jk>],
  D t_d = P(i/jk) P(a/bc) t_i^a <jk||bc>,   E(T) = sum t_c D (t_c + t_d) / 36.
It equals ``closed_shell_triples``, and the reference's term ``spin_triples``
is its negative: the reference's c1 multiplies amp^2 by D > 0.
"""
from __future__ import annotations

import numpy as np

from .spin_ccsd import spin_integrals


def _e(s, *a):
    return np.einsum(s, *a, optimize=True)


def spin_amplitudes(t1, t2):
    """Spin-orbital t1, t2 (occupied spin orbitals first, 2p + s) of closed-shell t1[i, a], t2[i, j, a, b]."""
    o, v = t1.shape
    no, nv = 2 * o, 2 * v
    si = np.arange(no) % 2
    sa = np.arange(nv) % 2
    pi = np.arange(no) // 2
    pa = np.arange(nv) // 2
    t1s = t1[np.ix_(pi, pa)] * (si[:, None] == sa[None, :])
    T = t2                                           # T[i, j, a, b] = t_ij^ab
    direct = T[np.ix_(pi, pi, pa, pa)] * ((si[:, None, None, None] == sa[None, None, :, None])
                                          & (si[None, :, None, None] == sa[None, None, None, :]))
    exch = T[np.ix_(pi, pi, pa, pa)].transpose(0, 1, 3, 2) * ((si[:, None, None, None] == sa[None, None, None, :])
                                                             & (si[None, :, None, None] == sa[None, None, :, None]))
    return t1s, direct - exch


def spin_triples(C, G, h_core, o, t1, t2):
    """E(T) = c1 + c2 + c3 of the reference's spin-orbital loop; returns (E, c1, c2, c3)."""
    f, anti, no, ns = spin_integrals(C, G, h_core, o)
    R = anti.transpose(0, 2, 1, 3)                   # R(p,q,r,s) = <pr||qs>
    t1s, t2s = spin_amplitudes(t1, t2)
    O, Vs = slice(0, no), slice(no, ns)
    eo, ev = np.diag(f)[O], np.diag(f)[Vs]
    Rvooo = R[Vs, O, O, O]                           # R(j?) blocks are taken below explicitly
    # sum1 terms: R(x,y,k,l) t2(i,l,a,b) with x in {i, j}, y in {a, b, c}
    Rovoo = R[O, Vs, O, O]                           # R(j, c, k, l)
    Rvovv = R[Vs, O, Vs, Vs]                         # R(b, k, c, d)
    s1 = (_e("jckl,ilab->ijkabc", Rovoo, t2s) - _e("ickl,jlab->ijkabc", Rovoo, t2s)
          - _e("jcil,klab->ijkabc", Rovoo, t2s) - _e("jakl,ilcb->ijkabc", Rovoo, t2s)
          + _e("iakl,jlcb->ijkabc", Rovoo, t2s) + _e("jail,klcb->ijkabc", Rovoo, t2s)
          - _e("jbkl,ilac->ijkabc", Rovoo, t2s) + _e("ibkl,jlac->ijkabc", Rovoo, t2s)
          + _e("jbil,klac->ijkabc", Rovoo, t2s))
    s2 = (_e("bkcd,ijad->ijkabc", Rvovv, t2s) - _e("bicd,kjad->ijkabc", Rvovv, t2s)
          - _e("bjcd,ikad->ijkabc", Rvovv, t2s) - _e("akcd,ijbd->ijkabc", Rvovv, t2s)
          + _e("aicd,kjbd->ijkabc", Rvovv, t2s) + _e("ajcd,ikbd->ijkabc", Rvovv, t2s)
          - _e("bkad,ijcd->ijkabc", Rvovv, t2s) + _e("biad,kjcd->ijkabc", Rvovv, t2s)
          + _e("bjad,ikcd->ijkabc", Rvovv, t2s))
    del Rvooo
    D = (ev[None, None, None, :, None, None] + ev[None, None, None, None, :, None] + ev[None, None, None, None, None, :]
         - eo[:, None, None, None, None, None] - eo[None, :, None, None, None, None] - eo[None, None, :, None, None, None])
    amp = (s1 - s2) / D
    c1 = float(np.sum(amp * amp * D)) / 36.0
    c2 = float(_e("ijkabc,ia,bjck->", amp, t1s, R[Vs, O, Vs, O])) / 4.0
    c3 = float(_e("ijkabc,ijab,kc->", amp, t2s, f[O, Vs]))
    return c1 + c2 + c3, c1, c2, c3


def mo_integrals(C, G):
    """(pq|rs) over spatial MOs from the ZDO site basis."""
    B = _e("mp,mq->mpq", C, C)
    return _e("mpq,mn,nrs->pqrs", B, G, B)


def closed_shell_triples(C, G, eps, o, t1, t2):
    """The spin-adapted (T) on spatial orbitals; returns E(T)."""
    eri = mo_integrals(C, G)
    v = C.shape[1] - o
    O, V = slice(0, o), slice(o, o + v)
    T = t2                                           # T[i, j, a, b] = t_ij^ab
    vvvo = eri[V, V, V, O]                           # (bd|ai) -> [b, d, a, i]
    vooo = eri[V, O, O, O]                           # (ck|jl) -> [c, k, j, l]
    X = _e("bdai,kjcd->ijkabc", vvvo, T) - _e("ckjl,ilab->ijkabc", vooo, T)
    # W: the six simultaneous permutations of the pairs (ia), (jb), (kc)
    W = (X + X.transpose(0, 2, 1, 3, 5, 4) + X.transpose(1, 0, 2, 4, 3, 5)
         + X.transpose(1, 2, 0, 4, 5, 3) + X.transpose(2, 0, 1, 5, 3, 4) + X.transpose(2, 1, 0, 5, 4, 3))
    ovov = eri[O, V, O, V]                           # (ia|jb) -> [i, a, j, b]
    Vt = (W + _e("jbkc,ia->ijkabc", ovov, t1) + _e("iakc,jb->ijkabc", ovov, t1)
          + _e("iajb,kc->ijkabc", ovov, t1))
    eo, ev = eps[:o], eps[o:]
    D = (eo[:, None, None, None, None, None] + eo[None, :, None, None, None, None] + eo[None, None, :, None, None, None]
         - ev[None, None, None, :, None, None] - ev[None, None, None, None, :, None] - ev[None, None, None, None, None, :])
    Y = (4.0 * W + W.transpose(0, 1, 2, 4, 5, 3) + W.transpose(0, 1, 2, 5, 3, 4)
         - 2.0 * W.transpose(0, 1, 2, 3, 5, 4) - 2.0 * W.transpose(0, 1, 2, 4, 3, 5) - 2.0 * W.transpose(0, 1, 2, 5, 4, 3))
    return float(np.sum(Vt * Y / D)) / 3.0


def textbook_triples(C, G, h_core, o, t1, t2):
    """Spin-orbital (T) of the published formulas; returns (E, E4, E5)."""
    f, g, no, ns = spin_integrals(C, G, h_core, o)
    t1s, t2s = spin_amplitudes(t1, t2)
    O, V = slice(0, no), slice(no, ns)
    eo, ev = np.diag(f)[O], np.diag(f)[V]
    raw = _e("jkae,eibc->ijkabc", t2s, g[V, O, V, V]) - _e("imbc,majk->ijkabc", t2s, g[O, V, O, O])

    def P(x):     # P(i/jk) P(a/bc): f(ijk) - f(jik) - f(kji), then the same on a, b, c
        x = x - x.transpose(1, 0, 2, 3, 4, 5) - x.transpose(2, 1, 0, 3, 4, 5)
        return x - x.transpose(0, 1, 2, 4, 3, 5) - x.transpose(0, 1, 2, 5, 4, 3)

    D = (eo[:, None, None, None, None, None] + eo[None, :, None, None, None, None] + eo[None, None, :, None, None, None]
         - ev[None, None, None, :, None, None] - ev[None, None, None, None, :, None] - ev[None, None, None, None, None, :])
    tc = P(raw) / D
    td = P(_e("ia,jkbc->ijkabc", t1s, g[O, O, V, V])) / D
    e4 = float(np.sum(tc * D * tc)) / 36.0
    e5 = float(np.sum(tc * D * td)) / 36.0
    return e4 + e5, e4, e5
