"""ORACLE (test infrastructure only) -- LR-CCSD excited states of r-ccsd.

Restates the reference's linear-response CCSD (src/methods/coupledCluster/
lrccsd/), which getEnergy runs after a converged r-ccsd when
``states:excited-states-number`` > 0 (src/modules/mod_property.f90:159-175):

* getCCSolution (mod_lrccsd.f90:738-876): the closed-shell t1, t2 become
  spin-orbital amplitudes (convertSpatialToSpinCC, mod_cc.f90:2601-2678), the
  MO Fock matrix is copied to both spins and R(p,q,r,s) = [pq|rs] - [ps|qr]
  = <pr||qs> is built over all 2N spin orbitals (spin_hf_int, :1449-1475).
  Spin orbital 2P+s (0-based) is spatial orbital P with spin s, occupied
  spin orbitals first: the reference's 1-based 2P-1 / 2P.
* projection_lrccsd_spin_hf_intermediates_1 (proj-lrccsd-spin-hf-
  intermediates.f90:1-387): ai1..ai7, Fab, Fij, Fia from t1, t2, R, F, once.
* per iteration: projection_lrccsd_spin_hf_intermediates_2 (:391-515) gives
  at1..at4 from r1, r2 (at5, at6 are computed there but never read);
  projection_lrccsd_singles_spin_hf (proj-lrccsd-spin-hf-1.f90:1-76) and
  projection_lrccsd_doubles_spin_hf (proj-lrccsd-spin-hf-2.f90:1-98) give the
  sigma vector d1, d2 = (H-bar - E_cc) r, doubles on pairs i<j, a<b of equal
  spin parity, antisymmetrised.
* stepLR (mod_lrccsd.f90:216-326): omega = <d|r> / <r|r> over the unique
  amplitudes, d -= omega r, r -= step d, accuracy = (max|d1|, max|d2|), r1 made
  singlet (r1(ia, alpha) = r1(ia, beta)) or triplet (opposite signs),
  normalised (normalize, :393-453), optionally orthogonalised to the states
  found before (orthogonalization, :457-527); then DIIS over (r, d)
  (pushLRVectors / newLRVectors / diisDotProduct, :1081-1225).
* energyLR (:330-389): omega, the reference weight
  r0 = (sum Fia r1 + 1/4 sum R(j,b,i,a) r2(i,j,a,b)) / omega and the average
  excitation level (sum r1^2 + 2 sum' r2^2) / (sum r1^2 + sum' r2^2).
* initLR (:125-172): the CIS guess (prepareGuess, :1229-1355; guessState,
  :1359-1419), one iterator run per state with accuracy lrbd%accuracy * 2^(k-1),
  then the states sorted by omega (resortStates, :531-574).

``hbar_block`` is an independent pin, not a restatement: it builds
e^{-T} H e^{T} exactly in the determinant space of a small molecule and
returns its singles-doubles block minus E_cc, which the sigma equations must
reproduce element by element.

``closed_shell_jacobian`` is the second pin and the design of the device
path: the Jacobian of the closed-shell r-ccsd residual (the same equations
the engine evaluates) with respect to the spatial amplitudes, in the
coordinates t1[i, a] and the packed pairs (ia) <= (jb). The residual is a
polynomial of degree four in the amplitudes, so its linear part is extracted
exactly from four evaluations. Its eigenvalues are the singlet LR-CCSD
excitation energies.

Feasible for N <= 12 sites (R holds (2N)^4 doubles); ``hbar_block`` for N <= 6.
"""
from __future__ import annotations

import numpy as np

from .rhf import IteratorRules
from .spin_ccsd import spin_integrals
from .triples import spin_amplitudes


def _e(s, *a):
    return np.einsum(s, *a, optimize=True)


# ---------------------------------------------------------------- spin-orbital problem

class SpinProblem:
    """F, R = <pr||qs>, t1, t2 in spin orbitals (getCCSolution), with index masks."""

    def __init__(self, C, G, h_core, o, t1, t2):
        f, anti, no, ns = spin_integrals(C, G, h_core, o)
        self.F = f
        self.R = anti.transpose(0, 2, 1, 3)          # R(p,q,r,s) = <pr||qs>
        self.no, self.ns = no, ns
        self.nv = ns - no
        self.t1, self.t2 = spin_amplitudes(t1, t2)
        so = np.arange(no) % 2
        sv = np.arange(self.nv) % 2
        self.same1 = (so[:, None] == sv[None, :])                                  # singles allowed
        par_o = (so[:, None] + so[None, :]) % 2
        par_v = (sv[:, None] + sv[None, :]) % 2
        self.par2 = par_o[:, :, None, None] == par_v[None, None, :, :]             # doubles allowed
        iu = np.arange(no)[:, None] < np.arange(no)[None, :]
        au = np.arange(self.nv)[:, None] < np.arange(self.nv)[None, :]
        self.upper = iu[:, :, None, None] & au[None, None, :, :]                   # i<j, a<b
        self.O, self.V = slice(0, no), slice(no, ns)

    def blk(self, spec):
        return self.R[tuple(self.O if c == "o" else self.V for c in spec)]


def intermediates(P: SpinProblem):
    """projection_lrccsd_spin_hf_intermediates_1, parts 1-10 in order."""
    t1, t2, F = P.t1, P.t2, P.F
    O, V = P.O, P.V
    ovov, ovvv, oovo, ooov = P.blk("ovov"), P.blk("ovvv"), P.blk("oovo"), P.blk("ooov")
    X = {}
    # part 1 (:16-32)
    X["ai7"] = _e("ibac->iabc", ovvv) - _e("ibjc,ja->iabc", ovov, t1)
    # part 2 (:34-50)
    X["ai6"] = _e("ikja->ijka", ooov) - _e("iajc,kc->ijka", ovov, t1)
    # part 3 (:52-83)
    s1 = _e("ka,kcbd->abcd", t1, ovvv) - _e("kb,kcad->abcd", t1, ovvv)
    s2 = _e("ka,lb,kcld->abcd", t1, t1, ovov)
    s3 = _e("klab,kcld->abcd", t2, ovov)
    ai5 = (_e("acbd->abcd", P.blk("vvvv")) - s1 + s2) / 2 + s3 / 4
    X["ai5"] = ai5
    # part 4 (:85-116)
    s1 = _e("jc,kilc->ijkl", t1, ooov) - _e("ic,kjlc->ijkl", t1, ooov)
    s2 = _e("ic,jd,kcld->ijkl", t1, t1, ovov)
    s3 = _e("ijcd,kcld->ijkl", t2, ovov)
    ai4 = (_e("ikjl->ijkl", P.blk("oooo")) + s1 + s2) / 2 + s3 / 4
    X["ai4"] = ai4
    # part 5 (:118-183)
    s1 = _e("id,abcd->icab", t1, ai5)
    Q = P.blk("oovv") - _e("ikad,lckd->liac", t2, ovov)        # ss1/ss2 of part 5
    s2 = _e("lb,liac->icab", t1, Q) - _e("la,libc->icab", t1, Q)
    s3 = _e("la,kb,clik->icab", t1, t1, P.blk("vooo"))
    s4 = _e("ld,kiab,ckdl->icab", t1, t2, P.blk("vovo"))
    s5 = _e("ikab,kc->icab", t2, F[O, V])
    s6 = _e("klab,ikcl->icab", t2, oovo)
    s7 = _e("ikad,kcbd->icab", t2, ovvv) - _e("ikbd,kcad->icab", t2, ovvv)
    X["ai3"] = -_e("iacb->icab", ovvv) + 2 * s1 - s2 + s3 - s4 + s5 - s6 / 2 + s7
    # part 6 (:185-252)
    s1 = _e("la,ijkl->ijka", t1, ai4)
    Pm = P.blk("oovv") - _e("xlac,kdlc->xkda", t2, ovov)        # ss1/ss2 of part 6
    s2 = _e("id,jkda->ijka", t1, Pm) - _e("jd,ikda->ijka", t1, Pm)
    s3 = _e("id,jc,kdac->ijka", t1, t1, ovvv)
    s4 = _e("ld,ijac,kdlc->ijka", t1, t2, ovov)
    s5 = _e("ijac,kc->ijka", t2, F[O, V])
    s6 = _e("ijcd,kcad->ijka", t2, ovvv)
    s7 = _e("ilac,jkcl->ijka", t2, oovo) - _e("jlac,ikcl->ijka", t2, oovo)
    X["ai2"] = -_e("ikja->ijka", ooov) + 2 * s1 + s2 - s3 - s4 + s5 - s6 / 2 + s7
    # part 7 (:254-284)
    s1 = _e("lb,jila->iajb", t1, ooov)
    s2 = _e("id,jabd->iajb", t1, ovvv)
    s3 = _e("id,lb,jald->iajb", t1, t1, ovov) - _e("ilbd,jald->iajb", t2, ovov)
    X["ai1"] = _e("ijab->iajb", P.blk("oovv")) - s1 - s2 + s3
    # part 8 (:286-325)
    s1 = _e("ka,kb->ab", t1, F[O, V])
    s2 = _e("kc,kbac->ab", t1, ovvv)
    s3 = _e("kc,la,lbkc->ab", t1, t1, ovov)
    s4 = _e("lkac,lbkc->ab", t2, ovov)
    X["Fab"] = F[V, V] - s1 - s2 - s3 - s4 / 2
    # part 9 (:327-366)
    s1 = _e("ic,jc->ij", t1, F[O, V])
    s2 = _e("kc,jikc->ij", t1, ooov)
    s3 = _e("ic,kd,jckd->ij", t1, t1, ovov)
    s4 = _e("ikdc,jdkc->ij", t2, ovov)
    X["Fij"] = F[O, O] + s1 + s2 + s3 + s4 / 2
    # part 10 (:368-383)
    X["Fia"] = F[O, V] + _e("kd,iakd->ia", t1, ovov)
    return X


def sigma(P: SpinProblem, X, r1, r2):
    """intermediates_2 + singles + doubles projections: (d1, d2) for (r1, r2)."""
    t2 = P.t2
    ovov = P.blk("ovov")
    at1 = _e("kc,jkic->ij", r1, X["ai6"])
    at2 = _e("kc,kabc->ab", r1, X["ai7"])
    at3 = _e("ikcd,jckd->ij", r2, ovov) / 2
    at4 = _e("klac,kblc->ab", r2, ovov) / 2
    d1 = (_e("ab,ib->ia", X["Fab"], r1) - _e("ij,ja->ia", X["Fij"], r1) - _e("ibja,jb->ia", X["ai1"], r1)
          + _e("jb,ijab->ia", X["Fia"], r2) - _e("jkib,jkab->ia", X["ai6"], r2) / 2
          - _e("jabc,ijbc->ia", X["ai7"], r2) / 2)
    d1 = d1 * P.same1
    ai1, ai2, ai3 = X["ai1"], X["ai2"], X["ai3"]
    A13, A24 = at1 + at3, at2 + at4
    x = (_e("ic,jcab->ijab", r1, ai3) - _e("jc,icab->ijab", r1, ai3)
         + _e("bc,ijac->ijab", X["Fab"], r2) - _e("ac,ijbc->ijab", X["Fab"], r2)
         + _e("ka,ijkb->ijab", r1, ai2) - _e("kb,ijka->ijab", r1, ai2)
         + _e("ik,jkab->ijab", X["Fij"], r2) - _e("jk,ikab->ijab", X["Fij"], r2)
         + _e("il,jlab->ijab", A13, t2) - _e("jl,ilab->ijab", A13, t2)
         + _e("ad,ijbd->ijab", A24, t2) - _e("bd,ijad->ijab", A24, t2)
         + _e("jkac,ickb->ijab", r2, ai1) - _e("ikac,jckb->ijab", r2, ai1)
         + _e("ikbc,jcka->ijab", r2, ai1) - _e("jkbc,icka->ijab", r2, ai1)
         + _e("klab,ijkl->ijab", r2, X["ai4"]) + _e("ijcd,abcd->ijab", r2, X["ai5"]))
    return d1, antisym_from_upper(P, x * P.par2)


def antisym_from_upper(P: SpinProblem, x):
    """x on i<j, a<b copied to the three other antisymmetric positions; the rest zero."""
    u = np.where(P.upper, x, 0.0)
    return u - u.transpose(1, 0, 2, 3) - u.transpose(0, 1, 3, 2) + u.transpose(1, 0, 3, 2)


# ---------------------------------------------------------------- the iteration

def cis_guess(F, C, G, o, nstates, threshold=0.1):
    """prepareGuess 'cis' + guessState for r-ccsd: per state the spatial singles
    whose CIS coefficient reaches the threshold, as (i, a, coefficient) lists.

    A(ia, jb) = 2(ai|jb) - (ab|ji) + delta (e_a - e_i) (spat_hf_int with
    (a,i,j,b), mod_lrccsd.f90:1262-1282); states in ascending order. The reference
    diagonalises the two-copy block matrix [[A, 0], [0, A]] and takes every
    other root; each root is doubly degenerate there, so which vector of the
    pair its eigensolver returns is not fixed. The restatement takes A's own
    eigenvector, which is one member of every such pair.
    """
    v = C.shape[1] - o
    B = _e("mp,mq->mpq", C, C)
    eri = _e("mpq,mn,nrs->pqrs", B, G, B)
    e = np.diag(F)
    Ov, Vv = slice(0, o), slice(o, o + v)
    A = (2 * _e("aijb->iajb", eri[Vv, Ov, Ov, Vv]) - _e("abji->iajb", eri[Vv, Vv, Ov, Ov])).reshape(o * v, o * v)
    A[np.diag_indices_from(A)] += (e[None, o:] - e[:o, None]).ravel()
    w, U = np.linalg.eigh(A)
    out = []
    for k in range(nstates):
        sel = [(m // v, m % v, float(U[m, k])) for m in range(o * v) if abs(U[m, k]) >= threshold]
        out.append(sel)
    return out, w


def state_vector(P: SpinProblem, sel, spin=0):
    """guessState: r1(2i, 2a) = c, r1(2i+1, 2a+1) = +-c (0-based spin orbitals), r2 = 0."""
    r1 = np.zeros((P.no, P.nv))
    for i, a, c in sel:
        r1[2 * i, 2 * a] = c
        r1[2 * i + 1, 2 * a + 1] = c if spin == 0 else -c
    return r1, np.zeros((P.no, P.no, P.nv, P.nv))


class LRDiis:
    """pushLRVectors / newLRVectors / diisDotProduct over the allowed unique amplitudes."""

    def __init__(self, P: SpinProblem, nd):
        self.P, self.nd = P, nd
        self.m1 = P.same1
        self.m2 = P.upper & P.par2
        self.st, self.sd = [], []
        self.B = np.zeros((nd + 1, nd + 1))

    def push(self, r1, r2, d1, d2):
        self.st.insert(0, np.concatenate([r1[self.m1], r2[self.m2]]))
        self.sd.insert(0, np.concatenate([d1[self.m1], d2[self.m2]]))
        del self.st[self.nd:], self.sd[self.nd:]

    def extrapolate(self, iteration, r1, r2):
        n = min(iteration, self.nd)
        B = self.B
        B[1:n, 1:n] = B[0:n - 1, 0:n - 1].copy()
        for k in range(n):
            B[k, 0] = B[0, k] = float(self.sd[k] @ self.sd[0])
        if n == 1:
            return r1, r2
        A = np.ones((n + 1, n + 1)); A[:n, :n] = B[:n, :n]; A[n, n] = 0.0
        lam, U = np.linalg.eigh(A)                     # tred4 + pseudo-inverse, :1148-1155
        c = (U[:n, :] * U[n, :][None, :] / lam[None, :]).sum(axis=1)
        x = sum(c[k] * self.st[k] for k in range(n))
        n1 = int(self.m1.sum())
        r1 = r1.copy(); r1[self.m1] = x[:n1]
        u = np.zeros_like(r2); u[self.m2] = x[n1:]
        return r1, u - u.transpose(1, 0, 2, 3) - u.transpose(0, 1, 3, 2) + u.transpose(1, 0, 3, 2)


def _norms(P, r1, r2):
    return float((r1 * r1).sum()), float((r2[P.upper] ** 2).sum())


def lr_energy(P: SpinProblem, X, r1, r2, omega):
    """energyLR: (omega, r0, average excitation level)."""
    s1, s2 = _norms(P, r1, r2)
    ael = (s1 + 2 * s2) / (s1 + s2)
    num = float((X["Fia"] * r1).sum()) + float(_e("jbia,ijab->", P.blk("ovov"), r2)) / 4
    return omega, num / omega, ael


def lr_solve(C, G, h_core, F, o, t1, t2, nstates=1, spin=0, eps=1e-6, maxiter=10000, step=(0.03, 0.03),
             diis=True, nd=20, orthogonalize=False, guess_threshold=0.1, guesses=None):
    """initLR: returns dict(omega[k], r0[k], ael[k], status[k], iterations[k], r1[k], r2[k]) sorted by omega."""
    P = SpinProblem(C, G, h_core, o, t1, t2)
    X = intermediates(P)
    if guesses is None:
        guesses, _ = cis_guess(F, C, G, o, nstates, guess_threshold)
    held = []
    for k in range(nstates):
        r1, r2 = state_vector(P, guesses[k], spin)
        hist = LRDiis(P, nd) if diis else None
        rules = IteratorRules(maxiter, eps * 2.0 ** k)
        status, omega = None, 0.0
        while status is None:
            d1, d2 = sigma(P, X, r1, r2)
            # stepLR
            s_dr = float((d1 * r1).sum()) + float((d2[P.upper] * r2[P.upper]).sum())
            s1, s2 = _norms(P, r1, r2)
            omega = s_dr / (s1 + s2)
            d1 = d1 - omega * r1
            r1 = r1 - step[0] * d1
            d2 = d2 - omega * r2
            r2 = r2 - step[1] * d2
            acc = (float(np.abs(d1).max()), float(np.abs(d2).max()))
            ra, rb = r1[0::2, 0::2], r1[1::2, 1::2]
            rez = (ra + rb) / 2 if spin == 0 else (ra - rb) / 2
            r1 = r1.copy()
            r1[0::2, 0::2] = rez
            r1[1::2, 1::2] = rez if spin == 0 else -rez
            s1, s2 = _norms(P, r1, r2)
            scale = 1.0 / np.sqrt(s1 + s2)
            r1 = r1 * scale
            r2 = antisym_from_upper(P, r2 * scale)
            if orthogonalize and held:
                ov = [float((r1 * h1).sum()) + float((r2 * h2).sum()) for h1, h2, _ in held]
                r1 = r1 - sum(c * h1 for c, (h1, _, _) in zip(ov, held))
                r2 = r2 - sum(c * h2 for c, (_, h2, _) in zip(ov, held))
            if max(acc) >= rules.eps and hist is not None:
                hist.push(r1, r2, d1, d2)
                r1, r2 = hist.extrapolate(rules.iteration + 1, r1, r2)
            status = rules.update(max(acc))
        w, r0, ael = lr_energy(P, X, r1, r2, omega)
        held.append((r1, r2, {"omega": w, "r0": r0, "ael": ael, "status": status, "iterations": rules.iteration}))
    held.sort(key=lambda h: h[2]["omega"])             # resortStates
    out = {key: np.array([h[2][key] for h in held]) for key in ("omega", "r0", "ael", "status", "iterations")}
    out["r1"] = [h[0] for h in held]
    out["r2"] = [h[1] for h in held]
    return out


# ---------------------------------------------------------------- pin 1: determinant-space H-bar

def _jw_annihilators(n):
    """Jordan-Wigner annihilation operators of n modes as sparse 2^n x 2^n matrices (mode 0 leftmost)."""
    import scipy.sparse as sp
    Z = sp.csr_matrix(np.diag([1.0, -1.0]))
    I2 = sp.identity(2, format="csr")
    lower = sp.csr_matrix(np.array([[0.0, 1.0], [0.0, 0.0]]))     # |0><1|
    ops = []
    for p in range(n):
        m = sp.identity(1, format="csr")
        for q in range(n):
            m = sp.kron(m, Z if q < p else (lower if q == p else I2), format="csr")
        ops.append(m)
    return ops


def hbar_block(C, G, h_core, o, t1, t2):
    """The singles-doubles block of e^{-T} H e^{T} - E_cc in the determinant space.

    Basis: |i->a> = a+_a a_i |HF> for every (i, a), |ij->ab> = a+_a a+_b a_j a_i |HF>
    for i<j, a<b (all spins). Returns (A, singles index list, doubles index list, E_cc,
    top) with E_cc = <HF|H-bar|HF> (electronic, without the site-site repulsion
    constant) and top[mu] = <HF|H-bar|mu>, the row that gives a state's reference
    weight r0 = top . r / omega.
    """
    import scipy.sparse as sp
    f, anti, no, ns = spin_integrals(C, G, h_core, o)
    N = C.shape[0]
    hmo = C.T @ h_core @ C
    order = [2 * p + s for p in range(o) for s in (0, 1)] + [2 * p + s for p in range(o, N) for s in (0, 1)]
    spat = np.array([k // 2 for k in order]); spin = np.array([k % 2 for k in order])
    h = hmo[np.ix_(spat, spat)] * (spin[:, None] == spin[None, :])
    a = _jw_annihilators(ns)
    ad = [x.T.tocsr() for x in a]
    dim = 2 ** ns
    terms = []
    for p in range(ns):
        for q in range(ns):
            if h[p, q] != 0.0:
                terms.append((h[p, q] * (ad[p] @ a[q])).tocoo())
    pairs = [(p, q) for p in range(ns) for q in range(p + 1, ns)]
    dens = {pq: ad[pq[0]] @ ad[pq[1]] for pq in pairs}
    ann = {rs: a[rs[1]] @ a[rs[0]] for rs in pairs}
    for pq in pairs:                                  # sum_{p<q, r<s} <pq||rs> a+p a+q a_s a_r
        for rs in pairs:
            g = anti[pq[0], pq[1], rs[0], rs[1]]
            if g != 0.0:
                terms.append((g * (dens[pq] @ ann[rs])).tocoo())
    H = sp.csr_matrix((np.concatenate([m.data for m in terms]),
                       (np.concatenate([m.row for m in terms]), np.concatenate([m.col for m in terms]))),
                      shape=(dim, dim))
    t1s, t2s = spin_amplitudes(t1, t2)
    nv = ns - no
    T = sp.csr_matrix((dim, dim))
    singles = [(i, c) for i in range(no) for c in range(nv)]
    doubles = [(i, j, c, d) for i in range(no) for j in range(i + 1, no) for c in range(nv) for d in range(c + 1, nv)]
    exc1 = {(i, c): ad[no + c] @ a[i] for i, c in singles}
    exc2 = {(i, j, c, d): ad[no + c] @ ad[no + d] @ a[j] @ a[i] for i, j, c, d in doubles}
    for (i, c), op in exc1.items():
        if t1s[i, c] != 0.0:
            T = T + t1s[i, c] * op
    for (i, j, c, d), op in exc2.items():
        if t2s[i, j, c, d] != 0.0:
            T = T + t2s[i, j, c, d] * op
    hf = np.zeros(dim)
    hf[int("".join("1" if p < no else "0" for p in range(ns)), 2)] = 1.0

    def expT(x, sign):
        out, term = x.copy(), x.copy()
        for k in range(1, no + 1):
            term = sign * (T @ term) / k
            out = out + term
        return out

    def hbar(x):
        return expT(H @ expT(x, 1.0), -1.0)

    e_cc = float(hf @ hbar(hf))
    basis = [exc1[s] @ hf for s in singles] + [exc2[d] @ hf for d in doubles]
    Bm = np.array(basis)                              # rows: basis vectors
    A = np.empty((len(basis), len(basis)))
    top = np.empty(len(basis))
    for col, x in enumerate(basis):
        y = hbar(x)
        A[:, col] = Bm @ y - e_cc * (Bm @ x)
        top[col] = hf @ y
    return A, singles, doubles, e_cc, top


# ---------------------------------------------------------------- pin 2: closed-shell Jacobian

def closed_shell_pack(x1, x2):
    """t1[i, a] and the pairs (ia) <= (jb) of x2[i, j, a, b] (i outer, a inner) as one vector."""
    from .ccsd_fact import pair_matrix
    return np.concatenate([x1.ravel(), pair_matrix(x2)[np.triu_indices(x1.size)]])


def closed_shell_unpack(x, o, v):
    """Inverse of closed_shell_pack; x2 gets the pair symmetry x2[j, i, b, a] = x2[i, j, a, b]."""
    from .ccsd_fact import from_pair_matrix
    n1 = o * v
    M = np.zeros((n1, n1)); M[np.triu_indices(n1)] = x[n1:]
    M = M + np.triu(M, 1).T
    return x[:n1].reshape(o, v), from_pair_matrix(M, o, v)


def closed_shell_jacobian(F, C, G, o, t1, t2, eps=1e-3):
    """d(Omega)/d(t) of the closed-shell residual at (t1, t2), in the coordinates
    t1[i, a] + packed pairs (ia) <= (jb); Omega1 = d1 and Omega2 = (2 d2 + d2^(ab)) / 3
    (the reference's d2 is 2 Omega2(ijab) - Omega2(ijba), so this inverts its '2-1' form).

    Omega is a polynomial of degree four, so its odd part in a step h r is
    h J r + h^3 K(r) exactly and [8 (O(h) - O(-h)) - (O(2h) - O(-2h))] / (12 h) = J r.
    """
    from . import ccsd_fact
    I = ccsd_fact.Integrals(C, G, o)
    v = t1.shape[1]
    n = o * v + o * v * (o * v + 1) // 2

    def omega(x):
        a1, a2 = closed_shell_unpack(x, o, v)
        d1, d2 = ccsd_fact.residuals(F, I, a1, a2)
        return closed_shell_pack(d1, (2 * d2 + d2.transpose(0, 1, 3, 2)) / 3)

    x0 = closed_shell_pack(t1, t2)
    J = np.empty((n, n))
    for k in range(n):
        r = np.zeros(n); r[k] = 1.0
        odd1 = omega(x0 + eps * r) - omega(x0 - eps * r)
        odd2 = omega(x0 + 2 * eps * r) - omega(x0 - 2 * eps * r)
        J[:, k] = (8 * odd1 - odd2) / (12 * eps)
    return J
