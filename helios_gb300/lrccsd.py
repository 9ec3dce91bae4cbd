"""LR-CCSD excited states (lr-r-ccsd) on the GB300 CCSD engine.

helios runs linear-response CCSD after a converged r-ccsd when
``states:excited-states-number`` > 0 (getEnergy, src/modules/mod_property.f90:
159-175; src/methods/coupledCluster/lrccsd/mod_lrccsd.f90). It solves the
right eigenproblem (H-bar - E_cc) r = omega r over singles and doubles, one
state at a time, with its own iteration, and reports E_CCSD + omega.

The sigma vector (H-bar - E_cc) r needs no equations of its own here. The
r-ccsd residual Omega(t) that the engine evaluates is a polynomial of degree
four in the amplitudes, and its Jacobian at the converged amplitudes is
H-bar - E_cc on singlet excitations, written in the spin-adapted coordinates
t1[i, a], t2[i, j, a, b]. The odd part of Omega(t + h r) in h is
h J r + h^3 K(r), so

    J r = [8 (Omega(t + h r) - Omega(t - h r)) - (Omega(t + 2h r) - Omega(t - 2h r))] / (12 h)

holds exactly. The four residuals are four copies of the molecule in ONE
engine batch, and every state being solved adds four copies, so all states
advance in the same launches. The engine hands a residual back through one
stepCC: after ``set_guess(x)`` (which also clears the DIIS history, so the
iteration mixes nothing) and one ``iterationCC`` with unit steps,
t1' = x1 + d1 / (F_ii - F_aa) and t2' = x2 + 3 Omega2 / (F_ii + F_jj - F_aa - F_bb)
(mod_cc.f90:987-1017).

The host part restates the reference's iteration on those coordinates:

* stepLR (mod_lrccsd.f90:216-326), normalize (:393-453), orthogonalization
  (:457-527), pushLRVectors / newLRVectors / diisDotProduct (:1081-1225) and
  energyLR (:330-389). The reference works on spin orbitals and sums over its
  unique amplitudes (i<j, a<b). A singlet vector's spin-orbital form follows
  from the spatial one by the amplitude rules of convertSpatialToSpinCC
  (mod_cc.f90:2601-2678), which turns those sums into
      <x, y> = 2 sum x1 y1 + sum x2 y2 + 1/2 sum (x2 - x2^ab)(y2 - y2^ab)
  (x2^ab: a and b swapped). The largest spin-orbital doubles element is
  max(|x2|, |x2 - x2^ab|). With these, every iterate equals the reference's.
* prepareGuess / guessState (:1229-1419): the lowest CIS (or 'rpa') roots
  of A(ia, jb) = 2(ai|jb) - (ab|ji) + delta (e_a - e_i), keeping the singles
  whose coefficient reaches linear-response:guess-threshold.
* initLR (:125-172): state k converges to accuracy * 2^(k-1); the states are
  sorted by omega at the end (resortStates, :531-574). Without
  orthogonalization the states do not depend on each other and iterate
  together; with it they run one after another as in the reference.
* energyLR's reference weight r0 = (2 sum Ft_ia r1 + sum L_iajb r2) / omega,
  Ft_ia = F_ia + sum_kd L_iakd t1_kd, L_iajb = 2(ia|jb) - (ib|ja) (the
  spin-summed form of sum Fia r1 + 1/4 sum R(j,b,i,a) r2(i,j,a,b)).

The CIS matrix and r0 need MO integrals on the host; they come from the
engine's orbitals and the Coulomb matrix of ``coulomb_matrix``, which follows
the engine's model builder (readMoleculeInformation.f90:216-264).

Triplet states (``states:spin`` = 1) have no spin-adapted closed-shell
residual to differentiate and are not provided.
"""
from __future__ import annotations

from dataclasses import dataclass, replace

import numpy as np

from . import api
from .molecules import Molecule
from .polariz import BOHR_RADIUS, HARTREE_ENERGY, _align

STATUS_CONVERGED, STATUS_MAXITER, STATUS_DIVERGED, STATUS_STAGNATED = 1, -1, -2, -3


@dataclass
class LRKeywords:
    """``states`` and ``linear-response`` keys (src/input/definebd.f90:71-72, 159-171)."""
    excited_states_number: int = 1      # states:excited-states-number (0..3; 0 means no LR run)
    spin: int = 0                       # states:spin (0 singlet)
    guess: str = "cis"                  # linear-response:guess ('cis' or 'rpa')
    guess_threshold: float = 0.1        # linear-response:guess-threshold
    max_iterations: int = 10000         # linear-response:max-iterations
    accuracy: float = 6                 # linear-response:accuracy (exponent, 10^-value)
    r1_step: float = 0.03               # linear-response:r1-step
    r2_step: float = 0.03               # linear-response:r2-step
    orthogonalization: bool = False     # linear-response:orthogonalization
    diis_enabled: bool = True           # linear-response:diis-enabled
    diis_steps: int = 20                # linear-response:diis-steps
    store_solution: bool = True         # linear-response:store-solution (seed the next run, e.g. the next field point)
    store_solution_threshold: float = 2  # linear-response:store-solution-threshold (exponent)
    store_solution_mode: str = "r1r2"   # linear-response:store-solution-mode


# ---------------------------------------------------------------- spin-adapted vector algebra

def swap_ab(x2):
    return x2.transpose(0, 1, 3, 2)


def _dots(x, y):
    """(sum x1 y1, sum x2 y2, sum x2 y2^ab) without temporaries of the doubles size."""
    return (float(np.vdot(x[0], y[0])), float(np.vdot(x[1], y[1])),
            float(np.einsum("ijab,ijba->", x[1], y[1], optimize=False)))


def inner(x, y):
    """Sum over the reference's unique spin-orbital amplitudes of two singlet vectors:
    2 sum x1 y1 + sum x2 y2 + 1/2 sum (x2 - x2^ab)(y2 - y2^ab) = 2 x1.y1 + 2 x2.y2 - x2.y2^ab."""
    s1, s2, sx = _dots(x, y)
    return 2.0 * s1 + 2.0 * s2 - sx


def inner_full(x, y):
    """Sum over ALL spin-orbital elements (orthogonalization's overlap, :466-496):
    2 x1.y1 + 4 x2.y2 + 2 (x2 - x2^ab).(y2 - y2^ab) = 2 x1.y1 + 8 x2.y2 - 4 x2.y2^ab."""
    s1, s2, sx = _dots(x, y)
    return 2.0 * s1 + 8.0 * s2 - 4.0 * sx


def pair_symmetric(x2):
    """x2 made exactly pair-symmetric, x2[j, i, b, a] = x2[i, j, a, b]: the spin-adapted form of
    normalize's refill of the antisymmetric r2 from its unique elements (:436-447)."""
    return 0.5 * (x2 + x2.transpose(1, 0, 3, 2))


def max_abs(x):
    """(max|d1|, max|d2|) of the spin-orbital vector."""
    x1, x2 = x
    return float(np.abs(x1).max()), max(float(np.abs(x2).max()), float(np.abs(x2 - swap_ab(x2)).max()))


# ---------------------------------------------------------------- integrals on the host

def coulomb_matrix(mol: Molecule, kind: str = "ohno-klopman") -> np.ndarray:
    """The engine's site Coulomb matrix gamma (centred coordinates, trConst = 1/(a0 Eh))."""
    c = np.asarray(mol.coords, dtype=np.float64)
    c = c - c.sum(axis=0) / c.shape[0]
    g_site = np.asarray(mol.gamma, dtype=np.float64)
    r = np.sqrt(((c[:, None, :] - c[None, :, :]) ** 2).sum(-1))
    med = (g_site[:, None] + g_site[None, :]) / 2.0
    tr = 1.0 / (BOHR_RADIUS * HARTREE_ENERGY)
    if kind == "ohno-klopman":
        return med / np.sqrt(1.0 + (tr * med * r) ** 2)
    if kind == "mataga-nishimoto":
        return med / (1.0 + tr * med * r)
    if kind == "hubbard":
        return np.diag(g_site)
    raise ValueError(f"unknown coulomb-integrals type {kind!r}")


class MOIntegrals:
    """(pq|rs) blocks of the ZDO model in the MO basis: J[i,a,j,b] = (ia|jb), Kvo[i,a,j,b] = (ab|ij)."""

    def __init__(self, C, G, o):
        N = C.shape[0]
        v = N - o
        Co, Cv = C[:, :o], C[:, o:]
        Bov = (Co[:, :, None] * Cv[:, None, :]).reshape(N, o * v)
        Bvv = (Cv[:, :, None] * Cv[:, None, :]).reshape(N, v * v)
        Boo = (Co[:, :, None] * Co[:, None, :]).reshape(N, o * o)
        self.J = (Bov.T @ G @ Bov).reshape(o, v, o, v)                            # (ia|jb)
        self.Kvo = (Bvv.T @ G @ Boo).reshape(v, v, o, o).transpose(2, 0, 3, 1)     # (ab|ij) -> [i,a,j,b]
        self.L = 2.0 * self.J - self.J.transpose(0, 3, 2, 1)                     # 2(ia|jb) - (ib|ja)


def cis_matrix(F, I: MOIntegrals):
    """A(ia, jb) = 2(ai|jb) - (ab|ji) + delta (e_a - e_i) (prepareGuess, mod_lrccsd.f90:1262-1276)."""
    o, v = I.J.shape[0], I.J.shape[1]
    e = np.diag(F)
    A = (2.0 * I.J - I.Kvo).reshape(o * v, o * v)
    A[np.diag_indices_from(A)] += (e[None, o:] - e[:o, None]).ravel()
    return A


def guess_vectors(F, I: MOIntegrals, nstates, kind="cis", threshold=0.1):
    """prepareGuess + guessState: per state the singles (i, a, c) with |c| >= threshold, and the roots."""
    o, v = I.J.shape[0], I.J.shape[1]
    A = cis_matrix(F, I)
    if kind == "cis":
        w, U = np.linalg.eigh(A)
    elif kind == "rpa":
        Bm = (2.0 * I.J - I.J.transpose(0, 3, 2, 1)).reshape(o * v, o * v)   # 2(ai|bj) - (aj|bi)
        w, U = np.linalg.eigh(np.block([[A, Bm], [Bm, A]]))
        U = U[:o * v]
    else:
        raise ValueError(f"linear-response:guess {kind!r}: the guesses are 'cis' and 'rpa'")
    out = []
    for k in range(nstates):
        out.append([(m // v, m % v, float(U[m, k])) for m in range(o * v) if abs(U[m, k]) >= threshold])
    return out, w


def guess_space(F, I: MOIntegrals, n):
    """The n lowest CIS vectors, whole, as (r1, 0) (the Davidson solver's first basis)."""
    o, v = I.J.shape[0], I.J.shape[1]
    _, U = np.linalg.eigh(cis_matrix(F, I))
    return [(U[:, k].reshape(o, v).copy(), np.zeros((o, o, v, v))) for k in range(n)]


def seed_vector(sel, o, v):
    r1 = np.zeros((o, v))
    for i, a, c in sel:
        r1[i, a] = c
    return r1, np.zeros((o, o, v, v))


# ---------------------------------------------------------------- the device sigma

class DeviceSigma:
    """J r for up to ``nvec`` vectors per call: four residual evaluations per vector in one batch."""

    def __init__(self, mol: Molecule, keywords: api.Keywords, t1, t2, C0, nvec=1, h=1e-2, engine=None,
                 precision="exact"):
        # the residual comes back through the "2-1" step: t2' = x2 + 3 Omega2 / D2; its
        # contractions run on the 7-slice tensor-core GEMM, whose error is below the FP64
        # GEMM's (precision "exact"), or on the FP64 CUDA cores ("fp64")
        kw = replace(keywords, precision=precision, guess="reference", t1_step=1.0, t2_step=1.0, projection_type="2-1")
        self.cc = (engine or api.CoupledCluster)([mol] * (4 * nvec), kw)
        self.cc.initCC()
        # arrays in the engine's column-major layout, so that no call transposes
        self.t1 = np.asfortranarray(t1, dtype=np.float64)
        self.t2 = np.asfortranarray(t2, dtype=np.float64)
        self.h, self.nvec = h, nvec
        self.calls = 0                                      # engine iterations (one per call)
        self.eps = 10.0 ** (-keywords.accuracy)
        o = t1.shape[0]
        # each copy's orbital signs as +-1 tensors (None where every sign is +1; copies with
        # the same signs share them) and its denominators times those signs, which turn a
        # copy's step in its own signs, stepCC(x) - x, into the ground state's residual
        self.signs, self._sign_tensors, self._t_in, self.DS1, self.DS2 = [], {}, {}, [], []
        for k in range(4 * nvec):
            s = self.cc.scf(k)
            sg = _align(C0, s["C"])
            if np.abs(s["C"] * sg[None, :] - C0).max() > 1e-8:
                raise RuntimeError("the evaluator's orbitals differ from the ground state's beyond a sign")
            key = sg.tobytes()
            if key not in self._sign_tensors:
                so, sv = sg[:o], sg[o:]
                self._sign_tensors[key] = None if np.all(sg == 1.0) else (
                    np.asfortranarray(so[:, None] * sv[None, :]),
                    np.asfortranarray(so[:, None, None, None] * so[None, :, None, None]
                                      * sv[None, None, :, None] * sv[None, None, None, :]))
                self._t_in[key] = self._basis_of(key, self.t1, self.t2)
            self.signs.append(key)
            e = np.diag(s["F"])
            eo, ev = e[:o], e[o:]
            D1 = np.asfortranarray(eo[:, None] - ev[None, :])
            D2 = np.asfortranarray(eo[:, None, None, None] + eo[None, :, None, None]
                                   - ev[None, None, :, None] - ev[None, None, None, :])
            DS1, DS2 = self._basis_of(key, D1, D2)
            self.DS1.append(np.asfortranarray(DS1))
            self.DS2.append(np.asfortranarray(DS2))

    def _basis_of(self, key, x1, x2):
        """Amplitudes between the ground state's orbital signs and a copy's (a product with +-1)."""
        S = self._sign_tensors[key]
        return (x1, x2) if S is None else (x1 * S[0], x2 * S[1])

    def __call__(self, vecs):
        """J r for each r: the five-point stencil (8 (O(+h) - O(-h)) - (O(+2h) - O(-2h))) / 12 h
        of the residual O(t + c h r) = (stepCC(x) - x) D for t1 and (stepCC(x) - x) D / 3 for t2,
        formed in place (the signs are exact: (a - x s) s d = (a s - x) d bit for bit)."""
        if len(vecs) > self.nvec:
            raise ValueError(f"{len(vecs)} vectors for an evaluator of {self.nvec}")
        guesses = []
        for q, (r1, r2) in enumerate(vecs):
            hr1 = np.multiply(self.h, r1, dtype=np.float64, order="F")
            hr2 = np.multiply(self.h, r2, dtype=np.float64, order="F")
            hr1x2, hr2x2 = hr1 + hr1, hr2 + hr2                         # (2 h) r, exactly
            points = ((self.t1 + hr1, self.t2 + hr2), (self.t1 - hr1, self.t2 - hr2),
                      (self.t1 + hr1x2, self.t2 + hr2x2), (self.t1 - hr1x2, self.t2 - hr2x2))
            for m, (x1, x2) in enumerate(points):
                k = 4 * q + m
                xb = self._basis_of(self.signs[k], x1, x2)
                self.cc.set_guess(k, *xb)
                guesses.append(xb)
        for k in range(4 * len(vecs), 4 * self.nvec):      # idle copies restart from t every call
            self.cc.set_guess(k, *self._t_in[self.signs[k]])
        self.cc.iterationCC(1, self.eps)
        self.calls += 1
        out = []
        for q in range(len(vecs)):
            om = []
            for m in range(4):
                k = 4 * q + m
                a1, a2 = self.cc.amplitudes(k)
                a1 -= guesses[k][0]
                a1 *= self.DS1[k]
                a2 -= guesses[k][1]
                a2 *= self.DS2[k]
                a2 /= 3.0
                om.append((a1, a2))
            res = []
            for p in range(2):
                d, e = om[0][p], om[2][p]
                d -= om[1][p]
                d *= 8.0
                e -= om[3][p]
                d -= e
                d /= 12.0 * self.h
                res.append(d)
            # row-major like the caller's vectors: numpy products of arrays in different
            # layouts run strided (the solvers' dot products took twice as long)
            out.append((np.ascontiguousarray(res[0]), pair_symmetric(np.ascontiguousarray(res[1]))))
        return out

    def close(self):
        self.cc.finalizeCC()


# ---------------------------------------------------------------- the iteration

class _Rules:
    """Stop rules of the generic iterator (gIterator.f90:88-210), the iteration block's settings."""

    def __init__(self, kw: api.Keywords, maxiter, eps):
        self.kw, self.maxiter, self.eps = kw, maxiter, eps
        self.iteration, self.successful, self.current = 0, 1, 0.0

    def update(self, acc):
        self.iteration += 1
        previous, self.current = self.current, acc
        if self.current < previous:
            self.successful += 1
        if self.current < self.eps:
            return STATUS_CONVERGED
        if not np.isfinite(self.current) or (self.kw.enable_divergence_check
                                             and self.current > 10.0 ** self.kw.divergence_threshold):
            return STATUS_DIVERGED
        if self.iteration + 1 > self.maxiter:
            return STATUS_MAXITER
        if (self.kw.enable_stagnation_check and self.iteration > self.kw.stagnation_check_after
                and 100.0 * self.successful / self.iteration <= self.kw.stagnation_threshold):
            return STATUS_STAGNATED
        return None


class _Diis:
    """pushLRVectors / newLRVectors / diisDotProduct on spin-adapted vectors."""

    def __init__(self, nd):
        self.nd, self.st, self.sd = nd, [], []
        self.B = np.zeros((nd + 1, nd + 1))

    def push(self, r, d):
        self.st.insert(0, (r[0].copy(), r[1].copy()))
        self.sd.insert(0, (d[0].copy(), d[1].copy()))
        del self.st[self.nd:], self.sd[self.nd:]

    def extrapolate(self, iteration, r):
        n = min(iteration, self.nd)
        B = self.B
        B[1:n, 1:n] = B[0:n - 1, 0:n - 1].copy()
        for k in range(n):
            B[k, 0] = B[0, k] = inner(self.sd[k], self.sd[0])
        if n == 1:
            return r
        A = np.ones((n + 1, n + 1)); A[:n, :n] = B[:n, :n]; A[n, n] = 0.0
        lam, U = np.linalg.eigh(A)
        c = (U[:n, :] * U[n, :][None, :] / lam[None, :]).sum(axis=1)
        return (sum(c[k] * self.st[k][0] for k in range(n)), sum(c[k] * self.st[k][1] for k in range(n)))


class _State:
    def __init__(self, r, kw, lr, eps):
        self.r = r
        self.rules = _Rules(kw, lr.max_iterations, eps)
        self.diis = _Diis(lr.diis_steps) if lr.diis_enabled else None
        self.status, self.omega = None, 0.0


def iterate_states(sigma, seeds, kw: api.Keywords, lr: LRKeywords, held=()):
    """Run the reference's iteration for every seed vector together; returns the finished states.

    ``sigma`` maps a list of vectors to their J r (one call per iteration);
    ``held`` are (r1, r2) of states found before (for orthogonalization).
    """
    base = 10.0 ** (-lr.accuracy)
    first = len(held)
    states = [_State(r, kw, lr, base * 2.0 ** (first + k)) for k, r in enumerate(seeds)]
    held = list(held)
    while any(s.status is None for s in states):
        live = [s for s in states if s.status is None]
        for s, d in zip(live, sigma([s.r for s in live])):
            r = s.r
            # stepLR
            s.omega = inner(d, r) / inner(r, r)
            d = (d[0] - s.omega * r[0], d[1] - s.omega * r[1])
            r = (r[0] - lr.r1_step * d[0], r[1] - lr.r2_step * d[1])
            acc = max_abs(d)
            scale = 1.0 / np.sqrt(inner(r, r))
            r = (r[0] * scale, pair_symmetric(r[1]) * scale)
            if lr.orthogonalization and held:
                ov = [inner_full(r, h) for h in held]
                r = (r[0] - sum(c * h[0] for c, h in zip(ov, held)), r[1] - sum(c * h[1] for c, h in zip(ov, held)))
            if max(acc) >= s.rules.eps and s.diis is not None:
                s.diis.push(r, d)
                r = s.diis.extrapolate(s.rules.iteration + 1, r)
            s.r = r
            s.status = s.rules.update(max(acc))
    return states


class _Basis:
    """Davidson basis vectors V and their sigma vectors W stacked as rows of
    contiguous arrays, so that projections, the projected matrix and Ritz
    vectors are matrix products. The doubles of V are also kept with the
    metric applied, G = 2 V2 - V2^ab (a and b swapped): inner(x, y) =
    2 x1.y1 + (2 x2 - x2^ab).y2, so a projection is one product per part."""

    def __init__(self, o, v, cap):
        self.o, self.v, self.cap, self.m = o, v, cap, 0
        n1, n2 = o * v, o * o * v * v
        self.V1, self.V2, self.G2 = np.empty((cap, n1)), np.empty((cap, n2)), np.empty((cap, n2))
        self.W1, self.W2 = np.empty((cap, n1)), np.empty((cap, n2))

    def vec(self, j):
        o, v = self.o, self.v
        return self.V1[j].reshape(o, v), self.V2[j].reshape(o, o, v, v)

    def coeffs(self, x):
        """inner(V_j, x) for every basis vector."""
        m = self.m
        return 2.0 * (self.V1[:m] @ x[0].reshape(-1)) + self.G2[:m] @ x[1].reshape(-1)

    def orthonormal(self, x):
        """x orthonormalised against the basis in ``inner`` (twice, as classical Gram-Schmidt
        needs), or None when nothing of it is left."""
        n0 = np.sqrt(max(inner(x, x), 0.0))
        if n0 == 0.0:
            return None
        x1, x2 = np.array(x[0], dtype=np.float64) / n0, np.array(x[1], dtype=np.float64) / n0
        for _ in range(2):
            if self.m:
                c = self.coeffs((x1, x2))
                x1 -= (c @ self.V1[:self.m]).reshape(x1.shape)
                x2 -= (c @ self.V2[:self.m]).reshape(x2.shape)
        n = np.sqrt(max(inner((x1, x2), (x1, x2)), 0.0))
        return None if n < 1e-10 else (x1 / n, x2 / n)

    def add(self, y):
        j = self.m
        self.V1[j], self.V2[j] = y[0].reshape(-1), y[1].reshape(-1)
        self.G2[j] = (2.0 * y[1] - swap_ab(y[1])).reshape(-1)
        self.m += 1
        return j

    def set_sigma(self, j, w):
        self.W1[j], self.W2[j] = w[0].reshape(-1), w[1].reshape(-1)

    def projected(self, rows, cols):
        """inner(V_i, W_j) for i in rows, j in cols."""
        return 2.0 * (self.V1[rows] @ self.W1[cols].T) + self.G2[rows] @ self.W2[cols].T


def davidson_states(sigma, seeds, nroots, F, kw: api.Keywords, lr: LRKeywords, track=None, max_space=None):
    """The lowest ``nroots`` roots of J by block Davidson (not the reference's iteration).

    The basis starts from ``seeds`` (more of them than roots, so that every
    symmetry of the low roots is present) and stays orthonormal in ``inner``.
    The lowest ``track`` Ritz pairs of the projected matrix (more than
    ``nroots``: a state dominated by doubles starts high in a basis of CIS
    vectors and has to be followed down) are refined with the residual divided
    by (theta - orbital energy differences) until max|residual| of root k is
    below accuracy * 2^k (the reference's per-state targets; the extra roots
    take the last one). Each iteration evaluates the new basis vectors in one
    ``sigma`` call. Deterministic: it converges to the lowest roots of the
    symmetries the seeds span, whatever the rounding of the sigma vectors.
    """
    k = min(track or nroots + 4, len(seeds))
    o, v = seeds[0][0].shape
    e = np.diag(F)
    eo, ev = e[:o], e[o:]
    D1 = ev[None, :] - eo[:, None]
    D2 = (ev[None, None, :, None] + ev[None, None, None, :] - eo[:, None, None, None] - eo[None, :, None, None])
    max_space = max_space or max(8 * k, 2 * len(seeds), 16)
    targets = [10.0 ** (-lr.accuracy) * 2.0 ** min(q, nroots - 1) for q in range(k)]
    B = _Basis(o, v, max_space + len(seeds) + k)

    def extend(vectors):
        new = []
        for x in vectors:
            y = B.orthonormal(x)
            if y is not None:
                new.append(B.add(y))
        for lo in range(0, len(new), sigma.nvec):
            block = new[lo:lo + sigma.nvec]
            for j, w in zip(block, sigma([B.vec(j) for j in block])):
                B.set_sigma(j, w)
        return len(new)

    extend(list(seeds))
    states = [_State(None, kw, lr, t) for t in targets]
    iteration = 0
    H = np.zeros((0, 0))
    while True:
        iteration += 1
        m, m0 = B.m, H.shape[0]
        Hn = np.zeros((m, m))                          # projected matrix, new rows and columns only
        Hn[:m0, :m0] = H
        if m > m0:
            Hn[m0:, :] = B.projected(slice(m0, m), slice(0, m))
            Hn[:m0, m0:] = B.projected(slice(0, m0), slice(m0, m))
        H = Hn
        theta, Y = np.linalg.eig(H)
        order = np.argsort(theta.real)[:k]
        Yk = np.ascontiguousarray(Y[:, order].real.T)  # k x m
        # unit Ritz vectors: the basis is orthonormal in inner, so inner(x, x) = |y|^2
        Yk /= np.linalg.norm(Yk, axis=1)[:, None]
        X1, X2 = Yk @ B.V1[:m], Yk @ B.V2[:m]
        S1, S2 = Yk @ B.W1[:m], Yk @ B.W2[:m]
        ritz = []
        for q, idx in enumerate(order):
            x = (X1[q].reshape(o, v), X2[q].reshape(o, o, v, v))
            s = (S1[q].reshape(o, v), S2[q].reshape(o, o, v, v))
            w = float(theta[idx].real)
            res = (s[0] - w * x[0], s[1] - w * x[1])
            ritz.append((w, x, s, res, max(max_abs(res))))
        for st, (w, x, _, _, acc) in zip(states, ritz):
            st.omega, st.r = w, x
            st.rules.iteration = iteration
            st.status = STATUS_CONVERGED if acc < st.rules.eps else None
        if all(st.status == STATUS_CONVERGED for st in states):
            return states[:nroots]
        if iteration >= lr.max_iterations:
            for st in states:
                st.status = st.status or STATUS_MAXITER
            return states[:nroots]
        corr = []
        for st, (w, x, s, res, acc) in zip(states, ritz):
            if st.status is None:
                d1, d2 = w - D1, w - D2
                d1 = np.where(np.abs(d1) < 1e-3, 1e-3, d1)
                d2 = np.where(np.abs(d2) < 1e-3, 1e-3, d2)
                corr.append((res[0] / d1, pair_symmetric(res[1] / d2)))
        if B.m + len(corr) > max_space:                # restart on the Ritz vectors
            B.m = 0
            H = np.zeros((0, 0))
            extend([x for (w, x, s, res, acc) in ritz])
        if extend(corr) == 0:
            for st in states:
                st.status = st.status or STATUS_STAGNATED
            return states[:nroots]


def linear_response(mol: Molecule, keywords: api.Keywords | None = None, lr: LRKeywords | None = None,
                    seeds=None, seed_orbitals=None, engine=None, solver: str = "reference") -> dict:
    """getEnergy('r-ccsd') with excited states: the r-ccsd ground state, then lr-r-ccsd.

    Returns energy (E_CCSD), ccsd status/iterations, the ground state's t1, t2
    and scf (orbitals C, MO Fock F), and per state (sorted by omega, as
    resortStates): omega, E_total = E_CCSD + omega, r0, ael (average
    excitation level), status, iterations, r1, r2 (in the orbitals C).
    ``seeds`` replaces the CIS guess by earlier states (loadSolution): a list
    of (r1, r2), in the orbitals ``seed_orbitals`` when given (their signs are
    matched to this run's orbitals).

    ``solver`` "reference" runs the reference's iteration. Which eigenpair
    each of its states settles on depends on rounding: the damped step with
    DIIS amplifies the components of lower states that rounding puts into a
    vector of another symmetry, so two runs whose sigma vectors differ in the
    last bits can end on different states (the reference's own OpenMP
    reductions differ from run to run in the same way). Every state it returns
    is an eigenpair of the problem. ``solver`` "davidson" returns the lowest
    roots instead (``davidson_states``), reproducibly.
    """
    kw = keywords or api.Keywords()
    lr = lr or LRKeywords()
    nstates = lr.excited_states_number
    if not 1 <= nstates <= 3:
        raise ValueError("states:excited-states-number must be 1..3 for an LR run")
    if lr.spin != 0:
        raise NotImplementedError("states:spin = 1 (triplets) is not provided: the engine's residual is spin-adapted")
    factory = engine or api.CoupledCluster
    c0 = factory(mol, kw)
    c0.initCC()
    gs = c0.iterate()
    t1, t2 = c0.amplitudes(0)
    scf = c0.scf(0)
    c0.finalizeCC()
    out = {"energy": float(gs["energy"][0]), "ccsd_status": int(gs["status"]),
           "ccsd_iterations": int(gs["iterations"]), "ccsd_energy": np.array(gs["energy"]),
           "t1": t1, "t2": t2, "scf": scf}
    if gs["status"] != STATUS_CONVERGED:
        raise RuntimeError(f"r-ccsd did not converge (status {gs['status']}): no LR run")
    o = t1.shape[0]
    C, F = scf["C"], scf["F"]
    I = MOIntegrals(C, coulomb_matrix(mol, kw.coulomb_integrals), o)
    v = t1.shape[1]
    davidson_seeds = None
    if seeds is None:
        sel, _ = guess_vectors(F, I, nstates, lr.guess, lr.guess_threshold)
        seeds = [seed_vector(s, o, v) for s in sel]
        if solver == "davidson":
            davidson_seeds = guess_space(F, I, min(o * v, max(2 * nstates, nstates + 4)))
    seeds = list(seeds)[:nstates]
    if seed_orbitals is not None:
        sg = _align(C, seed_orbitals)
        so, sv = sg[:o], sg[o:]
        seeds = [(a1 * so[:, None] * sv[None, :],
                  a2 * so[:, None, None, None] * so[None, :, None, None] * sv[None, None, :, None]
                  * sv[None, None, None, :]) for a1, a2 in seeds]
    if any(inner(s, s) == 0.0 for s in seeds):
        raise ValueError("a guess vector is empty (no singles reach linear-response:guess-threshold)")
    if solver not in ("reference", "davidson"):
        raise ValueError(f"solver {solver!r}: 'reference' or 'davidson'")
    sequential = lr.orthogonalization and solver == "reference"
    nvec = 1 if sequential else nstates
    if solver == "davidson":
        nvec = min(nstates + 4, len(davidson_seeds or seeds))
    sig = DeviceSigma(mol, kw, t1, t2, C, nvec=nvec, engine=engine)
    try:
        if solver == "davidson":
            states = davidson_states(sig, davidson_seeds or seeds, nstates, F, kw, lr, track=nvec)
        elif sequential:
            states = []
            for r in seeds:
                states += iterate_states(sig, [r], kw, lr, held=[s.r for s in states])
        else:
            states = iterate_states(sig, seeds, kw, lr)
    finally:
        sig.close()
    out["sigma_calls"] = sig.calls
    out["engine_copies"] = 4 * sig.nvec
    Ft = F[:o, o:] + np.einsum("iakd,kd->ia", I.L, t1)
    rows = []
    for s in states:
        r1, r2 = s.r
        s1 = 2.0 * float((r1 * r1).sum())
        s2 = inner((0 * r1, r2), (0 * r1, r2))
        r0 = (2.0 * float((Ft * r1).sum()) + float(np.einsum("iajb,ijab->", I.L, r2))) / s.omega
        rows.append({"omega": s.omega, "r0": r0, "ael": (s1 + 2 * s2) / (s1 + s2), "status": s.status,
                     "iterations": s.rules.iteration, "r1": r1, "r2": r2})
    rows.sort(key=lambda x: x["omega"])
    for key in ("omega", "r0", "ael", "status", "iterations"):
        out[key] = np.array([x[key] for x in rows])
    out["E_total"] = out["energy"] + out["omega"]
    out["r1"] = [x["r1"] for x in rows]
    out["r2"] = [x["r2"] for x in rows]
    return out


def stored_seeds(result: dict, lr: LRKeywords | None = None):
    """dumpSolution / loadSolution (:593-734): the states' amplitudes above the store threshold
    (in the spin-adapted coordinates), by store-solution-mode, as seeds for the next run."""
    lr = lr or LRKeywords()
    thr = 10.0 ** (-lr.store_solution_threshold)
    seeds = []
    for r1, r2 in zip(result["r1"], result["r2"]):
        a1 = np.where(np.abs(r1) > thr, r1, 0.0) if "r1" in lr.store_solution_mode else 0 * r1
        a2 = np.where(np.abs(r2) > thr, r2, 0.0) if lr.store_solution_mode in ("r2", "r1r2") else 0 * r2
        seeds.append((a1, a2))
    return seeds
