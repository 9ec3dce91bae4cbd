"""ORACLE (test infrastructure only) -- ctypes front end of the literal C restatement.

``solve_literal`` runs the whole reference chain for one molecule:
PPP model -> RHF (``oracle.rhf``) -> MO Fock + reference energy
(``prepareFock``/``referenceEnergy``, mod_cc.f90:2336-2396,2474-2504) -> full
N^4 integrals ``R`` (mod_cc.f90:547-557) -> guess (mod_cc.f90:634-650) ->
``orc_ccsd_solve`` (iterationCC + energyCC under the gIterator rules).
Feasible up to N ~ 16 (the doubles residual is o^4 v^4 per iteration).
"""
from __future__ import annotations

import ctypes
import numpy as np

from . import build as _build
from .ppp import build_model
from .rhf import rhf, mo_fock

_lib = None
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(_build.build())
        for name in ("orc_integrals", "orc_guess", "orc_singles", "orc_doubles", "orc_step",
                     "orc_energy", "orc_doubles_sample"):
            getattr(_lib, name).restype = None
        _lib.orc_ccsd_solve.restype = ctypes.c_int
        _lib.orc_num_threads.restype = ctypes.c_int
    return _lib


def _p(a):
    return a.ctypes.data_as(_dp)


def c64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def integrals(C, G):
    """Full R[p,q,r,s] = 2(pq|rs) - (ps|rq) (N^4, FP64). C[mu, p] = MO p on site mu."""
    N = C.shape[0]
    R = np.zeros((N, N, N, N))
    lib().orc_integrals(N, _p(c64(C)), _p(c64(G)), _p(R))
    return R


def guess(F, R, o):
    N = F.shape[0]
    v = N - o
    t1 = np.zeros((o, v)); t2 = np.zeros((o, o, v, v))
    lib().orc_guess(N, o, _p(c64(F)), _p(c64(R)), _p(t1), _p(t2))
    return t1, t2


def residuals(F, R, t1, t2):
    """Reference residuals d1 (o,v) and d2 (o,o,v,v) at amplitudes t1, t2."""
    N = F.shape[0]
    o, v = t1.shape
    d1 = np.zeros((o, v)); d2 = np.zeros((o, o, v, v))
    F, R, t1, t2 = c64(F), c64(R), c64(t1), c64(t2)
    lib().orc_singles(N, o, _p(F), _p(R), _p(t1), _p(t2), _p(d1))
    lib().orc_doubles(N, o, _p(F), _p(R), _p(t1), _p(t2), _p(d2))
    return d1, d2


def doubles_sample(F, R, t1, t2, mm, nn):
    """Reference doubles residual on the excitation pairs (mm[k], nn[k]) only."""
    N = F.shape[0]
    o = t1.shape[0]
    mm = np.ascontiguousarray(mm, dtype=np.int32)
    nn = np.ascontiguousarray(nn, dtype=np.int32)
    out = np.zeros(len(mm))
    F, R, t1, t2 = c64(F), c64(R), c64(t1), c64(t2)
    lib().orc_doubles_sample(N, o, _p(F), _p(R), _p(t1), _p(t2), mm.ctypes.data_as(_ip), nn.ctypes.data_as(_ip),
                             len(mm), _p(out))
    return out


def energy(F, R, t1, t2, eref):
    N = F.shape[0]
    o = t1.shape[0]
    e = np.zeros(5)
    lib().orc_energy(N, o, _p(c64(F)), _p(c64(R)), _p(c64(t1)), _p(c64(t2)), ctypes.c_double(eref), _p(e))
    return e


def ccsd(F, R, eref, o, t1=None, t2=None, eps=1e-12, maxiter=2000, diis=True, nd=20,
         step1=1.0, step2=1.0, projtype=2, diis_solver=0, trace_cap=4000):
    """orc_ccsd_solve: returns dict(energy[5], status, iterations, t1, t2, trace)."""
    N = F.shape[0]
    if t1 is None:
        t1, t2 = guess(F, R, o)
    t1 = c64(t1).copy(); t2 = c64(t2).copy()
    params = np.array([step1, step2, eps, 1e3, 60.0])
    iparams = np.array([maxiter, int(diis), nd, projtype, 200, 1, 1, diis_solver], dtype=np.int32)
    e = np.zeros(5)
    it = ctypes.c_int(0)
    trace = np.zeros(3 * trace_cap)
    status = lib().orc_ccsd_solve(N, o, _p(c64(F)), _p(c64(R)), ctypes.c_double(eref), _p(t1), _p(t2),
                                  _p(params), iparams.ctypes.data_as(_ip), _p(e), ctypes.byref(it),
                                  _p(trace), trace_cap)
    n = it.value
    return {"energy": e, "status": status, "iterations": n, "t1": t1, "t2": t2,
            "trace": trace[:3 * min(n, trace_cap)].reshape(-1, 3)}


def solve_literal(mol, alternation=0.1, coulomb="ohno-klopman", field=(0.0, 0.0, 0.0), eps=1e-12,
                  scf_eps=1e-12, **kw):
    """PPP -> RHF -> literal r-ccsd for one molecule. Returns a dict of results."""
    model = build_model(mol, coulomb=coulomb, alternation=alternation, field=field)
    scf = rhf(model, eps=scf_eps)
    F, eref = mo_fock(model, scf["V"], scf["D"])
    R = integrals(scf["V"], model["G"])
    o = model["nel"] // 2
    out = ccsd(F, R, eref, o, eps=eps, **kw)
    out.update({"model": model, "scf": scf, "F": F, "R": R, "eref": eref, "o": o,
                "ecorr": out["energy"][0] - eref})
    return out
