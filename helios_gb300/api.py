"""Python front end of the GB300 CCSD engine, shaped like helios's CC interface.

The reference drives r-ccsd through module routines
(src/methods/coupledCluster/mod_cc.f90): ``setCCParameters``, ``initCC``,
``iterationCC(iteration, epsilon, accuracy)``, ``energyCC(energy)`` and
``finalizeCC``, looped by ``iterator`` (src/calculation/gIterator.f90). The
``CoupledCluster`` class exposes the same routines, with the same argument
meaning and 5-element accuracy/energy vectors, over the C ABI of
``include/helios_cc.h`` (``libhelios_gb300.so``). ``get_energy`` mirrors
``getEnergy('r-ccsd')`` (src/modules/mod_property.f90:55-338).

There is no CPU path: every call runs the CUDA engine, and importing the
module fails if the library has not been built.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field as dc_field

import numpy as np

from .molecules import Molecule

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libhelios_gb300.so")

STATUS = {1: "converged", -1: "failed", -2: "diverged", -3: "stagnated", -4: "interrupted"}
COULOMB = {"ohno-klopman": 0, "mataga-nishimoto": 1, "hubbard": 2}

_c_d = ctypes.POINTER(ctypes.c_double)
_c_i = ctypes.POINTER(ctypes.c_int32)
_c_f = ctypes.POINTER(ctypes.c_float)
_c_l = ctypes.POINTER(ctypes.c_int64)


class PPPModel(ctypes.Structure):
    _fields_ = [("n_sites", ctypes.c_int32), ("coords", _c_d), ("alpha", _c_d), ("gamma", _c_d),
                ("nels", _c_i), ("n_bonds", ctypes.c_int32), ("bond_i", _c_i), ("bond_j", _c_i),
                ("beta", _c_d), ("bond_kind", _c_i)]


class CCParams(ctypes.Structure):
    _fields_ = [("coulomb", ctypes.c_int32), ("bond_alternation", ctypes.c_double),
                ("field", ctypes.c_double * 3), ("scf_maxiter", ctypes.c_int32), ("scf_eps", ctypes.c_double),
                ("scf_step", ctypes.c_double), ("projection_type", ctypes.c_int32),
                ("cc_maxiter", ctypes.c_int32), ("cc_eps", ctypes.c_double), ("t1_step", ctypes.c_double),
                ("t2_step", ctypes.c_double), ("diis_enabled", ctypes.c_int32), ("diis_steps", ctypes.c_int32),
                ("check_divergence", ctypes.c_int32), ("divergence_threshold", ctypes.c_double),
                ("check_stagnation", ctypes.c_int32), ("stagnation_threshold", ctypes.c_double),
                ("stagnation_after", ctypes.c_int32), ("precision", ctypes.c_int32), ("guess", ctypes.c_int32),
                ("mixed_switch", ctypes.c_double), ("mixed_patience", ctypes.c_int32),
                ("mixed_check", ctypes.c_int32), ("tile_tuning", ctypes.c_int32), ("tile_force", ctypes.c_int32)]


class HxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"helios_gb300 error {code}: {msg}")
        self.code = code


_lib = None


def library():
    """Load libhelios_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python -m helios_gb300.build` "
                              "(the engine has no CPU fallback)")
        lib = ctypes.CDLL(LIB_PATH)
        lib.hx_cc_params_default.restype = None
        lib.hx_ccsd_cancel.restype = None
        lib.hx_ccsd_destroy.restype = None
        for name in ("hx_ccsd_create", "hx_ccsd_create_batch", "hx_ccsd_init", "hx_ccsd_set_guess",
                     "hx_ccsd_iterate", "hx_ccsd_energy", "hx_ccsd_solve", "hx_ccsd_solve_batch",
                     "hx_ccsd_get_amplitudes", "hx_ccsd_get_scf", "hx_ccsd_dims", "hx_ccsd_trace",
                     "hx_gemm", "hx_gemm_tile", "hx_ccsd_timing", "hx_last_error", "hx_ccsd_set_model", "hx_ccsd_training_rows",
                     "hx_mlp_nparam", "hx_mlp_predict", "hx_mlp_grad", "hx_mlp_train", "hx_ccsd_triples",
                     "hx_tile_table", "hx_tile_table_load", "hx_tile_variants", "hx_ccsd_tile_choices"):
            getattr(lib, name).restype = ctypes.c_int
        _lib = lib
        if os.path.exists(TILE_TABLE_PATH):
            load_tile_table(read_tile_table(TILE_TABLE_PATH))
    return _lib


# ---------------------------------------------------------------- tile autotuner
TILE_TABLE_PATH = os.path.join(_HERE, "data", "tile_table.json")
TILE_TUNING = {"table": 0, "tune": 1, "default": 2}


def tile_variants(mode: int):
    """Output tile widths of the candidates of a precision mode (0..3: 3, 4, 5, 7 slices);
    candidates of equal width differ in their pipeline depth."""
    bn = (ctypes.c_int32 * 8)()
    n = _check(library().hx_tile_variants(int(mode), bn, 8))
    return [int(bn[k]) for k in range(n)]


def tile_table():
    """The process-wide tile table: list of (mode, group, size class N, size class work, variant)."""
    n = _check(library().hx_tile_table(None, 0))
    buf = (ctypes.c_int32 * max(5 * n, 1))()
    _check(library().hx_tile_table(buf, n))
    return [tuple(int(buf[5 * k + c]) for c in range(5)) for k in range(n)]


def load_tile_table(entries):
    """Merge entries (mode, group, size class N, size class work, variant) into the tile table."""
    flat = np.ascontiguousarray(np.asarray(entries, dtype=np.int32).reshape(-1, 5))
    _check(library().hx_tile_table_load(flat.ctypes.data_as(_c_i), int(flat.shape[0])))


def read_tile_table(path):
    import json
    with open(path) as f:
        d = json.load(f)
    return [tuple(int(x) for x in e) for e in d["entries"]]


def write_tile_table(path, entries, note=""):
    import json
    entries = sorted(tuple(int(x) for x in e) for e in entries)
    head = json.dumps({"format": "mode, plan group, ceil log2 of the widest N, floor log2 of the multiply-adds, variant",
                       "note": note})
    with open(path, "w") as f:       # one entry per line
        f.write(head[:-1] + ', "entries": [\n' + ",\n".join(json.dumps(list(e)) for e in entries) + "\n]}\n")


def gemm(A, B, precision="fp64", reps=1, variant=-1):
    """C = A @ B.T on the engine's FP64 ("fp64") or tensor-core GEMM ("mixed": 3 slices,
    "mid": 4 slices, "high": 5 slices, "exact": 7 slices, FP64 emulated), on tile candidate
    `variant` of the mode (-1: the default); returns (C, ms per launch)."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    M, K = A.shape
    N = B.shape[0]
    C = np.zeros((M, N))
    ms = ctypes.c_double()
    _check(library().hx_gemm_tile(A.ctypes.data_as(_c_d), B.ctypes.data_as(_c_d), C.ctypes.data_as(_c_d), M, N, K,
                                  {"fp64": 0, "mixed": 1, "high": 2, "mid": 3, "exact": 4}[precision], int(variant),
                                  reps, ctypes.byref(ms)))
    return C, ms.value


def mlp_nparam() -> int:
    return library().hx_mlp_nparam()


def mlp_predict(params, X):
    """Learned-guess network on input rows X [n, 8] (tcgen05 inference kernel)."""
    P = np.ascontiguousarray(params, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.float32)
    Y = np.zeros(X.shape[0], dtype=np.float32)
    _check(library().hx_mlp_predict(P.ctypes.data_as(_c_f), X.ctypes.data_as(_c_f), ctypes.c_int64(X.shape[0]),
                                    Y.ctypes.data_as(_c_f)))
    return Y


def mlp_grad(params, X, T):
    """(loss, gradient blob) of the mean-squared error on rows X, T (GPU training kernels)."""
    P = np.ascontiguousarray(params, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.float32)
    T = np.ascontiguousarray(T, dtype=np.float32)
    loss = ctypes.c_float()
    G = np.zeros_like(P)
    _check(library().hx_mlp_grad(P.ctypes.data_as(_c_f), X.ctypes.data_as(_c_f), T.ctypes.data_as(_c_f),
                                 X.shape[0], ctypes.byref(loss), G.ctypes.data_as(_c_f)))
    return float(loss.value), G


def mlp_train(params, X, T, epochs=10, batch=4096, lr=1e-3, seed=0):
    """Train on the GPU (Adam, cosine decay); returns (new params, per-epoch mean loss)."""
    P = np.array(params, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.float32)
    T = np.ascontiguousarray(T, dtype=np.float32)
    L = np.zeros(epochs, dtype=np.float32)
    _check(library().hx_mlp_train(P.ctypes.data_as(_c_f), X.ctypes.data_as(_c_f), T.ctypes.data_as(_c_f),
                                  ctypes.c_int64(X.shape[0]), epochs, batch, ctypes.c_float(lr),
                                  ctypes.c_uint64(seed), L.ctypes.data_as(_c_f)))
    return P, L


def last_error() -> str:
    buf = ctypes.create_string_buffer(1024)
    library().hx_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def _check(rc):
    if rc < 0:
        raise HxError(rc, last_error())
    return rc


@dataclass
class Keywords:
    """Input keywords of the path with helios's defaults (src/input/definebd.f90)."""
    coulomb_integrals: str = "ohno-klopman"      # parametrization:coulomb-integrals
    bond_alternation: float = 0.0                # parametrization:bond-alternation
    field: tuple = (0.0, 0.0, 0.0)               # field:along-x/y/z (eV per Angstrom)
    scf_max_iterations: int = 400                # scf:max-iterations
    scf_accuracy: float = 12                     # scf:accuracy (exponent, 10^-value)
    scf_iter_step: float = 0.05                  # scf:iter-step
    projection_type: str = "2-1"                 # coupled-cluster:projection-type
    max_iterations: int = 2000                   # coupled-cluster:max-iterations
    accuracy: float = 12                         # coupled-cluster:accuracy (exponent)
    t1_step: float = 1.0                         # coupled-cluster:t1-step
    t2_step: float = 1.0                         # coupled-cluster:t2-step
    diis_enabled: bool = True                    # coupled-cluster:diis-enabled
    diis_steps: int = 20                         # coupled-cluster:diis-steps
    enable_divergence_check: bool = True         # iteration:enable-divergence-check
    divergence_threshold: float = 3              # iteration:divergence-threshold (exponent, 10^value)
    enable_stagnation_check: bool = True         # iteration:enable-stagnation-check
    stagnation_threshold: float = 60.0           # iteration:stagnation-threshold
    stagnation_check_after: int = 200            # iteration:stagnation-check-after
    precision: str = "fp64"                      # engine: "fp64", "mixed" or "exact" (7-slice emulated FP64 throughout)
    guess: str = "reference"                     # engine: "reference" (guessCC) or "learned"
    model: object = None                         # engine: learned-guess parameters (None = the shipped model)
    mixed_switch: float = 1e-3                   # engine: residual where 3-slice hands over to 4-slice
    mixed_patience: int = 3                      # engine: non-improving iterations before the next phase
    mixed_check: str = "emulated"                # engine: convergence checks on "emulated" (7-slice) or "fp64"
    tile_tuning: str = "table"                   # engine: tensor-core tile shapes "table", "tune" or "default"
    tile_force: int = -1                         # engine: >= 0 forces one tile candidate in every mode

    def to_c(self) -> CCParams:
        p = CCParams()
        library().hx_cc_params_default(ctypes.byref(p))
        p.coulomb = COULOMB[self.coulomb_integrals]
        p.bond_alternation = self.bond_alternation
        for k in range(3):
            p.field[k] = float(self.field[k])
        p.scf_maxiter = self.scf_max_iterations
        p.scf_eps = 10.0 ** (-self.scf_accuracy)
        p.scf_step = self.scf_iter_step
        p.projection_type = {"1": 1, "2-1": 2}[self.projection_type]
        p.cc_maxiter = self.max_iterations
        p.cc_eps = 10.0 ** (-self.accuracy)
        p.t1_step, p.t2_step = self.t1_step, self.t2_step
        p.diis_enabled = int(self.diis_enabled)
        p.diis_steps = self.diis_steps
        p.check_divergence = int(self.enable_divergence_check)
        p.divergence_threshold = 10.0 ** self.divergence_threshold
        p.check_stagnation = int(self.enable_stagnation_check)
        p.stagnation_threshold = self.stagnation_threshold
        p.stagnation_after = self.stagnation_check_after
        p.precision = {"fp64": 0, "mixed": 1, "exact": 2}[self.precision]
        p.guess = {"reference": 0, "learned": 1}[self.guess]
        p.mixed_switch = self.mixed_switch
        p.mixed_patience = self.mixed_patience
        p.mixed_check = {"emulated": 0, "fp64": 1}[self.mixed_check]
        p.tile_tuning = TILE_TUNING[self.tile_tuning]
        p.tile_force = int(self.tile_force)
        return p


class _ModelArrays:
    """Keeps the numpy buffers behind one PPPModel alive."""

    def __init__(self, mol: Molecule):
        self.coords = np.ascontiguousarray(mol.coords, dtype=np.float64)
        self.alpha = np.ascontiguousarray(mol.alpha, dtype=np.float64)
        self.gamma = np.ascontiguousarray(mol.gamma, dtype=np.float64)
        self.nels = np.ascontiguousarray(mol.nels, dtype=np.int32)
        bi, bj, beta, kind = mol.bond_arrays()
        self.bi, self.bj, self.beta, self.kind = (np.ascontiguousarray(x) for x in (bi, bj, beta, kind))
        self.c = PPPModel(mol.n_sites, self.coords.ctypes.data_as(_c_d), self.alpha.ctypes.data_as(_c_d),
                          self.gamma.ctypes.data_as(_c_d), self.nels.ctypes.data_as(_c_i), len(self.bi),
                          self.bi.ctypes.data_as(_c_i), self.bj.ctypes.data_as(_c_i),
                          self.beta.ctypes.data_as(_c_d), self.kind.ctypes.data_as(_c_i))


class CoupledCluster:
    """One engine handle (one molecule or a batch) with the reference's routine names."""

    def __init__(self, molecules, keywords: Keywords | None = None):
        self.keywords = keywords or Keywords()
        self.molecules = [molecules] if isinstance(molecules, Molecule) else list(molecules)
        self._h = ctypes.c_void_p()
        self.setCCParameters()

    # -- mod_cc.f90:82-485
    def setCCParameters(self):
        arrs = [_ModelArrays(m) for m in self.molecules]
        models = (PPPModel * len(arrs))(*[a.c for a in arrs])
        self._params = self.keywords.to_c()
        _check(library().hx_ccsd_create_batch(models, len(arrs), ctypes.byref(self._params), ctypes.byref(self._h)))
        if self.keywords.guess == "learned":
            self.set_model(self.keywords.model)
        self.dims = []
        for k in range(len(arrs)):
            d = (ctypes.c_int32 * 4)()
            _check(library().hx_ccsd_dims(self._h, k, d))
            self.dims.append(tuple(d))

    # -- mod_cc.f90:489-603
    def initCC(self):
        _check(library().hx_ccsd_init(self._h))

    # -- mod_cc.f90:820-891
    def iterationCC(self, iteration: int, epsilon: float) -> np.ndarray:
        acc = (ctypes.c_double * 5)()
        _check(library().hx_ccsd_iterate(self._h, iteration, ctypes.c_double(epsilon), acc))
        return np.array(acc)

    # -- mod_cc.f90:1916-1952
    def energyCC(self) -> np.ndarray:
        e = (ctypes.c_double * 5)()
        _check(library().hx_ccsd_energy(self._h, e))
        return np.array(e)

    # -- iterator(iterationCC, energyCC, ...) for molecule 0
    def iterate(self, maxiter=None, eps=None):
        maxiter = self.keywords.max_iterations if maxiter is None else maxiter
        eps = 10.0 ** (-self.keywords.accuracy) if eps is None else eps
        st, it = ctypes.c_int32(), ctypes.c_int32()
        e = (ctypes.c_double * 5)()
        _check(library().hx_ccsd_solve(self._h, maxiter, ctypes.c_double(eps), ctypes.byref(st), ctypes.byref(it), e))
        return {"status": st.value, "iterations": it.value, "energy": np.array(e)}

    def solve_batch(self):
        n = len(self.molecules)
        st = np.zeros(n, dtype=np.int32)
        it = np.zeros(n, dtype=np.int32)
        e = np.zeros((n, 5))
        _check(library().hx_ccsd_solve_batch(self._h, st.ctypes.data_as(_c_i), it.ctypes.data_as(_c_i),
                                             e.ctypes.data_as(_c_d)))
        return {"status": st, "iterations": it, "energy": e}

    def set_model(self, params=None):
        """Install the learned-guess network (a float32 blob; None = the shipped model)."""
        if params is None:
            from .learned import default_model
            params = default_model()
        blob = np.ascontiguousarray(params, dtype=np.float32)
        if blob.size != mlp_nparam():
            raise ValueError(f"model blob has {blob.size} values, expected {mlp_nparam()}")
        self._model = blob
        _check(library().hx_ccsd_set_model(self._h, blob.ctypes.data_as(_c_f)))

    def training_rows(self, mol: int, rows):
        """Inputs X [n, 8] and targets t2 - guess [n] of canonical pairs `rows` of molecule mol."""
        rows = np.ascontiguousarray(rows, dtype=np.int64)
        X = np.zeros((rows.size, 8), dtype=np.float32)
        T = np.zeros(rows.size, dtype=np.float32)
        _check(library().hx_ccsd_training_rows(self._h, int(mol), rows.size, rows.ctypes.data_as(_c_l),
                                               X.ctypes.data_as(_c_f), T.ctypes.data_as(_c_f)))
        return X, T

    def set_guess(self, mol: int, t1, t2):
        t1 = np.asfortranarray(t1, dtype=np.float64)
        t2 = np.asfortranarray(t2, dtype=np.float64)
        _check(library().hx_ccsd_set_guess(self._h, int(mol), t1.ctypes.data_as(_c_d), t2.ctypes.data_as(_c_d)))

    def amplitudes(self, mol: int = 0):
        """t1 (o, v) and t2 (o, o, v, v) as numpy arrays indexed like the reference."""
        N, o, v, _ = self.dims[mol]
        t1 = np.empty((o, v), order="F")                  # every element is written
        t2 = np.empty((o, o, v, v), order="F")
        _check(library().hx_ccsd_get_amplitudes(self._h, int(mol), t1.ctypes.data_as(_c_d), t2.ctypes.data_as(_c_d)))
        return t1, t2

    def scf(self, mol: int = 0):
        N = self.dims[mol][0]
        C = np.zeros((N, N)); eps = np.zeros(N); fmo = np.zeros((N, N)); out = np.zeros(4)
        st = np.zeros(2, dtype=np.int32)
        _check(library().hx_ccsd_get_scf(self._h, int(mol), C.ctypes.data_as(_c_d), eps.ctypes.data_as(_c_d),
                                         fmo.ctypes.data_as(_c_d), out.ctypes.data_as(_c_d), st.ctypes.data_as(_c_i)))
        return {"C": C, "eps": eps, "F": fmo, "energy": out[0], "eel": out[1], "enuc": out[2],
                "accuracy": out[3], "status": int(st[0]), "iterations": int(st[1])}

    def triples(self, mol: int = 0) -> dict:
        """(T) of molecule mol after a solve: textbook (T) = E[4] + E[5], its parts, and the
        reference's r-ccsd(t) triples term (= -(T), see hx_ccsd_triples)."""
        e = np.zeros(4)
        _check(library().hx_ccsd_triples(self._h, int(mol), e.ctypes.data_as(_c_d)))
        return {"T": e[0], "E4": e[1], "E5": e[2], "reference_term": e[3]}

    def trace(self, mol: int = 0) -> np.ndarray:
        """Per-iteration (max|d1|, max|d2|, E_total, seconds, phase) of the last solve;
        phase 4, 3, 2 = 3-, 4-, 5-slice tensor cores, 1 = 7-slice (FP64 emulated), 0 = FP64."""
        n = _check(library().hx_ccsd_trace(self._h, int(mol), None, 0))
        out = np.zeros((max(n, 1), 5))
        library().hx_ccsd_trace(self._h, int(mol), out.ctypes.data_as(_c_d), n)
        return out[:n]

    def timing(self, profile: int = -1) -> dict:
        """Device timing of the last init/solve and the tcgen05 GEMM totals (see hx_ccsd_timing)."""
        out = np.zeros(8)
        _check(library().hx_ccsd_timing(self._h, out.ctypes.data_as(_c_d), profile))
        return {"init_ms": out[0], "solve_ms": out[1], "gemm_launches": int(out[2]), "gemm_ms": out[3],
                "gemm_flops": out[4], "gemm_hw_flops": out[5], "device_bytes": int(out[6]),
                "kernel_launches": int(out[7])}

    def tile_choices(self):
        """(variants [4, groups] of a mixed handle, milliseconds spent tuning at creation)."""
        ms = ctypes.c_double()
        n = _check(library().hx_ccsd_tile_choices(self._h, None, 0, ctypes.byref(ms)))
        buf = (ctypes.c_int32 * max(n, 1))()
        _check(library().hx_ccsd_tile_choices(self._h, buf, n, ctypes.byref(ms)))
        return np.array([buf[k] for k in range(n)], dtype=np.int32).reshape(4, -1) if n else np.zeros((4, 0), np.int32), ms.value

    def cancel(self):
        library().hx_ccsd_cancel(self._h)

    # -- mod_cc.f90 finalizeCC
    def finalizeCC(self):
        if self._h:
            library().hx_ccsd_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.finalizeCC()
        except Exception:
            pass


def get_energy(molecule: Molecule, keywords: Keywords | None = None):
    """getEnergy('r-ccsd'): SCF + CCSD for one molecule; returns the result dict."""
    cc = CoupledCluster(molecule, keywords)
    cc.initCC()
    out = cc.iterate()
    out["scf"] = cc.scf(0)
    out["ecorr"] = out["energy"][0] - out["energy"][1]
    cc.finalizeCC()
    return out
