"""helios input files for the engine: the block parser, the molecule block and the job.

A helios input (src/input/parseInput.f90, mod_blockdata.f90:496-630) is a
set of blocks ``%name{ key = value, key = value ... }`` -- any number of
lines, ``#`` starts a comment, names and keys are case-insensitive -- plus
the free-form ``%molecule{ ... }`` block read by readMoleculeInformation.f90
(:20-106): the name, the numbers of atoms and bonds, the alpha and beta
electron counts, one line per atom ``symbol x y z alpha gamma n_pi`` and one
per bond ``i j beta kind`` (1-based sites, kind single / double / nonset).

``read_input`` returns the molecule, the engine keywords (the keys of
definebd.f90 that the r-ccsd path reads, with their defaults and their
power-of-ten ("potentiate") conventions) and the job (method, jobtype,
polarizability grid, harvest, and the ``states`` / ``linear-response`` keys
of an LR-CCSD run); ``write_input`` writes the same format; ``run_input``
runs an energy job of method r-ccsd (with its excited states when
``states:excited-states-number`` > 0, as getEnergy, mod_property.f90:159-175)
or r-ccsd(t), or a polarizability job of r-ccsd. Engine options the
reference has no key for (precision, guess, mixed_check, lr-solver) go in a
``%engine{ }`` block, which the reference's reader never looks for.
"""
from __future__ import annotations

import re
import sys
from dataclasses import dataclass, field

import numpy as np

from . import api
from .lrccsd import LRKeywords
from .molecules import Molecule

# keys of definebd.f90 that the path reads: (block, key) -> (Keywords field, kind, default)
# kind: "float", "int", "bool", "str", "pow-" (value v means 10^-v), "pow+" (10^+v)
_KEYS = {
    ("parametrization", "coulomb-integrals"): ("coulomb_integrals", "str", "ohno-klopman"),
    ("parametrization", "bond-alternation"): ("bond_alternation", "float", 0.0),
    ("scf", "max-iterations"): ("scf_max_iterations", "int", 400),
    ("scf", "accuracy"): ("scf_accuracy", "float", 12.0),
    ("scf", "iter-step"): ("scf_iter_step", "float", 0.05),
    ("coupled-cluster", "projection-type"): ("projection_type", "str", "2-1"),
    ("coupled-cluster", "max-iterations"): ("max_iterations", "int", 2000),
    ("coupled-cluster", "accuracy"): ("accuracy", "float", 12.0),
    ("coupled-cluster", "t1-step"): ("t1_step", "float", 1.0),
    ("coupled-cluster", "t2-step"): ("t2_step", "float", 1.0),
    ("coupled-cluster", "diis-enabled"): ("diis_enabled", "bool", True),
    ("coupled-cluster", "diis-steps"): ("diis_steps", "int", 20),
    ("iteration", "enable-divergence-check"): ("enable_divergence_check", "bool", True),
    ("iteration", "divergence-threshold"): ("divergence_threshold", "float", 3.0),
    ("iteration", "enable-stagnation-check"): ("enable_stagnation_check", "bool", True),
    ("iteration", "stagnation-threshold"): ("stagnation_threshold", "float", 60.0),
    ("iteration", "stagnation-check-after"): ("stagnation_check_after", "int", 200),
    ("engine", "precision"): ("precision", "str", "fp64"),
    ("engine", "guess"): ("guess", "str", "reference"),
    ("engine", "mixed-check"): ("mixed_check", "str", "emulated"),
}

# keys of the states and linear-response blocks (definebd.f90:71-72, 159-171) -> LRKeywords field
_LR_KEYS = {
    ("states", "excited-states-number"): ("excited_states_number", "int"),
    ("states", "spin"): ("spin", "int"),
    ("linear-response", "guess"): ("guess", "str"),
    ("linear-response", "guess-threshold"): ("guess_threshold", "float"),
    ("linear-response", "max-iterations"): ("max_iterations", "int"),
    ("linear-response", "accuracy"): ("accuracy", "float"),
    ("linear-response", "r1-step"): ("r1_step", "float"),
    ("linear-response", "r2-step"): ("r2_step", "float"),
    ("linear-response", "orthogonalization"): ("orthogonalization", "bool"),
    ("linear-response", "diis-enabled"): ("diis_enabled", "bool"),
    ("linear-response", "diis-steps"): ("diis_steps", "int"),
    ("linear-response", "store-solution"): ("store_solution", "bool"),
    ("linear-response", "store-solution-threshold"): ("store_solution_threshold", "float"),
    ("linear-response", "store-solution-mode"): ("store_solution_mode", "str"),
}


@dataclass
class Job:
    methods: list = field(default_factory=lambda: ["r-ccsd"])
    jobtype: str = "energy"
    components: str = "x"              # polariz:components
    points: int = 5                    # polariz:points
    derive_step: float = 0.02          # polariz:derive-step (V/Angstrom)
    harvest: bool = False              # system:harvest
    output_file: str = "%input%"       # general:output-file
    symbols: list = field(default_factory=list)
    lr: LRKeywords = field(default_factory=lambda: LRKeywords(excited_states_number=0))  # states, linear-response
    lr_solver: str = "reference"       # engine:lr-solver ("reference" iteration or "davidson")


def strip_comments(text: str) -> str:
    return "\n".join(line.split("#", 1)[0] for line in text.splitlines())


def parse_blocks(text: str) -> tuple[dict, list]:
    """Keyed blocks {name: {key: value}} and the molecule block's lines."""
    body = strip_comments(text)
    blocks, mol_lines = {}, None
    for m in re.finditer(r"%([A-Za-z][\w-]*)\s*\{(.*?)\}", body, flags=re.S):
        name, content = m.group(1).lower(), m.group(2)
        if name == "molecule":
            mol_lines = [ln.strip() for ln in content.splitlines() if ln.strip()]
            continue
        entries = {}
        for item in re.split(r"[,\n]", content):
            item = item.strip()
            if not item:
                continue
            if "=" not in item:
                raise ValueError(f"%{name}: expected key = value, got {item!r}")
            k, v = (s.strip() for s in item.split("=", 1))
            entries[k.lower()] = v
        blocks.setdefault(name, {}).update(entries)
    return blocks, mol_lines or []


def _value(kind: str, text: str):
    t = text.strip().strip("'\"")
    if kind == "bool":
        if t.lower() in ("true", ".true.", "t", "yes", "1"):
            return True
        if t.lower() in ("false", ".false.", "f", "no", "0"):
            return False
        raise ValueError(f"not a logical value: {text!r}")
    if kind == "int":
        return int(float(t))
    if kind == "float":
        return float(t)
    return t.lower()


def parse_molecule(lines: list[str]) -> tuple[Molecule, list]:
    """readMoleculeInformation: the molecule and its atom symbols."""
    if len(lines) < 5:
        raise ValueError("the molecule block needs name, atoms, bonds, alpha and beta electrons")
    name = lines[0].split()[0]
    n, m, na, nb = (int(lines[k].split()[0]) for k in range(1, 5))
    if len(lines) < 5 + n + m:
        raise ValueError(f"the molecule block lists fewer than {n} atoms and {m} bonds")
    coords, alpha, gamma, nels, symbols = np.zeros((n, 3)), np.zeros(n), np.zeros(n), np.zeros(n, dtype=np.int32), []
    for i in range(n):
        f = lines[5 + i].split()
        symbols.append(f[0])
        coords[i] = [float(x) for x in f[1:4]]
        alpha[i], gamma[i], nels[i] = float(f[4]), float(f[5]), int(f[6])
    bonds = []
    for k in range(m):
        f = lines[5 + n + k].split()
        bonds.append((int(f[0]) - 1, int(f[1]) - 1, float(f[2]), f[3].lower() if len(f) > 3 else "nonset"))
    if int(nels.sum()) != na + nb:
        raise ValueError(f"the atoms hold {int(nels.sum())} pi electrons, the header {na} + {nb}")
    return Molecule(name, coords, alpha, gamma, nels, bonds), symbols


def read_input(source: str) -> tuple[Molecule, api.Keywords, Job]:
    """Parse an input file (path or text)."""
    text = source
    if "\n" not in source and "{" not in source:
        with open(source) as f:
            text = f.read()
    blocks, mol_lines = parse_blocks(text)
    mol, symbols = parse_molecule(mol_lines)
    kw = api.Keywords()
    for (blk, key), (attr, kind, _) in _KEYS.items():
        if key in blocks.get(blk, {}):
            setattr(kw, attr, _value(kind, blocks[blk][key]))
    fb = blocks.get("field", {})
    kw.field = tuple(float(fb.get(f"along-{a}", 0.0)) for a in "xyz")
    g, pz, sysb = blocks.get("general", {}), blocks.get("polariz", {}), blocks.get("system", {})
    job = Job(symbols=symbols)
    if "method" in g:
        job.methods = [s.strip().lower() for s in re.split(r"[+\s]+", g["method"]) if s.strip()]
    if "jobtype" in g:
        job.jobtype = g["jobtype"].strip().lower()
    job.output_file = g.get("output-file", job.output_file)
    job.components = pz.get("components", job.components).lower()
    job.points = int(float(pz.get("points", job.points)))
    job.derive_step = float(pz.get("derive-step", job.derive_step))
    job.harvest = _value("bool", sysb["harvest"]) if "harvest" in sysb else False
    for (blk, key), (attr, kind) in _LR_KEYS.items():
        if key in blocks.get(blk, {}):
            setattr(job.lr, attr, _value(kind, blocks[blk][key]))
    if "lr-solver" in blocks.get("engine", {}):
        job.lr_solver = _value("str", blocks["engine"]["lr-solver"])
    return mol, kw, job


def write_input(mol: Molecule, kw: api.Keywords | None = None, job: Job | None = None,
                symbols: list | None = None) -> str:
    """The input file of a molecule, keywords and job (every key the reader knows)."""
    kw = kw or api.Keywords()
    job = job or Job()
    lines = ["%general{", f"  method = {'+'.join(job.methods)},", f"  jobtype = {job.jobtype},",
             f"  output-file = {job.output_file}", "}", ""]
    by_block: dict[str, list] = {}
    for (blk, key), (attr, kind, _) in _KEYS.items():
        v = getattr(kw, attr)
        if kind == "bool":
            v = "true" if v else "false"
        by_block.setdefault(blk, []).append(f"  {key} = {v}")
    by_block["engine"].append(f"  lr-solver = {job.lr_solver}")
    for blk, items in by_block.items():
        lines += [f"%{blk}{{", ",\n".join(items), "}", ""]
    lines += ["%field{", ",\n".join(f"  along-{a} = {float(v)!r}" for a, v in zip("xyz", kw.field)), "}", ""]
    lines += ["%polariz{", f"  components = {job.components},", f"  points = {job.points},",
              f"  derive-step = {job.derive_step!r}", "}", ""]
    lines += ["%system{", f"  harvest = {'true' if job.harvest else 'false'}", "}", ""]
    by_block = {}
    for (blk, key), (attr, kind) in _LR_KEYS.items():
        v = getattr(job.lr, attr)
        by_block.setdefault(blk, []).append(f"  {key} = {('true' if v else 'false') if kind == 'bool' else v}")
    for blk, items in by_block.items():
        lines += [f"%{blk}{{", ",\n".join(items), "}", ""]
    sym = symbols or ["C"] * mol.n_sites
    ne = int(np.sum(mol.nels))
    lines += ["%molecule{", mol.name, str(mol.n_sites), str(len(mol.bonds)), str(ne - ne // 2), str(ne // 2)]
    for i in range(mol.n_sites):
        x, y, z = (float(c) for c in mol.coords[i])
        lines.append(f"{sym[i]} {x!r} {y!r} {z!r} {float(mol.alpha[i])!r} {float(mol.gamma[i])!r} {int(mol.nels[i])}")
    for (i, j, beta, kind) in mol.bonds:
        lines.append(f"{i + 1} {j + 1} {float(beta)!r} {kind}")
    lines += ["}", ""]
    return "\n".join(lines)


def run_input(source: str, harvest_file: str | None = None, engine=None) -> dict:
    """Run the job of an input file on the engine (methods r-ccsd and r-ccsd(t)).

    ``engine`` replaces api.CoupledCluster (a stand-in for tests without a GPU)."""
    mol, kw, job = read_input(source)
    if job.methods not in (["r-ccsd"], ["r-ccsd(t)"]):
        raise ValueError(f"methods {job.methods}: the engine runs r-ccsd and r-ccsd(t)")
    if job.jobtype == "energy" and job.methods == ["r-ccsd"] and job.lr.excited_states_number > 0:
        from . import lrccsd
        lr = lrccsd.linear_response(mol, kw, job.lr, engine=engine, solver=job.lr_solver)
        return {"job": job, "energy": lr["ccsd_energy"], "status": lr["ccsd_status"],
                "iterations": lr["ccsd_iterations"], "excited": lr}
    if job.jobtype == "energy":
        cc = (engine or api.CoupledCluster)(mol, kw)
        cc.initCC()
        out = cc.iterate()
        res = {"job": job, "energy": out["energy"], "status": out["status"], "iterations": out["iterations"]}
        if job.methods == ["r-ccsd(t)"] and out["status"] == 1:
            t = cc.triples(0)
            # the reference adds its triples term to the CCSD energy (energy(1), mod_cc.f90:2104)
            res["triples"] = t
            res["energy_ccsd_t"] = float(out["energy"][0] + t["reference_term"])
            res["energy_ccsd_t_textbook"] = float(out["energy"][0] + t["T"])
        cc.finalizeCC()
        return res
    if job.methods != ["r-ccsd"]:
        raise ValueError("polarizability jobs run r-ccsd")
    if job.jobtype == "polarizability":
        from . import properties
        res, report = properties.polarizability_job(mol, kw, scales=job.components, npoints=job.points,
                                                    step=job.derive_step, harvest_file=harvest_file if job.harvest else None,
                                                    lr=job.lr, lr_solver=job.lr_solver, engine=engine)
        return {"job": job, "properties": res, "report": report}
    raise ValueError(f"jobtype {job.jobtype!r}: the engine runs energy and polarizability jobs")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        print("usage: python -m helios_gb300.inputfile <input-file>", file=sys.stderr)
        sys.exit(2)
    src = sys.argv[1]
    stem = src[:-4] if src.endswith(".inp") else src
    r = run_input(src, harvest_file=stem + ".hrv")
    if "report" in r:
        print(r["report"])
    else:
        e = r["energy"]
        print(f"status {r['status']} iterations {r['iterations']}")
        print(f"E_total {e[0]:.12f} eV  E_ref {e[1]:.12f} eV  E_corr {e[0] - e[1]:.12f} eV")
        if "triples" in r:
            print(f"(T) {r['triples']['T']:.12f} eV  E_CCSD(T) {r['energy_ccsd_t_textbook']:.12f} eV  "
                  f"(reference convention: {r['energy_ccsd_t']:.12f} eV)")
        if "excited" in r:
            x = r["excited"]
            for k in range(len(x["omega"])):
                print(f"state {k + 1}: omega {x['omega'][k]:.10f} eV  E_total {x['E_total'][k]:.12f} eV  "
                      f"r0 {x['r0'][k]:+.6f}  excitation level {x['ael'][k]:.6f}  "
                      f"status {x['status'][k]} iterations {x['iterations'][k]}")
