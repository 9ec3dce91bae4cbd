"""helios input files (helios_gb300/inputfile.py): block syntax of
mod_blockdata.f90:496-630, keys and defaults of definebd.f90, the molecule
block of readMoleculeInformation.f90:20-106. No GPU."""
import numpy as np
import pytest

from helios_gb300 import api, inputfile, molecules

DODECAHEXAENE = """
# all-trans dodecahexaene, C1 of the benchmark
%general{ method = r-ccsd, jobtype = energy }
%Parametrization{
   Coulomb-Integrals = ohno-klopman ,   # comments end at the line end
   bond-alternation = 0.1
}
%coupled-cluster{ accuracy = 10, diis-steps = 20,
                  max-iterations = 500 }
%scf{ accuracy = 11 }
%iteration{ divergence-threshold = 4, enable-stagnation-check = false }
%engine{ precision = mixed, guess = learned }
%molecule{
dodecahexaene
12
11
6
6
"""


def _dodecahexaene_text():
    mol = molecules.dodecahexaene()
    lines = [DODECAHEXAENE.rstrip("\n")]
    for i in range(12):
        x, y, z = mol.coords[i]
        lines.append(f"C {x:.12f} {y:.12f} {z:.12f} 0.0 {mol.gamma[i]} 1")
    for (i, j, beta, kind) in mol.bonds:
        lines.append(f"{i + 1} {j + 1} {beta} {kind}")
    lines.append("}")
    return "\n".join(lines) + "\n"


def test_hand_written_input():
    mol, kw, job = inputfile.read_input(_dodecahexaene_text())
    ref = molecules.dodecahexaene()
    assert mol.name == "dodecahexaene" and mol.n_sites == 12 and len(mol.bonds) == 11
    assert np.allclose(mol.coords, ref.coords, atol=1e-11)
    assert [(b[0], b[1], b[3]) for b in mol.bonds] == [(b[0], b[1], b[3]) for b in ref.bonds]
    assert kw.bond_alternation == 0.1 and kw.coulomb_integrals == "ohno-klopman"
    assert kw.accuracy == 10 and kw.max_iterations == 500 and kw.scf_accuracy == 11
    assert kw.divergence_threshold == 4 and kw.enable_stagnation_check is False
    assert kw.precision == "mixed" and kw.guess == "learned"
    assert kw.t1_step == 1.0 and kw.diis_enabled is True                # defaults
    assert job.methods == ["r-ccsd"] and job.jobtype == "energy" and job.symbols == ["C"] * 12


def test_write_read_round_trip():
    mol = molecules.ladder(10)
    kw = api.Keywords(bond_alternation=-0.05, accuracy=9, field=(0.01, -0.02, 0.0), projection_type="2-1")
    job = inputfile.Job(jobtype="polarizability", components="xy", points=7, derive_step=0.01, harvest=True)
    m2, kw2, job2 = inputfile.read_input(inputfile.write_input(mol, kw, job))
    assert np.array_equal(m2.coords, mol.coords) and np.array_equal(m2.alpha, mol.alpha)
    assert np.array_equal(m2.gamma, mol.gamma) and np.array_equal(m2.nels, mol.nels)
    assert m2.bonds == mol.bonds
    for f in ("bond_alternation", "accuracy", "field", "projection_type", "scf_accuracy", "diis_steps",
              "precision", "guess", "mixed_check"):
        assert getattr(kw2, f) == getattr(kw, f), f
    assert (job2.jobtype, job2.components, job2.points, job2.derive_step, job2.harvest) == \
        ("polarizability", "xy", 7, 0.01, True)


def test_malformed_inputs_are_rejected():
    text = _dodecahexaene_text()
    with pytest.raises(ValueError):                     # 13 pi electrons on 12 sites, header 6 + 6
        inputfile.read_input(text.replace("C 0.000000000000 0.000000000000 0.000000000000 0.0 11.13 1",
                                          "C 0.000000000000 0.000000000000 0.000000000000 0.0 11.13 2"))
    with pytest.raises(ValueError):
        inputfile.read_input(text.replace("bond-alternation = 0.1", "bond-alternation 0.1"))
    with pytest.raises(ValueError):
        inputfile.read_input(text.replace("max-iterations = 500", "max-iterations = 500, diis-enabled = maybe")
                             .replace("%iteration{", "%iteration{ enable-divergence-check = maybe,"))


def test_unknown_method_or_job_is_an_error():
    text = _dodecahexaene_text().replace("method = r-ccsd", "method = u-ccsd")
    with pytest.raises(ValueError):
        inputfile.run_input(text)


def test_states_and_linear_response_blocks():
    text = _dodecahexaene_text().replace(
        "%scf{ accuracy = 11 }",
        "%scf{ accuracy = 11 }\n%states{ excited-states-number = 2 }\n"
        "%Linear-Response{ accuracy = 7, orthogonalization = true, guess = rpa, r1-step = 0.05 }\n"
        "%engine{ lr-solver = davidson }")
    mol, kw, job = inputfile.read_input(text)
    assert job.lr.excited_states_number == 2 and job.lr.spin == 0
    assert job.lr.accuracy == 7 and job.lr.orthogonalization is True and job.lr.guess == "rpa"
    assert job.lr.r1_step == 0.05 and job.lr.r2_step == 0.03 and job.lr.diis_steps == 20     # defaults
    assert job.lr_solver == "davidson" and kw.precision == "mixed"                          # both engine blocks
    m2, kw2, job2 = inputfile.read_input(inputfile.write_input(mol, kw, job))
    assert job2.lr == job.lr and job2.lr_solver == job.lr_solver
    # no states block: no LR run
    assert inputfile.read_input(_dodecahexaene_text())[2].lr.excited_states_number == 0


def test_energy_job_with_excited_states_runs_lr(tmp_path):
    from fake_engine import FakeCoupledCluster
    mol = molecules.polyene(4)
    job = inputfile.Job(lr=inputfile.LRKeywords(excited_states_number=2, accuracy=7), lr_solver="davidson")
    r = inputfile.run_input(inputfile.write_input(mol, api.Keywords(bond_alternation=0.1, accuracy=12), job),
                            engine=FakeCoupledCluster)
    x = r["excited"]
    assert r["status"] == 1 and list(x["status"]) == [1, 1]
    assert np.allclose(x["E_total"], r["energy"][0] + x["omega"])
    assert 0 < x["omega"][0] < x["omega"][1]
