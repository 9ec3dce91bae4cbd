"""Jobs run from helios input files on the GPU (inputfile.run_input): the
energy of dodecahexaene against its golden FP64 oracle value, and a
polarizability job with harvesting against the same job built in Python."""
import json
import os

import pytest

from helios_gb300 import inputfile, molecules, properties
from test_inputfile import _dodecahexaene_text

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    from helios_gb300 import build
    build.build()
    from helios_gb300 import api as a
    return a


def test_energy_job_matches_the_golden_value(api):
    gold = {c["name"]: c for c in json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))["cases"]}
    want = gold["dodecahexaene"]["eref"] + gold["dodecahexaene"]["ecorr_1e10"]
    for precision in ("fp64", "mixed"):
        text = _dodecahexaene_text().replace("precision = mixed", f"precision = {precision}")
        r = inputfile.run_input(text)
        assert r["status"] == 1
        assert abs(r["energy"][0] - want) < (1e-9 if precision == "fp64" else 1e-6), precision


def test_polarizability_job_with_harvest(api, tmp_path):
    mol = molecules.polyene(6)
    kw = api.Keywords(bond_alternation=0.1, accuracy=11)
    job = inputfile.Job(jobtype="polarizability", components="x", points=5, derive_step=0.05, harvest=True)
    path = os.path.join(tmp_path, "hexatriene.hrv")
    r = inputfile.run_input(inputfile.write_input(mol, kw, job), harvest_file=path)
    want, _ = properties.polarizability_job(mol, kw, scales="x", npoints=5, step=0.05)
    assert r["properties"]["stencils"][5]["alpha"]["xx"] == pytest.approx(want["stencils"][5]["alpha"]["xx"], rel=1e-9)
    rec = properties.read_harvester(path)[0]
    assert rec["scales"] == "x" and rec["points"] == 5
    assert rec["a"][0] == pytest.approx(want["stencils"][5]["alpha"]["xx"], rel=1e-9)
    assert "Polarizability results for r-ccsd" in r["report"]


def test_ccsd_t_energy_job(api):
    text = _dodecahexaene_text().replace("precision = mixed", "precision = fp64").replace("method = r-ccsd", "method = r-ccsd(t)")
    r = inputfile.run_input(text)
    t = r["triples"]
    assert t["T"] < 0 and r["energy_ccsd_t_textbook"] == pytest.approx(r["energy"][0] + t["T"])
    assert r["energy_ccsd_t"] == pytest.approx(r["energy"][0] - t["T"])
