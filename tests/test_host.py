"""CPU tests of the host side: the C-ABI library, keywords, generators, replicas, stencils."""
import ctypes
import os
import re

import numpy as np
import pytest

from helios_gb300 import molecules, polariz, replicas

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="session")
def lib():
    import shutil
    if not (shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")):
        pytest.skip("nvcc is not installed")
    from helios_gb300 import build as b
    b.build()
    from helios_gb300 import api
    return api.library()


def test_library_exports_every_declared_symbol(lib):
    header = open(os.path.join(ROOT, "include", "helios_cc.h")).read()
    declared = set(re.findall(r"\b(hx_[a-z_0-9]+)\s*\(", header))
    assert {"hx_ccsd_create", "hx_ccsd_init", "hx_ccsd_iterate", "hx_ccsd_energy", "hx_ccsd_solve",
            "hx_ccsd_destroy", "hx_last_error"} <= declared
    for name in declared:
        assert hasattr(lib, name), name


def test_default_parameters_are_helios_defaults(lib):
    from helios_gb300 import api
    p = api.CCParams()
    lib.hx_cc_params_default(ctypes.byref(p))
    assert p.cc_maxiter == 2000 and p.cc_eps == 1e-12 and p.diis_steps == 20 and p.diis_enabled == 1
    assert p.scf_maxiter == 400 and p.scf_eps == 1e-12 and p.scf_step == 0.05
    assert p.projection_type == 2 and p.divergence_threshold == 1e3 and p.stagnation_after == 200
    assert p.stagnation_threshold == 60.0
    # engine keys after the reference's: mixed-precision ladder defaults
    assert p.mixed_switch == 1e-3 and p.mixed_patience == 3 and p.mixed_check == 0
    assert p.tile_tuning == 0 and p.tile_force == -1


def test_keywords_potentiate_like_the_reference(lib):
    from helios_gb300 import api
    p = api.Keywords(accuracy=10, scf_accuracy=11, divergence_threshold=4, projection_type="2-1").to_c()
    assert p.cc_eps == pytest.approx(1e-10) and p.scf_eps == pytest.approx(1e-11)
    assert p.divergence_threshold == pytest.approx(1e4) and p.projection_type == 2


def test_create_rejects_bad_input_without_a_gpu_call(lib):
    from helios_gb300 import api
    p = api.Keywords().to_c()
    h = ctypes.c_void_p()
    assert lib.hx_ccsd_create_batch(None, 0, ctypes.byref(p), ctypes.byref(h)) == -100
    buf = ctypes.create_string_buffer(256)
    assert lib.hx_last_error(buf, 256) > 0


@pytest.mark.parametrize("field,value", [("projection_type", 3), ("projection_type", 0), ("diis_steps", 1),
                                         ("diis_steps", 51), ("precision", 3), ("mixed_check", 2),
                                         ("tile_tuning", 3), ("tile_force", -2)])
def test_create_rejects_bad_keywords_without_a_gpu_call(lib, field, value):
    """Keyword values outside the ranges definebd.f90 accepts (and the engine options' ranges)
    are refused before any device is touched, with the error text set."""
    from helios_gb300 import api, molecules
    p = api.Keywords().to_c()
    setattr(p, field, value)
    arrays = api._ModelArrays(molecules.polyene(4))
    models = (api.PPPModel * 1)(arrays.c)
    h = ctypes.c_void_p()
    good = api.Keywords().to_c()                  # control: only the device is missing (or present)
    rc = lib.hx_ccsd_create_batch(models, 1, ctypes.byref(good), ctypes.byref(h))
    assert rc in (-101, 0)
    if rc == 0:
        lib.hx_ccsd_destroy(h)
        h = ctypes.c_void_p()
    assert lib.hx_ccsd_create_batch(models, 1, ctypes.byref(p), ctypes.byref(h)) == -100
    buf = ctypes.create_string_buffer(256)
    assert lib.hx_last_error(buf, 256) > 0 and not h.value


def test_tile_table_selection_logic(lib, tmp_path):
    # the autotuner's table on the host (no GPU call): candidates per mode, merging,
    # range checks, the shipped file format, and the keywords that steer it
    from helios_gb300 import api
    widths = [api.tile_variants(m) for m in range(4)]
    assert [w[0] for w in widths] == [64, 64, 48, 32]            # the defaults come first
    assert all(len(w) >= 2 and all(x % 16 == 0 for x in w) for w in widths)
    assert lib.hx_tile_variants(4, None, 0) == -100
    before = dict(((e[0], e[1], e[2], e[3]), e[4]) for e in api.tile_table())
    api.load_tile_table([(0, 900, 7, 20, 1), (3, 901, 4, 10, 1)])
    api.load_tile_table([(0, 900, 7, 20, 2)])                     # a later entry replaces an earlier one
    got = dict(((e[0], e[1], e[2], e[3]), e[4]) for e in api.tile_table())
    assert got[(0, 900, 7, 20)] == 2 and got[(3, 901, 4, 10)] == 1
    assert {k: v for k, v in got.items() if k[1] < 900} == before
    with pytest.raises(api.HxError):
        api.load_tile_table([(2, 902, 3, 3, len(widths[2]))])      # no such candidate
    with pytest.raises(api.HxError):
        api.load_tile_table([(4, 903, 3, 3, 0)])                   # no such mode
    path = str(tmp_path / "t.json")
    api.write_tile_table(path, [(1, 2, 3, 4, 1), (0, 1, 2, 3, 0)])
    assert api.read_tile_table(path) == [(0, 1, 2, 3, 0), (1, 2, 3, 4, 1)]
    p = api.Keywords(tile_tuning="tune", tile_force=2).to_c()
    assert p.tile_tuning == 1 and p.tile_force == 2
    assert api.Keywords(tile_tuning="default").to_c().tile_tuning == 2
    if os.path.exists(api.TILE_TABLE_PATH):                        # the shipped table is valid and loaded
        shipped = api.read_tile_table(api.TILE_TABLE_PATH)
        assert shipped and all(0 <= e[4] < len(widths[e[0]]) for e in shipped)
        assert set((e[0], e[1], e[2], e[3]) for e in shipped) <= set(got)


def _is_perfect_matching(mol):
    seen = set()
    for (i, j, beta, kind) in mol.bonds:
        if kind == "double":
            if i in seen or j in seen:
                return False
            seen.update((i, j))
    return len(seen) == mol.n_sites


@pytest.mark.parametrize("n", [4, 6, 8, 10, 12, 30, 64])
def test_ladder_geometry_and_kekule(n):
    m = molecules.ladder(n)
    assert m.n_sites == n and m.n_electrons == n
    assert _is_perfect_matching(m)
    assert np.allclose(m.coords[:, 2], 0.0)
    for (i, j, _, _) in m.bonds:
        assert np.linalg.norm(m.coords[i] - m.coords[j]) == pytest.approx(1.40)


@pytest.mark.parametrize("n", [2, 12, 160])
def test_polyene_geometry(n):
    m = molecules.polyene(n)
    assert _is_perfect_matching(m)
    for k, (i, j, _, kind) in enumerate(m.bonds):
        d = np.linalg.norm(m.coords[i] - m.coords[j])
        assert d == pytest.approx(1.35 if kind == "double" else 1.46)
    if n >= 3:
        a, b, c = m.coords[0], m.coords[1], m.coords[2]
        cosang = np.dot(a - b, c - b) / np.linalg.norm(a - b) / np.linalg.norm(c - b)
        assert cosang == pytest.approx(-0.5)


def test_random_ensemble_is_seeded_and_in_range():
    a = molecules.ensemble(100, 64)
    b = molecules.ensemble(100, 64)
    assert [m.name for m in a] == [m.name for m in b]
    assert all(8 <= m.n_sites <= 64 and m.n_sites % 2 == 0 for m in a)
    kinds = {m.name.split("-")[1] for m in a}
    assert kinds == {"polyene", "ladder"}
    assert all(_is_perfect_matching(m) for m in a)


def test_stencil_weights_match_oracle():
    from oracle.polariz import lagrange_derivative_weights
    for n in (3, 5, 7, 9):
        assert np.allclose(polariz.lagrange_weights(n, 2), lagrange_derivative_weights(n, 2), atol=1e-12)
    assert np.allclose(polariz.lagrange_weights(5, 2) * 12, [-1, 16, -30, 16, -1])


def test_alpha_of_a_quadratic_energy():
    # E(F) = E0 - alpha_ev F^2 / 2 in eV with F in V/Angstrom -> alpha in a.u.
    h = 0.0514221
    F = np.arange(-2, 3) * h
    a_au = 123.0
    alpha_ev = a_au / (polariz.HARTREE_ENERGY / polariz.BOHR_RADIUS ** 2)
    E = -5.0 - 0.5 * alpha_ev * F ** 2
    assert polariz.alpha_from_energies(E, h) == pytest.approx(a_au, rel=1e-12)


def test_field_molecule_equals_oracle_field_model():
    from oracle.ppp import build_model
    m = molecules.polyene(10)
    a = build_model(polariz.field_molecule(m, 0.03), alternation=0.1)
    b = build_model(m, alternation=0.1, field=(0.03, 0, 0))
    assert np.allclose(a["core"], b["core"], atol=1e-13)
    assert np.allclose(a["huckelCore"], b["huckelCore"], atol=1e-13)


def test_shards_cover_every_molecule_once():
    mols = molecules.ensemble(7, 50)
    for world in (1, 2, 3, 8):
        got = sorted(i for r in range(world) for i in replicas.shard(mols, r, world))
        assert got == list(range(len(mols)))


def _replica_worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle.literal import solve_literal
    mols = [molecules.polyene(n) for n in (4, 6, 8, 4, 6)]
    mine = replicas.shard(mols, rank, world)
    local = {i: solve_literal(mols[i], eps=1e-10)["ecorr"] for i in mine}
    out = replicas.gather(local, rank, world)
    if rank == 0:
        q.put(out)
    dist.destroy_process_group()


def test_replicas_gather_over_gloo():
    import multiprocessing as mp
    import random
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + random.randint(0, 2000)
    ps = [ctx.Process(target=_replica_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = q.get(timeout=120)
    for p in ps:
        p.join(timeout=60)
    assert sorted(out) == [0, 1, 2, 3, 4]
    assert out[0] == pytest.approx(out[3]) and out[1] == pytest.approx(out[4])


def test_tensor_core_slicing_is_an_exact_digit_expansion(tmp_path):
    """hx_slice.h on the host: |digits| <= 128 and sum_p s_p 2^-8p equals
    x 2^(7-e) to within half a unit of the last digit; e is frexp's exponent;
    the kernels' residue form of the splitting and their bf16 digit values
    agree with it for 3, 4, 5 and 7 digits."""
    import shutil
    import subprocess
    if shutil.which("g++") is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "slice_harness"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "helios_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "slice_harness.cpp"), "-o", str(exe)], check=True)
    rng = np.random.default_rng(4)
    rows = []
    for _ in range(4000):
        mx = float(np.exp(rng.uniform(-40, 40)))
        x = float(mx * rng.uniform(-1, 1))
        rows.append((mx, x))
    for mx in (1.0, 0.75, 3.0, 5e-324, 2.2250738585072014e-308, 1e300):
        rows += [(mx, mx), (mx, -mx), (mx, 0.0), (mx, mx * 0.5), (mx, float(np.nextafter(mx, 0)))]
    rows += [(2.0 ** 10, (2 ** 3 + 0.5) * 2.0 ** -13), (1.0, 2.0 ** -30), (1.0, -(2.0 ** -17) * 1.5)]
    for _ in range(4000):                 # digits near the half-way points between digit values
        mx = float(np.exp(rng.uniform(-40, 40)))
        e = int(np.frexp(mx)[1])
        n = int(rng.integers(-(2 ** 38), 2 ** 38)) * 256 + int(rng.choice([-128, 127, 128, -127, 0]))
        rows.append((mx, float(np.ldexp(float(n), e - 7 - 40))))
    inp = "".join(f"{mx.hex()} {x.hex()}\n" for mx, x in rows)
    out = subprocess.run([str(exe)], input=inp, capture_output=True, text=True, check=True).stdout.split("\n")
    for (mx, x), line in zip(rows, out):
        v = [int(t) for t in line.split()]
        e = np.frexp(mx)[1] if mx != 0 else 0
        assert v[0] == e and v[9] == 1
        a = np.ldexp(x, 7 - e)
        for digits in (v[1:4], v[4:9]):
            S = len(digits)
            assert max(abs(d) for d in digits) <= 128
            recon = sum(np.ldexp(float(d), -8 * p) for p, d in enumerate(digits))
            assert abs(recon - a) <= np.ldexp(1.0, -8 * (S - 1) - 1) * (1 + 1e-12)


def test_amplitude_layout_conversions(tmp_path):
    """hx_layout.h on the host: the reference's column-major t1(o, v) and
    t2(o, o, v, v) become the engine's row-major t1 [i][a] and pair-ordered
    t2 [i][a][j][b] (numpy's transposes of the same arrays), and back."""
    import shutil
    import subprocess
    if shutil.which("g++") is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "layout_harness"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "helios_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "layout_harness.cpp"), "-o", str(exe)], check=True)
    shapes = [(1, 1), (1, 3), (4, 1), (3, 5), (6, 2), (16, 16), (7, 33)]
    out = subprocess.run([str(exe)], input="".join(f"{o} {v}\n" for o, v in shapes),
                         capture_output=True, text=True, check=True).stdout.split()
    pos = 0
    for o, v in shapes:
        n1, n2 = o * v, (o * v) ** 2
        f1 = np.arange(n1).reshape((o, v), order="F")
        f2 = np.arange(n2).reshape((o, o, v, v), order="F")
        e1 = np.array(out[pos:pos + n1], dtype=np.int64)
        e2 = np.array(out[pos + n1:pos + n1 + n2], dtype=np.int64)
        assert np.array_equal(e1, f1.reshape(-1))
        assert np.array_equal(e2, f2.transpose(0, 2, 1, 3).reshape(-1))
        assert out[pos + n1 + n2] == "1"
        pos += n1 + n2 + 1
    assert pos == len(out)


def test_epilogue_integer_conversions(tmp_path):
    """The GEMM epilogue's integer routes (hx_slice.h) on the host: f2d_pow2
    of hi and of lo, added in FP64, give (hi + lo) 2^k to within one FP64 ulp
    (checked in exact rational arithmetic; FP32 subnormals count as zero);
    pow2_int is an exact power-of-two scale; class_count recovers the integer
    count of an exact class sum."""
    import shutil
    import subprocess
    from fractions import Fraction
    if shutil.which("g++") is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "epilogue_harness"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "helios_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "epilogue_harness.cpp"), "-o", str(exe)], check=True)
    rng = np.random.default_rng(11)
    f32 = lambda x: float(np.float32(x))
    cases = []
    for _ in range(3000):
        hi = f32(rng.normal() * 2.0 ** rng.integers(-30, 30))
        # lo below half an ulp of hi (what TwoSum leaves), or a little more
        lo = f32(hi * rng.uniform(-1, 1) * 2.0 ** -float(rng.integers(22, 60)))
        cases.append((hi, lo, int(rng.integers(-896, 897)), int(rng.integers(0, 2))))
    cases += [(0.0, 0.0, 3, 0), (0.0, 1.5, -2, 1), (1.0, 0.0, 0, 0), (-1.0, 2.0 ** -30, 5, 0),
              (1.0, -(2.0 ** -25), 0, 0), (2.0 ** -126, 0.0, 0, 0), (1e-45, 0.0, 0, 0),
              (1.0, 1.0, 0, 0), (3.0, 2.0 ** -100, 896, 0), (f32(3.4e38), 2.0 ** 100, 896, 0),
              (2.0 ** -126, 2.0 ** -126, -896, 1)]
    inp = "".join(f"f {hi.hex()} {lo.hex()} {k} {n}\n" for hi, lo, k, n in cases)
    xs = [(float(rng.normal() * 10.0 ** rng.integers(-200, 200)), int(rng.integers(-300, 300))) for _ in range(500)]
    xs += [(0.0, 7), (-0.0, -7), (5e-324, 3), (1e308, 100), (1.0, -1100)]
    inp += "".join(f"p {x.hex()} {k}\n" for x, k in xs)
    cs = []
    for _ in range(2000):
        q = int(rng.integers(0, 7))
        n = int(rng.integers(-(2 ** 24) + 1, 2 ** 24))
        cs.append((n, q))
    cs += [(0, 0), (0, 6), (1, 6), (-1, 0), (2 ** 24 - 1, 3), (-(2 ** 24 - 1), 5)]
    inp += "".join(f"c {float(np.ldexp(np.float32(n), -8 * q)).hex()} {q}\n" for n, q in cs)
    out = subprocess.run([str(exe)], input=inp, capture_output=True, text=True, check=True).stdout.split("\n")
    for (hi, lo, k, n), line in zip(cases, out):
        ok, val = line.split()
        flush = lambda x: 0.0 if abs(x) < 2.0 ** -126 else x
        exact = (Fraction(flush(hi)) + Fraction(flush(lo))) * Fraction(2) ** k * (-1 if n else 1)
        got = Fraction(float.fromhex(val))
        assert abs(got - exact) <= abs(exact) * Fraction(2) ** -52, (hi, lo, k, n, val)
    off = len(cases)
    for (x, k), line in zip(xs, out[off:]):
        ok, val = line.split()
        with np.errstate(over="ignore"):
            ref = np.ldexp(x, k)
        if ok == "1":
            assert float.fromhex(val) == ref
        else:
            assert not np.isfinite(ref) or abs(ref) < 2.3e-308 or abs(x) < 2.3e-308
    off += len(xs)
    for (n, q), line in zip(cs, out[off:]):
        assert int(line) == n
