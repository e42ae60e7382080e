"""CPU tests of the reference formats and set-up (include/cmsl_io.h) against
the reference's own host code (oracle/_ref) and the oracle."""
import os

import numpy as np
import pytest

import oracle
from cmsl_gb300 import formats as fm
from cmsl_gb300 import schedule as sch
from tests.films import random_film

_RR = oracle.reference_root()
REF_ROOT = os.path.join(_RR, "HZO_Code_github") if _RR else None


@pytest.fixture(scope="module")
def ref():
    r = oracle.load_ref()
    if r is None:
        pytest.skip("reference sources not available")
    return r


@pytest.fixture(scope="module", autouse=True)
def built():
    from cmsl_gb300 import build
    build.build()


DECK = """device_flag = 1
nx = 40
ny = 24
nz = 12
del_h = 0.5
del_t = 1.0e-3
delEap = 6.0e+05
Eap = 3.0e+08
num_steps = 2
out_flag = 0
dep_flag = 1
L_de = 1.0
kappa_de = 2.5e-09
kappa_fe = 5.066e-10
L_fe = 0.833
kappa_afe = 1.0e-09
L_afe = 0.2
dimx = 8
dimy = 4
dimz = 4
crystal_type = poly
PsNoise = 0.01
n_layers = 2
layer_counts = 5 7
G0 = 1.0
omg = 0.075
eps_fe = 30.0
eps_afe = 40.0
eps_de = 15.0
z_bc_type = neu
do_pre_relax = 1
nxtra = 99
"""


def _compare_decks(mine, theirs):
    for k in ("nx", "ny", "nz", "dep_flag", "num_steps", "dimx", "dimy", "dimz", "n_layers", "do_pre_relax"):
        assert mine[k] == theirs[k], k
    for k in ("del_h", "del_t", "delEap", "Eap", "kappa_fe", "L_fe", "kappa_afe", "L_afe", "kappa_de", "L_de",
              "eps_fe", "eps_afe", "eps_de"):
        assert mine[k] == theirs[k], k
    assert mine["crystal_type"] == theirs["crystal_type"]
    assert mine["z_bc_type"] == theirs["z_bc_type"]
    assert mine["layer_counts"] == theirs["layer_counts"]


def test_deck_synthetic_vs_reference_parser(ref, tmp_path):
    p = tmp_path / "InputParams"
    p.write_text(DECK)
    mine = fm.read_deck(str(p))
    theirs = ref.read_deck(str(p), str(tmp_path / "OutputParams_ref"))
    _compare_decks(mine, theirs)
    assert mine["nx"] == 40   # "nxtra = 99" does not match "nx = %d"


@pytest.mark.parametrize("rel", ["inputs/InputParams", "src/inputs/InputParams"])
def test_shipped_decks_vs_reference_parser(ref, tmp_path, rel):
    path = os.path.join(REF_ROOT, rel)
    if not os.path.exists(path):
        pytest.skip("shipped deck not available")
    mine = fm.read_deck(path)
    theirs = ref.read_deck(path, str(tmp_path / "OutputParams_ref"))
    _compare_decks(mine, theirs)


def test_deck_layer_sum_error(tmp_path):
    p = tmp_path / "bad"
    p.write_text(DECK.replace("layer_counts = 5 7", "layer_counts = 5 6"))
    import cmsl_gb300 as cg
    with pytest.raises(cg.CmslError) as e:
        fm.read_deck(str(p))
    assert e.value.status == 3


def test_deck_summary_matches_reference(ref, tmp_path):
    p = tmp_path / "InputParams"
    p.write_text(DECK)
    theirs_path = tmp_path / "OutputParams_ref"
    ref.read_deck(str(p), str(theirs_path))
    d = fm.read_deck(str(p))
    mine_path = tmp_path / "OutputParams_mine"
    fm.write_deck_summary(d, str(mine_path))
    assert mine_path.read_text() == theirs_path.read_text()


def test_grain_files_round_trip_through_reference_reader(ref, tmp_path):
    nx, ny, nz, ng = 20, 12, 6, 9
    om, cent, eul = fm.voronoi_columnar(nx, ny, nz, ng, 5)
    eta = np.random.default_rng(1).uniform(0, 1, nx * ny * nz)
    fm.write_grains(str(tmp_path), "poly", str(tmp_path / "gnumb_poly.txt"), nx, ny, nz, om, cent, eul, eta)
    assert fm.grain_count(str(tmp_path / "gnumb_poly.txt")) == ng
    o2, e2, c2, u2, tr2 = fm.read_grains(str(tmp_path), "poly", nx, ny, nz, ng)
    o3, e3, tr3, c3, u3 = ref.load_grain(str(tmp_path), "poly", nx, ny, nz, ng)
    assert np.array_equal(o2, om) and np.array_equal(o3, om)
    assert np.array_equal(e2, eta) and np.array_equal(e3, eta)
    assert np.array_equal(c2, c3) and np.array_equal(u2, u3)
    assert np.array_equal(tr2, tr3)


def test_grain_read_errors(tmp_path):
    import cmsl_gb300 as cg
    with pytest.raises(cg.CmslError):
        fm.read_grains(str(tmp_path), "none", 4, 4, 4, 2)
    (tmp_path / "gdata_short.bin").write_bytes(b"\0" * 10)
    with pytest.raises(cg.CmslError):
        fm.read_grains(str(tmp_path), "short", 4, 4, 4, 2)


@pytest.mark.parametrize("fr", [(0.4, 0.6, 0.0), (0.3, 0.5, 0.2), (0.0, 1.0, 0.0), (0.2, 0.2, 0.6)])
def test_material_assignment_vs_reference(ref, fr):
    f, _ = random_film(30, 22, 8, seed=16, n_grains=40)
    cz = np.full(int(f.grain_mat.size), 3.5)
    mine = fm.assign_materials(30, 22, 8, f.omega, cz, [8], [fr[0]], [fr[1]], [fr[2]])
    theirs = ref.assign_materials(30, 22, 8, f.omega, cz, [8], [fr[0]], [fr[1]], [fr[2]])
    assert np.array_equal(mine, theirs)


def test_nondim_vs_reference(ref):
    fe = dict(alpha=-2.98e8, beta=-8.52e9, gamma1=3.134e11, g=-2.484e8, a0=1e9, L=0.833, kappa=5.066e-10, eps_r=30.0)
    afe = dict(alpha=5.022532e8, beta=-9.065448e10, gamma1=2.189509e12, g=5.45348e8, a0=1e9, L=0.2, kappa=1e-9,
               eps_r=40.0)
    de = dict(alpha=9.5e9, beta=0.0, gamma1=0.0, g=0.0, a0=2.372e9, L=1.0, kappa=2.5e-9, eps_r=15.0)
    raw = [afe, fe, de]
    for ref_type in (0, 1):
        mats, sc = fm.nondim(raw, ref_type, 3.0e8, 6.0e5)
        for q in range(3):
            want, (ar, p0) = ref.make_nd(raw[q], raw[ref_type])
            assert np.array_equal(mats[q], want)
            assert sc["alpha_ref"] == ar and sc["P0_ref"] == p0
        assert sc["E0_ref"] == (0.25 * sc["alpha_ref"] * sc["P0_ref"] * sc["P0_ref"]) / sc["P0_ref"]
        assert sc["maxEz"] == 3.0e8 / sc["E0_ref"] and sc["delEz"] == 6.0e5 / sc["E0_ref"]


def test_interface_flags_vs_oracle():
    f, _ = random_film(18, 14, 9, seed=3, layered=True)
    o = oracle.load()
    assert np.array_equal(fm.interface_flags(18, 14, 9, f.omega, f.grain_mat),
                          o.interface_flags(18, 14, 9, f.omega, f.grain_mat))


def test_tr_matches_oracle():
    rng = np.random.default_rng(4)
    a = [rng.uniform(0, 6.28, 11) for _ in range(3)]
    assert np.array_equal(fm.tr_from_euler(*a), oracle.load().tr_from_euler(*a))


@pytest.mark.parametrize("args", [(0.335, 6.7e-4, 1, 1), (0.5, 0.01, 3, 1), (0.4, 0.02, 1, 2)])
def test_schedule_cpp_matches_python(args):
    maxEz, delEz, ns, npd = args
    Ez, rows, rE, rc = fm.evolve_schedule(maxEz, delEz, ns, npd)
    s = sch.evolve_schedule(maxEz, delEz, ns, n_periods=npd)
    assert np.array_equal(Ez, s.Ez) and np.array_equal(rows, s.rows)
    assert np.array_equal(rE, s.row_E) and np.array_equal(rc, s.row_count)


def test_landau_and_phase_pools(tmp_path):
    p = tmp_path / "pool.txt"
    p.write_text("# header\n\n"
                 "5.0e8 -9.0e10 2.1e12 5.4e8 1.0e9 -3.0e8 -8.5e9 3.1e11 -2.5e8 1.0e9 9.5e9 2.4e9 AFE\n"
                 "5.0e8 -9.0e10 2.1e12 5.4e8 1.0e9 -3.0e8 -8.5e9 3.1e11 -2.5e8 1.0e9 9.5e9 2.4e9 10 90 0 FE\n"
                 "1 2 3 bad\n")
    sets = fm.read_landau_pool(str(p))
    assert len(sets) == 2
    assert sets[0]["ref_type"] == 0 and sets[0]["fractions"] is None
    assert sets[1]["ref_type"] == 1 and sets[1]["fractions"] == (10.0, 90.0, 0.0)
    assert sets[0]["afe"][0] == 5.0e8 and sets[0]["de"][1] == 2.4e9
    q = tmp_path / "phase.txt"
    q.write_text("40 60 0\n10 30 60\n20 50 30\n")
    a, f, d = fm.read_phase_pool(str(q))
    assert np.allclose(a, [0.4, 0.2]) and np.allclose(d, [0.0, 0.3])


@pytest.mark.parametrize("rel", ["inputs/SingleL_input.txt", "inputs/TwoL_input.txt"])
def test_shipped_16_column_tables(rel):
    path = os.path.join(REF_ROOT, rel) if REF_ROOT else None
    if not path or not os.path.exists(path):
        pytest.skip("shipped table not available")
    sets = fm.read_landau_pool(path)
    assert len(sets) > 0 and all(s["fractions"] is not None for s in sets)


def test_voronoi_deterministic():
    a = fm.voronoi_columnar(32, 24, 5, 13, 7)
    b = fm.voronoi_columnar(32, 24, 5, 13, 7)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    om = a[0].reshape(5, 24, 32)
    assert (om == om[0]).all() and om.min() >= 0 and om.max() < 13
    ct = np.abs(np.cos(a[2][:, 1]))
    assert (ct >= 0.3 - 1e-12).all() and (ct <= 1.0).all()


def test_loop_metrics_known_loop():
    """Pr and Ec of an analytic loop P = tanh((E +- Ec)/w) on a triangle wave."""
    from cmsl_gb300 import pe
    Ec, wd, n = 0.3, 0.1, 4000
    t = np.arange(n)
    E = 1.0 - np.abs(2.0 * t / (n - 1) - 1.0) * 2.0          # +1 -> -1 -> +1
    down = np.r_[True, np.diff(E) < 0]
    P = np.where(down, np.tanh((E + Ec) / wd), np.tanh((E - Ec) / wd))
    m = pe.loop_metrics(E, P)
    assert abs(m["Ec"] - Ec) < 1e-3 and abs(m["Ec_plus"] - Ec) < 1e-3 and abs(m["Ec_minus"] + Ec) < 1e-3
    want = np.tanh(Ec / wd)
    assert abs(m["Pr"] - want) < 1e-3
    r = pe.relative_errors(m, m)
    assert r["Pr"] == 0.0 and r["Ec"] == 0.0


def _fields(n, seed):
    rng = np.random.default_rng(seed)
    return [rng.normal(size=n) for _ in range(6)], [rng.normal(size=n) for _ in range(3)]


def test_checkpoint_bytes_equal_reference_writer(ref, tmp_path):
    nx, ny, nz = 7, 5, 4
    P, E = _fields(nx * ny * nz, 1)
    mine, theirs = tmp_path / "mine.bin", tmp_path / "theirs.bin"
    fm.write_checkpoint(str(mine), nx, ny, nz, P, E, peloop=2, count=1234, Ez_ext=0.125, incEz=-3.5e-4)
    ref.write_checkpoint(str(theirs), P, E, nx, ny, nz, 0.125, 2, 1234, -3.5e-4)
    assert mine.read_bytes() == theirs.read_bytes()


def test_checkpoint_read_of_reference_file(ref, tmp_path):
    nx, ny, nz = 6, 4, 5
    P, E = _fields(nx * ny * nz, 2)
    p = tmp_path / "ck.bin"
    ref.write_checkpoint(str(p), P, E, nx, ny, nz, -0.25, 1, 77, 1e-3)
    P2, E2, pe, cnt, ez, inc = fm.read_checkpoint(str(p), nx, ny, nz)
    assert (pe, cnt, ez, inc) == (1, 77, -0.25, 1e-3)
    assert all(np.array_equal(a, b) for a, b in zip(P2 + E2, P + E))
    P3, E3, pe3, cnt3, ez3, inc3 = ref.read_checkpoint(str(p), nx, ny, nz)
    assert all(np.array_equal(a, b) for a, b in zip(P3 + E3, P + E)) and (pe3, cnt3) == (1, 77)


def test_checkpoint_errors(tmp_path):
    import cmsl_gb300 as cg
    P, E = _fields(24, 3)
    p = tmp_path / "ck.bin"
    fm.write_checkpoint(str(p), 2, 3, 4, P, E)
    with pytest.raises(cg.CmslError) as e:
        fm.read_checkpoint(str(p), 3, 2, 4)
    assert e.value.status == 3 and "mismatch" in str(e.value)
    p.write_bytes(p.read_bytes()[:100])
    with pytest.raises(cg.CmslError):
        fm.read_checkpoint(str(p), 2, 3, 4)


def test_vector_field_bytes_equal_reference(ref, tmp_path):
    nx, ny, nz = 5, 4, 3
    P, _ = _fields(nx * ny * nz, 4)
    mine, theirs = tmp_path / "m.bin", tmp_path / "t.bin"
    fm.write_vector_field(str(mine), P[0], P[1], P[2], 0.37)
    ref.write_vector_field(str(theirs), P[0], P[1], P[2], nx, ny, nz, 0.37)
    assert mine.read_bytes() == theirs.read_bytes()


@pytest.mark.parametrize("shape", [(5, 4, 3), (7, 6, 8)])
def test_midplane_slice_bytes_equal_reference(ref, tmp_path, shape):
    nx, ny, nz = shape
    v = np.random.default_rng(11).normal(size=nx * ny * nz) * 1e-3
    mine, theirs = tmp_path / "m.dat", tmp_path / "t.dat"
    fm.write_midplane_slice(str(mine), v, nx, ny, nz)
    ref.write_midplane_slice(str(theirs), v, nx, ny, nz)
    assert mine.read_bytes() == theirs.read_bytes()


def test_crystal_z_equals_reference_local_output(ref):
    """The crystal-frame z components are kernelCalc_antiferro's Pmz_local /
    Psz_local outputs (kernels_evol.cu:160-175), bit for bit."""
    f, P = random_film(9, 7, 5, seed=12)
    _, loc = ref.tdgl_step(f, P, 0.2)
    assert np.array_equal(fm.crystal_z(f.omega, f.TR, P[0], P[1], P[2]), loc[2])
    assert np.array_equal(fm.crystal_z(f.omega, f.TR, P[3], P[4], P[5]), loc[5])


@pytest.mark.parametrize("zbc", [oracle.DIRICHLET, oracle.NEUMANN])
def test_host_efield_matches_reference_kernel(ref, zbc):
    f, _ = random_film(9, 7, 5, seed=8, zbc=zbc)
    phi = np.random.default_rng(9).normal(size=f.N)
    mine = fm.efield(9, 7, 5, f.del_h, zbc, phi)
    theirs = ref.efield(f, phi)
    assert all(np.array_equal(a, b) for a, b in zip(mine, theirs))
