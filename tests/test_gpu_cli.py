"""End to end: the campaign driver cmsl_pe on a small inputs/ tree, against the
oracle run of the same simulation.

The driver reads the reference's formats (InputParams, Landau/phase pools,
inputs/struc1/gdata_poly.bin + gchar_poly.txt, inputs/gnumb_poly.txt) and
writes output/sweep001.txt in the reference's 12-column format.  The expected
rows are rebuilt here from the same inputs with the oracle (FP64, the
reference's PCG tolerances); values agree to the 7 significant digits the
format prints (relative 2e-6) and the count column exactly.
"""
import os
import subprocess

import numpy as np
import pytest

import oracle
from cmsl_gb300 import formats as fm

pytestmark = pytest.mark.gpu

NX, NY, NZ, NG = 24, 16, 6, 9

DECK = f"""device_flag = 0
nx = {NX}
ny = {NY}
nz = {NZ}
del_h = 1.0
del_t = 0.01
delEap = 3.0e+07
Eap = 3.0e+08
num_steps = 1
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
n_layers = 1
layer_counts = {NZ}
G0 = 1.0
omg = 0.075
eps_fe = 30.0
eps_afe = 40.0
eps_de = 15.0
z_bc_type = diri
do_pre_relax = 0
"""
LANDAU = ("5.022532e+08 -9.065448e+10 2.189509e+12 5.453480e+08 1.0e+09 "
          "-2.98e+08 -8.520e+09 3.134e+11 -2.484e+08 1.0e+09 9.5e+09 2.372e+09 FE\n")


def _splitmix(seed, n):
    M = (1 << 64) - 1
    s = seed
    out = np.empty(n)
    for i in range(n):
        s = (s + 0x9E3779B97F4A7C15) & M
        z = s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        z ^= z >> 31
        out[i] = (z >> 11) * (1.0 / 9007199254740992.0)
    return out


@pytest.fixture(scope="module")
def cli():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cmsl_gb300 import build
    build.build_all()
    return build.CLI


def test_campaign_driver_matches_oracle(cli, tmp_path):
    root = tmp_path
    (root / "inputs" / "struc1").mkdir(parents=True)
    (root / "inputs" / "InputParams").write_text(DECK)
    (root / "landau.txt").write_text(LANDAU)
    (root / "phase.txt").write_text("40 60 0\n")
    om, cent, eul = fm.voronoi_columnar(NX, NY, NZ, NG, 11)
    fm.write_grains(str(root / "inputs" / "struc1"), "poly", str(root / "inputs" / "gnumb_poly.txt"), NX, NY, NZ,
                    om, cent, eul)
    r = subprocess.run([cli, "0", str(root / "landau.txt"), str(root / "phase.txt"), "1", "--seed", "5",
                        "--root", str(root)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = (root / "output" / "sweep001.txt").read_text().strip().splitlines()
    assert (root / "OutputParams").exists() and (root / "microstructure.txt").exists()

    # the same simulation through the oracle
    deck = fm.read_deck(str(root / "inputs" / "InputParams"))
    v = [float(x) for x in LANDAU.split()[:12]]
    raw = [dict(alpha=v[0], beta=v[1], gamma1=v[2], g=v[3], a0=v[4], L=deck["L_afe"], kappa=deck["kappa_afe"],
                eps_r=deck["eps_afe"]),
           dict(alpha=v[5], beta=v[6], gamma1=v[7], g=v[8], a0=v[9], L=deck["L_fe"], kappa=deck["kappa_fe"],
                eps_r=deck["eps_fe"]),
           dict(alpha=v[10], beta=0.0, gamma1=0.0, g=0.0, a0=v[11], L=deck["L_de"], kappa=deck["kappa_de"],
                eps_r=deck["eps_de"])]
    mats, sc = fm.nondim(raw, 1, deck["Eap"], deck["delEap"])
    o2, _, c2, _, TR = fm.read_grains(str(root / "inputs" / "struc1"), "poly", NX, NY, NZ, NG)
    gm = fm.assign_materials(NX, NY, NZ, o2, c2[:, 2], [NZ], [0.4], [0.6], [0.0])
    gm[gm < 0] = 1
    orc = oracle.load()
    f = oracle.Film(nx=NX, ny=NY, nz=NZ, del_h=deck["del_h"], del_t=deck["del_t"], omega=o2, grain_mat=gm, TR=TR,
                    mats=mats, is_interface=orc.interface_flags(NX, NY, NZ, o2, gm), dep_flag=1, eps_0_nd=sc["eps_0_nd"])
    N = NX * NY * NZ
    u = _splitmix(34635, N)
    mat = gm[o2]
    P = [np.zeros(N) for _ in range(6)]
    for q in range(3):
        P[q] = np.where(mat == 1, 0.1 * (2.0 * u - 1.0), 0.0)
        P[3 + q] = np.where(mat == 0, 1.0, 0.0)
    Ez, rows, rE, rc = fm.evolve_schedule(sc["maxEz"], sc["delEz"], deck["num_steps"])
    _, _, _, stats, _, rcode = orc.run(f, P, np.zeros(N), Ez, rows)
    assert rcode == 0
    assert len(lines) == len(rE)
    Es, Ps = sc["E0_ref"] / 1.0e8, sc["P0_ref"] * 100.0
    for line, e, st, cnt in zip(lines, rE, stats, rc):
        got = [float(x) for x in line.split("\t")]
        want = [e * Es, st[0] * Ps, st[1] * Ps, st[2] * Ps, st[3] * Ps, st[4] * Ps, st[5], st[6] * Ps, st[7],
                st[8] * Ps, st[9]]
        assert int(got[11]) == cnt
        np.testing.assert_allclose(got[:11], want, rtol=2e-6, atol=1e-12)


@pytest.mark.parametrize("dims", [(32, 24, 5, 13, 7), (257, 130, 3, 600, 11), (64, 64, 16, 1, 2)])
def test_gpu_voronoi_equals_host(cli, dims):
    """The device grain-map generator gives the host generator's map bit for bit."""
    nx, ny, nz, ng, seed = dims
    a = fm.voronoi_columnar(nx, ny, nz, ng, seed)
    b = fm.voronoi_columnar(nx, ny, nz, ng, seed, device=True)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.mark.parametrize("shape", [(24, 20, 8), (64, 48, 12), (7, 5, 3)])
def test_interface_flags_on_device_match_reference_algorithm(cli, shape):
    """build_interface_flag (main.cu:13-52) on device arrays, bitwise against
    the oracle's restatement, on layered maps with FE / AFE / DE grains and
    a map with grain ids outside the table (counted as not FE)."""
    import torch
    import oracle
    from tests.films import voronoi_columnar
    nx, ny, nz = shape
    rng = np.random.default_rng(sum(shape))
    ng = 9
    om = voronoi_columnar(nx, ny, nz, ng, rng)
    kk = np.repeat(np.arange(nz), nx * ny)
    om = np.where(kk % 3 == 1, (om + 4) % ng, om).astype(np.int32)      # z interfaces between grains
    gm = rng.choice([0, 1, 2], size=ng, p=[0.3, 0.5, 0.2]).astype(np.int32)
    gm[0] = 1
    want = oracle.load().interface_flags(nx, ny, nz, om, gm)
    dev = torch.device("cuda", 0)
    d_om = torch.as_tensor(om, device=dev)
    d_gm = torch.as_tensor(gm, device=dev)
    d_fl = torch.full((om.size,), -7, dtype=torch.int32, device=dev)
    L = fm._bind()
    torch.cuda.synchronize()
    fm.check(L.cmsl_interface_flags_gpu(nx, ny, nz, ng, d_om.data_ptr(), d_gm.data_ptr(), d_fl.data_ptr(), None))
    torch.cuda.synchronize()
    assert np.array_equal(d_fl.cpu().numpy(), want)
    # ids outside [0, ng): never read beyond the table, counted as not FE
    om2 = om.copy()
    om2[nx * ny * (nz // 2)] = ng + 5
    om2[nx * ny * (nz // 2) + 1] = -1
    d_om2 = torch.as_tensor(om2, device=dev)
    fm.check(L.cmsl_interface_flags_gpu(nx, ny, nz, ng, d_om2.data_ptr(), d_gm.data_ptr(), d_fl.data_ptr(), None))
    torch.cuda.synchronize()
    got = d_fl.cpu().numpy()
    gmx = np.concatenate([gm, [-1]])
    mat = np.where((om2 >= 0) & (om2 < ng), gmx[np.clip(om2, 0, ng)], -1)
    exp = np.zeros(om2.size, np.int32)
    plane = nx * ny
    for i in range(plane, om2.size - plane):
        if mat[i] == 1:
            exp[i] = int(mat[i + plane] != 1 or mat[i - plane] != 1)
    assert np.array_equal(got, exp)
