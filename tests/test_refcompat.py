"""The reference's driver entry points (Evolve, Depol_field,
evolve_resources_init/cleanup) provided by cmsl_gb300/cmsl_refcompat.o over the
reference's globals.

* CPU: the reference's own program (main.cu and the set-up sources, compiled
  where they lie) links against libcmsl_gb with the compat object in place of
  evolve.cu, kernels_evol.cu and depol_varEPS.cu.
* GPU: Evolve() driven through reference-layout globals
  (tests/refcompat/globals_stub.cu) writes the sweep file and final state the
  oracle computes for the same inputs.
"""
import os
import struct
import subprocess

import numpy as np
import pytest

import oracle
from cmsl_gb300 import formats as fm
from tests.films import random_film

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


@pytest.fixture(scope="module")
def compat():
    from cmsl_gb300 import build
    build.build_all()
    return build


def test_reference_program_links_against_compat_layer(compat, tmp_path):
    import oracle
    rr = oracle.reference_root()
    if rr is None:
        pytest.skip("reference sources not available")
    r = subprocess.run(["sh", os.path.join(HERE, "refcompat", "link_reference.sh"), rr, ROOT,
                        str(tmp_path)], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    assert os.path.exists(tmp_path / "Pfmhzo_gb")
    nm = subprocess.run(["nm", "-C", str(tmp_path / "Pfmhzo_gb")], capture_output=True, text=True).stdout
    assert " T Evolve()" in nm and " T Depol_field()" in nm


@pytest.fixture(scope="module")
def driver(compat, tmp_path_factory):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    exe = tmp_path_factory.mktemp("drive") / "drive"
    subprocess.run(["nvcc", ARCH, "-std=c++17", os.path.join(HERE, "refcompat", "drive_evolve.cu"),
                    os.path.join(HERE, "refcompat", "globals_stub.cu"), compat.REFCOMPAT,
                    "-L" + os.path.join(ROOT, "cmsl_gb300"), "-lcmsl_gb", "-Xlinker",
                    "-rpath," + os.path.join(ROOT, "cmsl_gb300"), "-o", str(exe)], check=True)
    return str(exe)


MAXEZ, DELEZ, E0, P0 = 0.3, 0.05, 7.5e7, 0.35


def _setup(path, f, P):
    with open(path, "wb") as fh:
        fh.write(struct.pack("7i", f.nx, f.ny, f.nz, int(f.grain_mat.size), 1, 0, 1))
        fh.write(struct.pack("7d", f.del_h, f.del_t, f.eps_0_nd, MAXEZ, DELEZ, E0, P0))
        fh.write(np.asarray(f.mats, np.float64).tobytes())
        fh.write(np.asarray(f.omega, np.int32).tobytes())
        fh.write(np.asarray(f.grain_mat, np.int32).tobytes())
        fh.write(np.asarray(f.TR, np.float64).tobytes())
        fh.write(np.stack(P).astype(np.float64).tobytes())


def _drive(driver, tmp_path, f, P, mode):
    _setup(tmp_path / "setup.bin", f, P)
    out = tmp_path / "out"
    out.mkdir(exist_ok=True)
    r = subprocess.run([driver, str(tmp_path / "setup.bin"), str(out), str(tmp_path / "result.bin"), mode],
                       capture_output=True, text=True, timeout=900, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    return (tmp_path / "result.bin").read_bytes(), out


def _check_sweep(out, rE, stats, rc, offset, rtol=2e-6):
    lines = (out / "sweep001.txt").read_text().strip().splitlines()
    assert len(lines) == len(rE)
    for line, e, st, cnt in zip(lines, rE, stats, rc):
        got = [float(x) for x in line.split("\t")]
        want = [e * E0 / 1e8] + [st[i] * P0 * 100.0 if i in (0, 1, 2, 3, 4, 6, 8) else st[i] for i in range(10)]
        assert int(got[11]) == cnt + offset
        np.testing.assert_allclose(got[:11], want, rtol=rtol, atol=1e-12)


@pytest.mark.gpu
def test_evolve_through_compat_matches_oracle(driver, tmp_path):
    f, P = random_film(24, 16, 6, seed=61, eps_0_nd=3.0, p_scale=0.2)
    raw, out = _drive(driver, tmp_path, f, P, "evolve")
    N = f.N
    Pg = np.frombuffer(raw[: 48 * N], np.float64).reshape(6, N)
    count, peloop = struct.unpack("2i", raw[48 * N:])
    Ez, rows, rE, rc = fm.evolve_schedule(MAXEZ, DELEZ, 1)
    o = oracle.load()
    f.tol_abs, f.tol_rel = 1e-3, 1e-2
    Pw, _, _, stats, _, rcode = o.run(f, P, np.zeros(N), Ez, rows)
    assert rcode == 0 and peloop == 2 and count == len(Ez)
    for a, b in zip(Pg, Pw):
        assert np.abs(a - b).max() <= 1e-10 * max(np.abs(b).max(), 1e-300)
    _check_sweep(out, rE, stats, rc, 0)


def _read_slice(path, nx, ny):
    vals = np.zeros((ny, nx))
    n = 0
    for line in path.read_text().splitlines():
        if line.strip():
            i, j, v = line.split()
            vals[int(j), int(i)] = float(v)
            n += 1
    assert n == nx * ny
    return vals


@pytest.mark.gpu
def test_evolve_with_pre_relax_writes_slices(driver, tmp_path):
    """do_pre_relax = 1 (evolve.cu:171-211): 15000 steps at E = 0 before the
    loop, then slice_E0_midplane.dat (Psz of the relaxed state) and
    slice_E0_midplane_local.dat (Psz in the crystal frame of the state the
    last relaxation step started from), then the loop with the sweep counts
    shifted by 15000.  Against the oracle run the same way; with the
    reference's loose PCG tolerances (1e-3 / 1e-2) an iteration count can
    differ by one between the two solvers somewhere in 15000 solves, so the
    fields are held to 1e-6 of their maximum."""
    from cmsl_gb300 import workloads as wl
    o = oracle.load()
    # an HZO film with half its grains AFE: their Ps survives the relaxation
    w = wl.hzo_film("pre_relax_16x12x6", 16, 12, 6, 6, 5, 0.5)
    f = oracle.Film(nx=w.nx, ny=w.ny, nz=w.nz, del_h=w.del_h, del_t=w.del_t, omega=w.omega,
                    grain_mat=w.grain_mat, TR=w.TR, mats=w.mats,
                    is_interface=o.interface_flags(w.nx, w.ny, w.nz, w.omega, w.grain_mat),
                    dep_flag=1, eps_0_nd=w.eps_0_nd)
    P = w.P_init
    raw, out = _drive(driver, tmp_path, f, P, "pre")
    N, pre = f.N, 15000
    Pg = np.frombuffer(raw[: 48 * N], np.float64).reshape(6, N)
    count, peloop = struct.unpack("2i", raw[48 * N:])
    f.tol_abs, f.tol_rel = 1e-3, 1e-2
    Pa, Ea, phia, _, _, rcode = o.run(f, P, np.zeros(N), np.zeros(pre - 1))
    assert rcode == 0
    loc = fm.crystal_z(f.omega, f.TR, Pa[3], Pa[4], Pa[5])
    Pb, Eb, phib, _, _, rcode = o.run(f, Pa, phia, np.zeros(1), E=Ea)
    assert rcode == 0
    Ez, rows, rE, rc = fm.evolve_schedule(MAXEZ, DELEZ, 1)
    Pw, _, _, stats, _, rcode = o.run(f, Pb, phib, Ez, rows, E=Eb)
    assert rcode == 0 and peloop == 2 and count == pre + len(Ez)
    mid = slice(f.nx * f.ny * (f.nz // 2), f.nx * f.ny * (f.nz // 2 + 1))
    assert np.abs(Pb[5][mid]).max() > 0.1 and np.abs(loc[mid]).max() > 0.1
    got = _read_slice(tmp_path / "slice_E0_midplane.dat", f.nx, f.ny).ravel()
    assert np.abs(got - Pb[5][mid]).max() <= 1e-6 * np.abs(Pb[5]).max()
    got = _read_slice(tmp_path / "slice_E0_midplane_local.dat", f.nx, f.ny).ravel()
    assert np.abs(got - loc[mid]).max() <= 1e-6 * np.abs(loc).max()
    for a, b in zip(Pg, Pw):
        assert np.abs(a - b).max() <= 1e-6 * max(np.abs(b).max(), 1e-300)
    _check_sweep(out, rE, stats, rc, pre, rtol=1e-5)


@pytest.mark.gpu
def test_depol_field_in_place_matches_oracle(driver, tmp_path):
    """Depol_field() on the reference's device arrays, twice: the second call
    with a new Pm, warm-started from the first call's phi_dep_d, on the film
    kept from the first call.  phi and E against the oracle's Depol_field at
    the reference's tolerances."""
    f, P = random_film(24, 16, 6, seed=63, eps_0_nd=3.0, p_scale=0.2)
    raw, _ = _drive(driver, tmp_path, f, P, "depol")
    N = f.N
    got = np.frombuffer(raw, np.float64).reshape(2, 4, N)
    o = oracle.load()
    f.tol_abs, f.tol_rel = 1e-3, 1e-2
    phi = np.zeros(N)
    for call, scale in enumerate((1.0, 0.9)):
        Pm = [scale * P[q] for q in range(3)]
        phi, E, _, info = o.depol_field(f, Pm, phi)
        assert info["status"] == 0
        want = [phi] + list(E)
        for a, b in zip(got[call], want):
            assert np.abs(a - b).max() <= 1e-10 * max(np.abs(b).max(), 1e-300), call
