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


@pytest.mark.gpu
def test_evolve_through_compat_matches_oracle(compat, tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    exe = tmp_path / "drive"
    subprocess.run(["nvcc", ARCH, "-std=c++17", os.path.join(HERE, "refcompat", "drive_evolve.cu"),
                    os.path.join(HERE, "refcompat", "globals_stub.cu"), compat.REFCOMPAT,
                    "-L" + os.path.join(ROOT, "cmsl_gb300"), "-lcmsl_gb", "-Xlinker",
                    "-rpath," + os.path.join(ROOT, "cmsl_gb300"), "-o", str(exe)], check=True)
    f, P = random_film(24, 16, 6, seed=61, eps_0_nd=3.0, p_scale=0.2)
    maxEz, delEz, E0, P0 = 0.3, 0.05, 7.5e7, 0.35
    with open(tmp_path / "setup.bin", "wb") as fh:
        fh.write(struct.pack("7i", f.nx, f.ny, f.nz, int(f.grain_mat.size), 1, 0, 1))
        fh.write(struct.pack("7d", f.del_h, f.del_t, f.eps_0_nd, maxEz, delEz, E0, P0))
        fh.write(np.asarray(f.mats, np.float64).tobytes())
        fh.write(np.asarray(f.omega, np.int32).tobytes())
        fh.write(np.asarray(f.grain_mat, np.int32).tobytes())
        fh.write(np.asarray(f.TR, np.float64).tobytes())
        fh.write(np.stack(P).astype(np.float64).tobytes())
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([str(exe), str(tmp_path / "setup.bin"), str(out), str(tmp_path / "final.bin")],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    raw = (tmp_path / "final.bin").read_bytes()
    N = f.N
    Pg = np.frombuffer(raw[: 48 * N], np.float64).reshape(6, N)
    count, peloop = struct.unpack("2i", raw[48 * N:])
    Ez, rows, rE, rc = fm.evolve_schedule(maxEz, delEz, 1)
    o = oracle.load()
    f.tol_abs, f.tol_rel = 1e-3, 1e-2
    Pw, _, _, stats, _, rcode = o.run(f, P, np.zeros(N), Ez, rows)
    assert rcode == 0 and peloop == 2 and count == len(Ez)
    for a, b in zip(Pg, Pw):
        assert np.abs(a - b).max() <= 1e-10 * max(np.abs(b).max(), 1e-300)
    lines = (out / "sweep001.txt").read_text().strip().splitlines()
    assert len(lines) == len(rE)
    for line, e, st, cnt in zip(lines, rE, stats, rc):
        got = [float(x) for x in line.split("\t")]
        want = [e * E0 / 1e8] + [st[i] * P0 * 100.0 if i in (0, 1, 2, 3, 4, 6, 8) else st[i] for i in range(10)]
        assert int(got[11]) == cnt
        np.testing.assert_allclose(got[:11], want, rtol=2e-6, atol=1e-12)
