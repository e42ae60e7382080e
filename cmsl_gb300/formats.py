"""The reference's input formats and set-up steps (include/cmsl_io.h).

Thin ctypes wrappers: the work is done by libcmsl_gb's host code
(cmsl_gb300/csrc/formats.cpp), which a C or C++ caller uses directly.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, lib

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class Deck(C.Structure):
    """InputParams deck (HZO_Code_github/src/get_InputParams.cu:8-92)."""
    _fields_ = [(n, C.c_int) for n in ("device_flag", "nx", "ny", "nz", "dep_flag", "num_steps", "out_flag",
                                        "dimx", "dimy", "dimz")] + \
               [(n, C.c_double) for n in ("del_h", "del_t", "delEap", "Eap", "kappa_fe", "L_fe", "kappa_afe",
                                           "L_afe", "kappa_de", "L_de", "eps_fe", "eps_afe", "eps_de", "PsNoise",
                                           "G0", "omg")] + \
               [("do_pre_relax", C.c_int), ("n_layers", C.c_int), ("layer_counts", C.c_int * 16),
                ("crystal_type", C.c_char * 20), ("z_bc_type", C.c_char * 20)]

    def as_dict(self) -> dict:
        d = {n: getattr(self, n) for n, _ in self._fields_ if n not in ("layer_counts", "crystal_type", "z_bc_type")}
        d["layer_counts"] = list(self.layer_counts[: self.n_layers])
        d["crystal_type"] = self.crystal_type.decode()
        d["z_bc_type"] = self.z_bc_type.decode()
        return d


class LandauSet(C.Structure):
    _fields_ = [("afe", C.c_double * 5), ("fe", C.c_double * 5), ("de", C.c_double * 2), ("ref_type", C.c_int),
                ("frac_afe", C.c_double), ("frac_fe", C.c_double), ("frac_de", C.c_double)]


class RawMaterial(C.Structure):
    _fields_ = [("alpha", C.c_double), ("beta", C.c_double), ("gamma1", C.c_double), ("g", C.c_double),
                ("a0", C.c_double), ("transition_type", C.c_int), ("L", C.c_double), ("kappa", C.c_double),
                ("eps_r", C.c_double)]


class Scales(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("alpha_ref", "P0_ref", "L_ref", "kappa_ref", "f0_ref", "E0_ref",
                                          "eps_0_nd", "maxEz", "delEz")]


_bound = False


def _bind():
    global _bound
    if _bound:
        return lib()
    L = lib()
    from ._lib import Material
    L.cmsl_deck_read.argtypes = [C.c_char_p, C.POINTER(Deck)]
    L.cmsl_deck_write_summary.argtypes = [C.POINTER(Deck), C.c_char_p]
    L.cmsl_grain_count.argtypes = [C.c_char_p, C.POINTER(C.c_int)]
    L.cmsl_grain_read.argtypes = [C.c_char_p, C.c_char_p] + [C.c_int] * 4 + [_ip, _dp, _dp, _dp, _dp]
    L.cmsl_grain_write.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p] + [C.c_int] * 4 + [_ip, _dp, _dp, _dp]
    L.cmsl_tr_from_euler.argtypes = [C.c_int, _dp, _dp, _dp, _dp]
    L.cmsl_landau_pool_read.argtypes = [C.c_char_p, C.POINTER(LandauSet), C.c_int, C.POINTER(C.c_int)]
    L.cmsl_phase_pool_read.argtypes = [C.c_char_p, _dp, _dp, _dp, C.c_int, C.POINTER(C.c_int)]
    L.cmsl_nondim.argtypes = [C.POINTER(RawMaterial), C.c_int, C.c_double, C.c_double, C.POINTER(Material),
                              C.POINTER(Scales)]
    L.cmsl_assign_materials.argtypes = [C.c_int] * 4 + [_ip, _dp, C.c_int, C.POINTER(C.c_int), _dp, _dp, _dp, _ip]
    L.cmsl_interface_flags.argtypes = [C.c_int] * 3 + [_ip, _ip, _ip]
    L.cmsl_evolve_schedule.argtypes = [C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int,
                                       _dp, _ip, C.POINTER(C.c_int), _dp, _ip, C.POINTER(C.c_int)]
    L.cmsl_voronoi_columnar.argtypes = [C.c_int] * 4 + [C.c_uint64, _ip, _dp, _dp]
    L.cmsl_voronoi_columnar_gpu.argtypes = [C.c_int] * 4 + [C.c_uint64, _ip, _dp, _dp]
    L.cmsl_interface_flags_gpu.argtypes = [C.c_int] * 4 + [C.c_void_p] * 4
    L.cmsl_checkpoint_write.argtypes = [C.c_char_p] + [C.c_int] * 5 + [C.c_double, C.c_double, C.POINTER(_dp),
                                                                       C.POINTER(_dp)]
    L.cmsl_checkpoint_read.argtypes = [C.c_char_p] + [C.c_int] * 3 + [C.POINTER(C.c_int), C.POINTER(C.c_int),
                                                                      _dp, _dp, C.POINTER(_dp), C.POINTER(_dp)]
    L.cmsl_vector_field_write.argtypes = [C.c_char_p, _dp, _dp, _dp, C.c_longlong, C.c_double]
    L.cmsl_efield_host.argtypes = [C.c_int] * 3 + [C.c_double, C.c_int, _dp, _dp, _dp, _dp]
    L.cmsl_midplane_slice_write.argtypes = [C.c_char_p, _dp, C.c_int, C.c_int, C.c_int]
    L.cmsl_crystal_z.argtypes = [C.c_longlong, _ip, _dp, _dp, _dp, _dp, _dp]
    _bound = True
    return L


def _d(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def _i(a):
    return a.ctypes.data_as(_ip) if a is not None else None


def read_deck(path: str) -> dict:
    L = _bind()
    d = Deck()
    check(L.cmsl_deck_read(path.encode(), C.byref(d)))
    return d.as_dict()


def write_deck_summary(deck: dict, path: str) -> None:
    L = _bind()
    d = Deck()
    for n, _ in Deck._fields_:
        if n in deck and n not in ("layer_counts", "crystal_type", "z_bc_type"):
            setattr(d, n, deck[n])
    check(L.cmsl_deck_write_summary(C.byref(d), path.encode()))


def grain_count(path: str) -> int:
    L = _bind()
    n = C.c_int()
    check(L.cmsl_grain_count(path.encode(), C.byref(n)))
    return n.value


def read_grains(directory: str, tag: str, nx: int, ny: int, nz: int, ng: int):
    """-> omega [N] int32, eta [N], cent [ng,3], euler [ng,3], TR [9 ng]."""
    L = _bind()
    N = nx * ny * nz
    om, eta = np.zeros(N, np.int32), np.zeros(N)
    cent, eul, tr = np.zeros(3 * ng), np.zeros(3 * ng), np.zeros(9 * ng)
    check(L.cmsl_grain_read(directory.encode(), tag.encode(), nx, ny, nz, ng, _i(om), _d(eta), _d(cent), _d(eul),
                            _d(tr)))
    return om, eta, cent.reshape(ng, 3), eul.reshape(ng, 3), tr


def write_grains(directory: str, tag: str, gnumb_path: str | None, nx, ny, nz, omega, cent, euler, eta=None):
    L = _bind()
    om = np.ascontiguousarray(omega, np.int32)
    c = np.ascontiguousarray(cent, np.float64).reshape(-1)
    e = np.ascontiguousarray(euler, np.float64).reshape(-1)
    et = None if eta is None else np.ascontiguousarray(eta, np.float64)
    check(L.cmsl_grain_write(directory.encode(), tag.encode(), gnumb_path.encode() if gnumb_path else None,
                             nx, ny, nz, c.size // 3, _i(om), _d(et), _d(c), _d(e)))


def tr_from_euler(phi, theta, psi) -> np.ndarray:
    L = _bind()
    a = [np.ascontiguousarray(v, np.float64) for v in (phi, theta, psi)]
    out = np.zeros(9 * a[0].size)
    check(L.cmsl_tr_from_euler(a[0].size, _d(a[0]), _d(a[1]), _d(a[2]), _d(out)))
    return out


def read_landau_pool(path: str, max_sets: int = 2000) -> list[dict]:
    L = _bind()
    buf = (LandauSet * max_sets)()
    n = C.c_int()
    check(L.cmsl_landau_pool_read(path.encode(), buf, max_sets, C.byref(n)))
    out = []
    for s in buf[: n.value]:
        out.append({"afe": list(s.afe), "fe": list(s.fe), "de": list(s.de), "ref_type": s.ref_type,
                    "fractions": (s.frac_afe, s.frac_fe, s.frac_de) if s.frac_afe >= 0 else None})
    return out


def read_phase_pool(path: str, max_entries: int = 20000):
    L = _bind()
    a, f, d = (np.zeros(max_entries) for _ in range(3))
    n = C.c_int()
    check(L.cmsl_phase_pool_read(path.encode(), _d(a), _d(f), _d(d), max_entries, C.byref(n)))
    return a[: n.value], f[: n.value], d[: n.value]


def nondim(raw: list[dict], ref_type: int, Eap: float, delEap: float):
    """raw: three dicts (AFE, FE, DE) with alpha, beta, gamma1, g, a0, L, kappa,
    eps_r[, transition_type] -> (mats [3, 8], scales dict)."""
    L = _bind()
    from ._lib import Material
    r = (RawMaterial * 3)()
    for q in range(3):
        for k in ("alpha", "beta", "gamma1", "g", "a0", "L", "kappa", "eps_r"):
            setattr(r[q], k, float(raw[q].get(k, 0.0)))
        r[q].transition_type = int(raw[q].get("transition_type", 0))
    m = (Material * 3)()
    sc = Scales()
    check(L.cmsl_nondim(r, int(ref_type), float(Eap), float(delEap), m, C.byref(sc)))
    mats = np.array([[getattr(m[q], k) for k in ("alpha", "beta", "gamma", "g", "a0", "kappa", "L", "eps_r")]
                     for q in range(3)])
    return mats, {n: getattr(sc, n) for n, _ in Scales._fields_}


def assign_materials(nx, ny, nz, omega, centz, layer_counts, afe, fe, de) -> np.ndarray:
    L = _bind()
    om = np.ascontiguousarray(omega, np.int32)
    cz = np.ascontiguousarray(centz, np.float64)
    lc = (C.c_int * len(layer_counts))(*[int(v) for v in layer_counts])
    a, f, d = (np.ascontiguousarray(v, np.float64) for v in (afe, fe, de))
    out = np.zeros(cz.size, np.int32)
    check(L.cmsl_assign_materials(nx, ny, nz, cz.size, _i(om), _d(cz), len(layer_counts), lc, _d(a), _d(f), _d(d),
                                  _i(out)))
    return out


def interface_flags(nx, ny, nz, omega, grain_mat) -> np.ndarray:
    L = _bind()
    om = np.ascontiguousarray(omega, np.int32)
    gm = np.ascontiguousarray(grain_mat, np.int32)
    out = np.zeros(om.size, np.int32)
    check(L.cmsl_interface_flags(nx, ny, nz, _i(om), _i(gm), _i(out)))
    return out


def evolve_schedule(maxEz, delEz, num_steps, n_periods=1, single_crystal=False, E0_ref=1.0, max_steps=50_000_000):
    """C++ restatement of the Evolve schedule -> (Ez, rows, row_E, row_count)."""
    L = _bind()
    ns, nr = C.c_int(), C.c_int()
    check(L.cmsl_evolve_schedule(maxEz, delEz, num_steps, n_periods, int(single_crystal), E0_ref, max_steps, None,
                                 None, C.byref(ns), None, None, C.byref(nr)))
    Ez, rows = np.zeros(ns.value), np.zeros(ns.value, np.int32)
    rE, rc = np.zeros(max(nr.value, 1)), np.zeros(max(nr.value, 1), np.int32)
    check(L.cmsl_evolve_schedule(maxEz, delEz, num_steps, n_periods, int(single_crystal), E0_ref, max_steps, _d(Ez),
                                 _i(rows), C.byref(ns), _d(rE), _i(rc), C.byref(nr)))
    return Ez, rows, rE[: nr.value], rc[: nr.value]


def voronoi_columnar(nx, ny, nz, n_grains, seed, device=False):
    """-> omega [N], cent [ng, 3], euler [ng, 3]; device=True computes the map
    on the GPU (identical result)."""
    L = _bind()
    om = np.zeros(nx * ny * nz, np.int32)
    cent, eul = np.zeros(3 * n_grains), np.zeros(3 * n_grains)
    fn = L.cmsl_voronoi_columnar_gpu if device else L.cmsl_voronoi_columnar
    check(fn(nx, ny, nz, n_grains, int(seed), _i(om), _d(cent), _d(eul)))
    return om, cent.reshape(n_grains, 3), eul.reshape(n_grains, 3)


def _parr(arrs):
    return (_dp * len(arrs))(*[_d(a) for a in arrs])


def write_checkpoint(path: str, nx, ny, nz, P, E, peloop=0, count=0, Ez_ext=0.0, incEz=0.0) -> None:
    """The reference's checkpoint file (generate.cu:90-163)."""
    L = _bind()
    P = [np.ascontiguousarray(x, np.float64) for x in P]
    E = [np.ascontiguousarray(x, np.float64) for x in E]
    check(L.cmsl_checkpoint_write(path.encode(), nx, ny, nz, int(peloop), int(count), float(Ez_ext), float(incEz),
                                  _parr(P), _parr(E)))


def read_checkpoint(path: str, nx, ny, nz):
    """-> (P[6], E[3], peloop, count, Ez_ext, incEz) (generate.cu:165-264)."""
    L = _bind()
    N = nx * ny * nz
    P = [np.zeros(N) for _ in range(6)]
    E = [np.zeros(N) for _ in range(3)]
    pe, cnt = C.c_int(), C.c_int()
    ez, inc = np.zeros(1), np.zeros(1)
    check(L.cmsl_checkpoint_read(path.encode(), nx, ny, nz, C.byref(pe), C.byref(cnt), _d(ez), _d(inc), _parr(P),
                                 _parr(E)))
    return P, E, pe.value, cnt.value, float(ez[0]), float(inc[0])


def write_vector_field(path: str, Px, Py, Pz, scale=1.0) -> None:
    """write_vector_field_binary (generate.cu:11-30)."""
    L = _bind()
    a = [np.ascontiguousarray(x, np.float64) for x in (Px, Py, Pz)]
    check(L.cmsl_vector_field_write(path.encode(), _d(a[0]), _d(a[1]), _d(a[2]), a[0].size, float(scale)))


def efield(nx, ny, nz, del_h, zbc, phi):
    """E = -grad(phi) on the host (Calc_EfieldMag)."""
    L = _bind()
    phi = np.ascontiguousarray(phi, np.float64)
    E = [np.zeros(phi.size) for _ in range(3)]
    check(L.cmsl_efield_host(nx, ny, nz, float(del_h), int(zbc), _d(phi), _d(E[0]), _d(E[1]), _d(E[2])))
    return E


def write_midplane_slice(path: str, v, nx, ny, nz) -> None:
    """write_midplane_slice (generate.cu:67-88): plane nz/2 as "i j value" lines."""
    L = _bind()
    v = np.ascontiguousarray(v, np.float64)
    check(L.cmsl_midplane_slice_write(path.encode(), _d(v), int(nx), int(ny), int(nz)))


def crystal_z(omega, TR, x, y, z):
    """Crystal-frame z component per cell (kernelCalc_antiferro's *_local)."""
    L = _bind()
    om = np.ascontiguousarray(omega, np.int32)
    tr = np.ascontiguousarray(TR, np.float64)
    a = [np.ascontiguousarray(v, np.float64) for v in (x, y, z)]
    out = np.zeros(om.size)
    check(L.cmsl_crystal_z(om.size, om.ctypes.data_as(_ip), _d(tr), _d(a[0]), _d(a[1]), _d(a[2]), _d(out)))
    return out
