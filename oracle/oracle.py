"""ctypes bindings of the oracle (``liboracle.so``) and of the reference-shim
library (``_ref/libcmsl_ref.so``).  Test infrastructure only."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
MAT_AFE, MAT_FE, MAT_DE = 0, 1, 2
DIRICHLET, NEUMANN = 0, 1
CRIT_REF, CRIT_RELRES = 0, 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class _Mat(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("alpha", "beta", "gamma", "g", "a0", "kappa", "L", "eps_r")]


class _Film(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("del_h", C.c_double), ("del_t", C.c_double),
        ("dep_flag", C.c_int), ("zbc", C.c_int), ("eps_0_nd", C.c_double),
        ("g_bot", C.c_double), ("g_top", C.c_double), ("ng", C.c_int),
        ("omega", _ip), ("grain_mat", _ip), ("TR", _dp), ("is_interface", _ip),
        ("mats", _Mat * 3), ("crit", C.c_int), ("tol_abs", C.c_double),
        ("tol_rel", C.c_double), ("max_iter", C.c_int),
    ]


class _PcgInfo(C.Structure):
    _fields_ = [("iters", C.c_int), ("status", C.c_int), ("rz0", C.c_double), ("rz", C.c_double),
                ("rr", C.c_double), ("bb", C.c_double)]


class _Raw(C.Structure):
    _fields_ = [("alpha", C.c_double), ("beta", C.c_double), ("gamma1", C.c_double),
                ("g", C.c_double), ("a0", C.c_double), ("transition_type", C.c_int),
                ("L", C.c_double), ("kappa", C.c_double), ("eps_r", C.c_double)]


class _Refs(C.Structure):
    _fields_ = [("alpha_ref", C.c_double), ("P0_ref", C.c_double), ("L_ref", C.c_double),
                ("kappa_ref", C.c_double)]


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _arr_d(arrs):
    return (_dp * len(arrs))(*[_d(a) for a in arrs])


@dataclass
class Film:
    """One film as the oracle sees it: grid, grain map and per-material
    non-dimensional parameters (rows: AFE, FE, DE; columns: alpha, beta, gamma,
    g, a0, kappa, L, eps_r)."""
    nx: int
    ny: int
    nz: int
    del_h: float
    del_t: float
    omega: np.ndarray
    grain_mat: np.ndarray
    TR: np.ndarray
    mats: np.ndarray
    is_interface: np.ndarray | None = None
    dep_flag: int = 1
    zbc: int = DIRICHLET
    eps_0_nd: float = 0.0
    crit: int = CRIT_REF
    tol_abs: float = 1.0e-3
    tol_rel: float = 1.0e-2
    max_iter: int = 4000
    _keep: list = field(default_factory=list, repr=False)

    @property
    def N(self) -> int:
        return self.nx * self.ny * self.nz

    def struct(self) -> _Film:
        om = np.ascontiguousarray(self.omega, dtype=np.int32)
        gm = np.ascontiguousarray(self.grain_mat, dtype=np.int32)
        tr = np.ascontiguousarray(self.TR, dtype=np.float64)
        fl = self.is_interface
        if fl is None:
            fl = np.zeros(self.N, np.int32)
        fl = np.ascontiguousarray(fl, dtype=np.int32)
        self._keep = [om, gm, tr, fl]
        s = _Film()
        s.nx, s.ny, s.nz = self.nx, self.ny, self.nz
        s.del_h, s.del_t = self.del_h, self.del_t
        s.dep_flag, s.zbc, s.eps_0_nd = int(self.dep_flag), int(self.zbc), float(self.eps_0_nd)
        s.g_bot = s.g_top = 0.0
        s.ng = int(gm.size)
        s.omega, s.grain_mat, s.TR, s.is_interface = _i(om), _i(gm), _d(tr), _i(fl)
        m = np.asarray(self.mats, dtype=np.float64).reshape(3, 8)
        for q in range(3):
            for c, n in enumerate(("alpha", "beta", "gamma", "g", "a0", "kappa", "L", "eps_r")):
                setattr(s.mats[q], n, float(m[q, c]))
        s.crit, s.tol_abs, s.tol_rel, s.max_iter = int(self.crit), self.tol_abs, self.tol_rel, int(self.max_iter)
        return s


# Where the reference sources lie: $CMSL_REFERENCE_ROOT, else the checkout
# this build was made against when it exists; None where neither does (the
# GPU machine), and everything that needs the sources skips.
_DEFAULT_REFERENCE_ROOT = "/root/reference"


def reference_root() -> str | None:
    """The reference checkout (the directory holding HZO_Code_github), or None."""
    for r in (os.environ.get("CMSL_REFERENCE_ROOT"), _DEFAULT_REFERENCE_ROOT):
        if r and os.path.isdir(os.path.join(r, "HZO_Code_github", "src")):
            return r
    return None


def build() -> str:
    """Builds liboracle.so with the committed Makefile; returns its path."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return os.path.join(HERE, "liboracle.so")


def build_ref(reference_root: str | None = None) -> str | None:
    """Builds _ref/libcmsl_ref.so from the reference sources when present."""
    reference_root = reference_root or reference_root_or_none()
    if not reference_root or not os.path.isdir(os.path.join(reference_root, "HZO_Code_github", "src")):
        return None
    subprocess.run(["sh", os.path.join(HERE, "build_ref.sh"), reference_root], check=True,
                   stdout=subprocess.DEVNULL)
    return os.path.join(HERE, "_ref", "libcmsl_ref.so")


def stage_ref_gpu(reference_root: str | None = None) -> bool:
    """Copies the reference program's sources (three mechanical fixes for
    CUDA 13) into baseline/_ref/hzo for building on a GPU machine
    (oracle/ref_gpu.sh stage); False when the sources are absent."""
    reference_root = reference_root or reference_root_or_none()
    if not reference_root:
        return False
    subprocess.run(["sh", os.path.join(HERE, "ref_gpu.sh"), "stage", reference_root], check=True,
                   stdout=subprocess.DEVNULL)
    return True


class OracleLib:
    def __init__(self, path: str):
        self.lib = L = C.CDLL(path)
        L.orc_tdgl_step.argtypes = [C.POINTER(_Film), C.POINTER(_dp), C.POINTER(_dp), C.c_double,
                                    C.POINTER(_dp), C.POINTER(_dp)]
        L.orc_divergence.argtypes = [C.POINTER(_Film), _dp, _dp, _dp, _dp]
        L.orc_apply_A.argtypes = [C.POINTER(_Film), _dp, _dp]
        L.orc_diag_inv.argtypes = [C.POINTER(_Film), _dp]
        L.orc_efield.argtypes = [C.POINTER(_Film), _dp, _dp, _dp, _dp]
        L.orc_eps_field.argtypes = [C.POINTER(_Film), _dp]
        L.orc_depol_field.argtypes = [C.POINTER(_Film), _dp, _dp, _dp, _dp, C.POINTER(_dp), _dp,
                                      C.POINTER(_PcgInfo)]
        L.orc_pcg.argtypes = [C.POINTER(_Film), _dp, _dp, C.POINTER(_PcgInfo)]
        L.orc_sweep_stats.argtypes = [C.POINTER(_Film), _dp, _dp, _dp, _dp, _dp]
        L.orc_run.argtypes = [C.POINTER(_Film), C.POINTER(_dp), C.POINTER(_dp), _dp, C.c_int,
                              _dp, _ip, _dp, _ip]
        L.orc_run.restype = C.c_int
        L.orc_compute_p0.argtypes = [C.c_double] * 4 + [C.c_int]
        L.orc_compute_p0.restype = C.c_double
        L.orc_make_phase_refs.argtypes = [_Raw]
        L.orc_make_phase_refs.restype = _Refs
        L.orc_make_nd.argtypes = [_Raw, _Refs, C.c_double, C.c_double]
        L.orc_make_nd.restype = _Mat
        L.orc_assign_materials.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _ip, _dp, C.c_int,
                                           C.POINTER(C.c_int), _dp, _dp, _dp, _ip]
        L.orc_assign_materials.restype = C.c_int
        L.orc_interface_flags.argtypes = [C.c_int, C.c_int, C.c_int, _ip, _ip, _ip]
        L.orc_tr_from_euler.argtypes = [C.c_int, _dp, _dp, _dp, _dp]

    # -- kernels --------------------------------------------------------
    def tdgl_step(self, film: Film, P, Ez: float, E=None, want_local=True):
        s = film.struct()
        P = [np.ascontiguousarray(p, np.float64) for p in P]
        Pn = [p.copy() for p in P]
        loc = [np.zeros(film.N) for _ in range(6)] if want_local else None
        Ea = [np.ascontiguousarray(e, np.float64) for e in E] if E is not None else [np.zeros(film.N)] * 3
        self.lib.orc_tdgl_step(C.byref(s), _arr_d(P), _arr_d(Pn), Ez, _arr_d(Ea),
                               _arr_d(loc) if loc else None)
        return Pn, loc

    def divergence(self, film: Film, Pmx, Pmy, Pmz):
        s = film.struct()
        a = [np.ascontiguousarray(x, np.float64) for x in (Pmx, Pmy, Pmz)]
        out = np.zeros(film.N)
        self.lib.orc_divergence(C.byref(s), _d(a[0]), _d(a[1]), _d(a[2]), _d(out))
        return out

    def apply_A(self, film: Film, x):
        s = film.struct()
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(film.N)
        self.lib.orc_apply_A(C.byref(s), _d(x), _d(y))
        return y

    def diag_inv(self, film: Film):
        s = film.struct()
        y = np.zeros(film.N)
        self.lib.orc_diag_inv(C.byref(s), _d(y))
        return y

    def efield(self, film: Film, phi):
        s = film.struct()
        phi = np.ascontiguousarray(phi, np.float64)
        E = [np.zeros(film.N) for _ in range(3)]
        self.lib.orc_efield(C.byref(s), _d(phi), _d(E[0]), _d(E[1]), _d(E[2]))
        return E

    def eps_field(self, film: Film):
        s = film.struct()
        y = np.zeros(film.N)
        self.lib.orc_eps_field(C.byref(s), _d(y))
        return y

    def depol_field(self, film: Film, Pm, phi):
        s = film.struct()
        Pm = [np.ascontiguousarray(x, np.float64) for x in Pm]
        phi = np.array(phi, np.float64, copy=True)
        E = [np.zeros(film.N) for _ in range(3)]
        div = np.zeros(film.N)
        info = _PcgInfo()
        self.lib.orc_depol_field(C.byref(s), _d(Pm[0]), _d(Pm[1]), _d(Pm[2]), _d(phi), _arr_d(E),
                                 _d(div), C.byref(info))
        return phi, E, div, {"iters": info.iters, "status": info.status, "rz0": info.rz0,
                             "rz": info.rz, "rr": info.rr, "bb": info.bb}

    def pcg(self, film: Film, b, x0):
        s = film.struct()
        b = np.ascontiguousarray(b, np.float64)
        x = np.array(x0, np.float64, copy=True)
        info = _PcgInfo()
        self.lib.orc_pcg(C.byref(s), _d(b), _d(x), C.byref(info))
        return x, {"iters": info.iters, "status": info.status, "rz0": info.rz0, "rz": info.rz,
                   "rr": info.rr, "bb": info.bb}

    def sweep_stats(self, film: Film, Pmz, Psz, Pmz_loc, Psz_loc):
        s = film.struct()
        a = [np.ascontiguousarray(x, np.float64) for x in (Pmz, Psz, Pmz_loc, Psz_loc)]
        out = np.zeros(11)
        self.lib.orc_sweep_stats(C.byref(s), _d(a[0]), _d(a[1]), _d(a[2]), _d(a[3]), _d(out))
        return out

    def run(self, film: Film, P, phi, Ez, rows=None, E=None):
        """Runs len(Ez) steps; returns (P, E, phi, stats[n_rows, 11], pcg_iters, rc)."""
        s = film.struct()
        P = [np.array(p, np.float64, copy=True) for p in P]
        E = [np.zeros(film.N) for _ in range(3)] if E is None else [np.array(e, np.float64, copy=True) for e in E]
        phi = np.array(phi, np.float64, copy=True)
        Ez = np.ascontiguousarray(Ez, np.float64)
        n = int(Ez.size)
        rows = np.full(n, -1, np.int32) if rows is None else np.ascontiguousarray(rows, np.int32)
        nrow = int(rows.max()) + 1 if n and rows.max() >= 0 else 0
        stats = np.zeros((max(nrow, 1), 11))
        iters = np.zeros(max(n, 1), np.int32)
        rc = self.lib.orc_run(C.byref(s), _arr_d(P), _arr_d(E), _d(phi), n, _d(Ez), _i(rows),
                              _d(stats), _i(iters))
        return P, E, phi, stats[:nrow], iters[:n], rc

    # -- set-up ---------------------------------------------------------
    def compute_p0(self, a, b, g, c, tt=0):
        return self.lib.orc_compute_p0(a, b, g, c, tt)

    def make_nd(self, raw: dict, ref_raw: dict, t0=3.0e-9, l0=1.0e-9):
        def mk(d):
            r = _Raw()
            for k in ("alpha", "beta", "gamma1", "g", "a0", "L", "kappa", "eps_r"):
                setattr(r, k, float(d.get(k, 0.0)))
            r.transition_type = int(d.get("transition_type", 0))
            return r
        refs = self.lib.orc_make_phase_refs(mk(ref_raw))
        m = self.lib.orc_make_nd(mk(raw), refs, t0, l0)
        return (np.array([m.alpha, m.beta, m.gamma, m.g, m.a0, m.kappa, m.L, m.eps_r]),
                (refs.alpha_ref, refs.P0_ref))

    def assign_materials(self, nx, ny, nz, omega, centz, layer_counts, afe, fe, de):
        om = np.ascontiguousarray(omega, np.int32)
        cz = np.ascontiguousarray(centz, np.float64)
        nl = len(layer_counts)
        lc = (C.c_int * nl)(*[int(v) for v in layer_counts])
        a, f, d = (np.ascontiguousarray(v, np.float64) for v in (afe, fe, de))
        out = np.zeros(cz.size, np.int32)
        rc = self.lib.orc_assign_materials(nx, ny, nz, cz.size, _i(om), _d(cz), nl, lc, _d(a), _d(f),
                                           _d(d), _i(out))
        return out, rc

    def interface_flags(self, nx, ny, nz, omega, grain_mat):
        om = np.ascontiguousarray(omega, np.int32)
        gm = np.ascontiguousarray(grain_mat, np.int32)
        out = np.zeros(om.size, np.int32)
        self.lib.orc_interface_flags(nx, ny, nz, _i(om), _i(gm), _i(out))
        return out

    def tr_from_euler(self, phi, theta, psi):
        a = [np.ascontiguousarray(v, np.float64) for v in (phi, theta, psi)]
        out = np.zeros(9 * a[0].size)
        self.lib.orc_tr_from_euler(a[0].size, _d(a[0]), _d(a[1]), _d(a[2]), _d(out))
        return out


class RefLib:
    """The reference's own kernels compiled for the host (oracle/_ref)."""

    def __init__(self, path: str):
        self.lib = L = C.CDLL(path)
        L.ref_tdgl_step.argtypes = [C.c_int] * 4 + [C.POINTER(_dp), C.POINTER(_dp), _ip, _dp,
                                                    C.POINTER(_dp), C.c_double, C.c_double,
                                                    C.POINTER(_dp), C.c_int, C.c_double,
                                                    C.POINTER(_dp), _ip]
        L.ref_divergence.argtypes = [C.c_int] * 3 + [_dp] * 3 + [C.c_double, C.c_double, _dp]
        L.ref_apply_A.argtypes = [C.c_int] * 4 + [_dp, _dp, C.c_double, _dp]
        L.ref_diag_inv.argtypes = [C.c_int] * 4 + [_dp, C.c_double, _dp]
        L.ref_efield.argtypes = [C.c_int] * 4 + [_dp, C.c_double, _dp, _dp, _dp]
        L.ref_interface_flag.argtypes = [C.c_int] * 3 + [_ip, _ip, _ip]
        L.ref_mat_mask.argtypes = [_dp, _ip, _ip, _dp, _dp, C.c_int, C.c_int]
        L.ref_compute_p0.argtypes = [C.c_double] * 4 + [C.c_int]
        L.ref_compute_p0.restype = C.c_double
        L.ref_make_nd.argtypes = [_dp, _dp, _dp, _dp]
        L.ref_read_deck.argtypes = [C.c_char_p, C.c_char_p, _ip, _dp, C.c_char_p, _ip]
        L.ref_load_grain.argtypes = [C.c_char_p, C.c_char_p] + [C.c_int] * 4 + [_ip, _dp, _dp, _dp, _dp]
        L.ref_assign_materials.argtypes = [C.c_int] * 4 + [_ip, _dp, C.c_int, _ip, _dp, _dp, _dp, _ip]
        L.ref_depol_field.argtypes = [C.c_int] * 4 + [_dp] * 4 + [C.c_double, C.c_double, _dp, _dp,
                                                                  _dp, _dp, C.c_double, C.c_double,
                                                                  C.c_int, _ip]
        L.ref_write_checkpoint.argtypes = [C.c_char_p, C.POINTER(_dp), C.POINTER(_dp)] + [C.c_int] * 3 + [
            C.c_double, C.c_int, C.c_int, C.c_double]
        L.ref_read_checkpoint.argtypes = [C.c_char_p, C.POINTER(_dp), C.POINTER(_dp)] + [C.c_int] * 3 + [
            _ip, _ip, _dp, _dp]
        L.ref_write_vector_field.argtypes = [C.c_char_p, _dp, _dp, _dp] + [C.c_int] * 3 + [C.c_double]
        L.ref_write_midplane_slice.argtypes = [C.c_char_p, _dp] + [C.c_int] * 3

    @staticmethod
    def per_voxel(film: Film):
        """The reference's eight per-voxel parameter arrays (InitConfKernel)."""
        m = np.asarray(film.mats, np.float64).reshape(3, 8)
        mat = np.asarray(film.grain_mat, np.int32)[np.asarray(film.omega, np.int64)]
        return [np.ascontiguousarray(m[mat, c]) for c in range(8)]

    def tdgl_step(self, film: Film, P, Ez: float, E=None):
        prm = self.per_voxel(film)
        P = [np.ascontiguousarray(p, np.float64) for p in P]
        Pn = [p.copy() for p in P]
        loc = [np.zeros(film.N) for _ in range(6)]
        Ea = [np.ascontiguousarray(e, np.float64) for e in E] if E is not None else [np.zeros(film.N)] * 3
        om = np.ascontiguousarray(film.omega, np.int32)
        fl = film.is_interface if film.is_interface is not None else np.zeros(film.N, np.int32)
        fl = np.ascontiguousarray(fl, np.int32)
        tr = np.ascontiguousarray(film.TR, np.float64)
        # kernel parameter order: alpha, beta, gamma, g, a0, kappa, L
        order = [prm[0], prm[1], prm[2], prm[3], prm[4], prm[5], prm[6]]
        self.lib.ref_tdgl_step(film.nx, film.ny, film.nz, int(np.asarray(film.grain_mat).size),
                               _arr_d(P), _arr_d(Pn), _i(om), _d(tr), _arr_d(order), film.del_h,
                               film.del_t, _arr_d(Ea), int(film.dep_flag), Ez, _arr_d(loc), _i(fl))
        return Pn, loc

    def divergence(self, film: Film, Pmx, Pmy, Pmz):
        a = [np.ascontiguousarray(x, np.float64) for x in (Pmx, Pmy, Pmz)]
        out = np.zeros(film.N)
        self.lib.ref_divergence(film.nx, film.ny, film.nz, _d(a[0]), _d(a[1]), _d(a[2]), film.del_h,
                                film.eps_0_nd, _d(out))
        return out

    def apply_A(self, film: Film, x):
        eps = self.per_voxel(film)[7]
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(film.N)
        self.lib.ref_apply_A(film.nx, film.ny, film.nz, int(film.zbc), _d(x), _d(eps), film.del_h, _d(y))
        return y

    def diag_inv(self, film: Film):
        eps = self.per_voxel(film)[7]
        y = np.zeros(film.N)
        self.lib.ref_diag_inv(film.nx, film.ny, film.nz, int(film.zbc), _d(eps), film.del_h, _d(y))
        return y

    def efield(self, film: Film, phi):
        phi = np.ascontiguousarray(phi, np.float64)
        E = [np.zeros(film.N) for _ in range(3)]
        self.lib.ref_efield(film.nx, film.ny, film.nz, int(film.zbc), _d(phi), film.del_h, _d(E[0]),
                            _d(E[1]), _d(E[2]))
        return E

    def interface_flags(self, nx, ny, nz, omega, grain_mat):
        om = np.ascontiguousarray(omega, np.int32)
        gm = np.ascontiguousarray(grain_mat, np.int32)
        out = np.zeros(om.size, np.int32)
        self.lib.ref_interface_flag(nx, ny, nz, _i(om), _i(gm), _i(out))
        return out

    def mat_mask(self, Pmz, omega, grain_mat, target):
        Pmz = np.ascontiguousarray(Pmz, np.float64)
        om = np.ascontiguousarray(omega, np.int32)
        gm = np.ascontiguousarray(grain_mat, np.int32)
        pm, mk = np.zeros(Pmz.size), np.zeros(Pmz.size)
        self.lib.ref_mat_mask(_d(Pmz), _i(om), _i(gm), _d(pm), _d(mk), Pmz.size, target)
        return pm, mk

    def compute_p0(self, a, b, g, c, tt=0):
        return self.lib.ref_compute_p0(a, b, g, c, tt)

    def make_nd(self, raw: dict, ref_raw: dict):
        def vec(d):
            return np.array([d.get("alpha", 0.0), d.get("beta", 0.0), d.get("gamma1", 0.0),
                             d.get("g", 0.0), d.get("a0", 0.0), d.get("transition_type", 0),
                             d.get("L", 0.0), d.get("kappa", 0.0), d.get("eps_r", 0.0)], np.float64)
        out, refs = np.zeros(8), np.zeros(2)
        a, b = vec(raw), vec(ref_raw)
        self.lib.ref_make_nd(_d(a), _d(b), _d(out), _d(refs))
        return out, (refs[0], refs[1])

    def read_deck(self, path: str, out_path: str):
        ints = np.zeros(10, np.int32)
        dbl = np.zeros(13)
        strs = C.create_string_buffer(40)
        lc = np.zeros(16, np.int32)
        self.lib.ref_read_deck(path.encode(), out_path.encode(), _i(ints), _d(dbl), strs, _i(lc))
        raw = strs.raw
        return {
            "nx": int(ints[0]), "ny": int(ints[1]), "nz": int(ints[2]), "dep_flag": int(ints[3]),
            "num_steps": int(ints[4]), "dimx": int(ints[5]), "dimy": int(ints[6]), "dimz": int(ints[7]),
            "n_layers": int(ints[8]), "do_pre_relax": int(ints[9]),
            "del_h": dbl[0], "del_t": dbl[1], "delEap": dbl[2], "Eap": dbl[3],
            "kappa_fe": dbl[4], "L_fe": dbl[5], "kappa_afe": dbl[6], "L_afe": dbl[7],
            "kappa_de": dbl[8], "L_de": dbl[9], "eps_fe": dbl[10], "eps_afe": dbl[11], "eps_de": dbl[12],
            "crystal_type": raw[:20].split(b"\0")[0].decode(),
            "z_bc_type": raw[20:40].split(b"\0")[0].decode(),
            "layer_counts": [int(v) for v in lc[: int(ints[8])]],
        }

    def load_grain(self, d: str, tag: str, nx, ny, nz, ng):
        N = nx * ny * nz
        om, eta = np.zeros(N, np.int32), np.zeros(N)
        tr, cent, eul = np.zeros(9 * ng), np.zeros(3 * ng), np.zeros(3 * ng)
        self.lib.ref_load_grain(d.encode(), tag.encode(), nx, ny, nz, ng, _i(om), _d(eta), _d(tr),
                                _d(cent), _d(eul))
        return om, eta, tr, cent.reshape(ng, 3), eul.reshape(ng, 3)

    def assign_materials(self, nx, ny, nz, omega, centz, layer_counts, afe, fe, de):
        om = np.ascontiguousarray(omega, np.int32)
        cz = np.ascontiguousarray(centz, np.float64)
        lc = np.ascontiguousarray(layer_counts, np.int32)
        a, f, d = (np.ascontiguousarray(v, np.float64) for v in (afe, fe, de))
        out = np.zeros(cz.size, np.int32)
        self.lib.ref_assign_materials(nx, ny, nz, cz.size, _i(om), _d(cz), lc.size, _i(lc), _d(a), _d(f),
                                      _d(d), _i(out))
        return out

    def write_checkpoint(self, path: str, P, E, nx, ny, nz, Ez_ext, peloop, count, incEz):
        """generate.cu write_checkpoint on host arrays."""
        P = [np.ascontiguousarray(x, np.float64) for x in P]
        E = [np.ascontiguousarray(x, np.float64) for x in E]
        self.lib.ref_write_checkpoint(path.encode(), _arr_d(P), _arr_d(E), nx, ny, nz, float(Ez_ext), int(peloop),
                                      int(count), float(incEz))

    def read_checkpoint(self, path: str, nx, ny, nz):
        """generate.cu read_checkpoint -> (P[6], E[3], peloop, count, Ez_ext, incEz)."""
        N = nx * ny * nz
        P = [np.zeros(N) for _ in range(6)]
        E = [np.zeros(N) for _ in range(3)]
        pe, cnt = np.zeros(1, np.int32), np.zeros(1, np.int32)
        ez, inc = np.zeros(1), np.zeros(1)
        self.lib.ref_read_checkpoint(path.encode(), _arr_d(P), _arr_d(E), nx, ny, nz, _i(pe), _i(cnt), _d(ez),
                                     _d(inc))
        return P, E, int(pe[0]), int(cnt[0]), float(ez[0]), float(inc[0])

    def write_vector_field(self, path: str, Px, Py, Pz, nx, ny, nz, p0):
        """generate.cu write_vector_field_binary."""
        a = [np.ascontiguousarray(x, np.float64) for x in (Px, Py, Pz)]
        self.lib.ref_write_vector_field(path.encode(), _d(a[0]), _d(a[1]), _d(a[2]), nx, ny, nz, float(p0))

    def write_midplane_slice(self, path: str, v, nx, ny, nz):
        """generate.cu write_midplane_slice."""
        v = np.ascontiguousarray(v, np.float64)
        self.lib.ref_write_midplane_slice(path.encode(), _d(v), nx, ny, nz)

    def depol_field(self, film: Film, Pm, phi, tol_abs=1e-3, tol_rel=1e-2, max_iter=4000):
        eps = self.per_voxel(film)[7]
        Pm = [np.ascontiguousarray(x, np.float64) for x in Pm]
        phi = np.array(phi, np.float64, copy=True)
        E = [np.zeros(film.N) for _ in range(3)]
        it = np.zeros(1, np.int32)
        self.lib.ref_depol_field(film.nx, film.ny, film.nz, int(film.zbc), _d(eps), _d(Pm[0]),
                                 _d(Pm[1]), _d(Pm[2]), film.del_h, film.eps_0_nd, _d(phi), _d(E[0]),
                                 _d(E[1]), _d(E[2]), tol_abs, tol_rel, max_iter, _i(it))
        return phi, E, int(it[0])


_cache: dict = {}


def load(rebuild: bool = False) -> OracleLib:
    path = os.path.join(HERE, "liboracle.so")
    if rebuild or not os.path.exists(path):
        build()
    if path not in _cache:
        _cache[path] = OracleLib(path)
    return _cache[path]


def reference_root_or_none() -> str | None:
    return reference_root()


def load_ref(reference_root: str | None = None) -> RefLib | None:
    path = os.path.join(HERE, "_ref", "libcmsl_ref.so")
    if not os.path.exists(path):
        if build_ref(reference_root) is None:
            return None
    if path not in _cache:
        _cache[path] = RefLib(path)
    return _cache[path]
