"""Python handle over a libcmsl_gb film (numpy in, numpy out).

Mirrors the reference's per-simulation objects: the grain map and material
table a ``SetupAndRunSimulation`` call builds (HZO_Code_github/src/main.cu:
261-359) and the ``Evolve`` loop (src/evolve.cu:73-440) that advances it.
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np

from . import _lib
from ._lib import check, lib

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)

MAT_COLS = ("alpha", "beta", "gamma", "g", "a0", "kappa", "L", "eps_r")


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def pinned_empty(shape, dtype=np.float64):
    """An uninitialised numpy array in page-locked host memory
    (cmsl_host_alloc), freed with the array.  ``get_state(out=...)`` converts
    on the GPU straight into such arrays."""
    dt = np.dtype(dtype)
    n = int(np.prod(shape)) * dt.itemsize
    p = C.c_void_p()
    check(lib().cmsl_host_alloc(n, C.byref(p)))
    buf = (C.c_char * max(n, 1)).from_address(p.value)
    weakref.finalize(buf, lib().cmsl_host_free, C.c_void_p(p.value))
    return np.frombuffer(buf, dtype=dt, count=n // dt.itemsize).reshape(shape)


def _state_out(out, n):
    """(P, phi) output arrays: fresh ones, or the caller's ``out`` checked."""
    if out is None:
        return [np.zeros(n) for _ in range(6)], np.zeros(n)
    P, phi = out
    P = list(P)
    for a in P + [phi]:
        if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.size == n and a.flags.c_contiguous
                and a.flags.writeable):
            raise ValueError("out arrays must be writeable contiguous float64 arrays of %d cells" % n)
    if len(P) != 6:
        raise ValueError("out needs six P arrays")
    return P, phi


class _Desc:
    """A cmsl_film_desc with the arrays it points to kept alive."""

    def __init__(self, nx, ny, nz, omega, grain_mat, TR, mats, *, del_h, del_t, dep_flag=1,
                 zbc=_lib.DIRICHLET, eps_0_nd=0.0, is_interface=None, precision=_lib.FP64,
                 pcg_crit=_lib.CRIT_REF, tol_abs=1e-3, tol_rel=1e-2, max_iter=4000,
                 refine_tol=1e-8, max_refine=6, inner_tol=1e-4, inner_max_iter=2000, warm_start=2,
                 inner_solver=_lib.INNER_AUTO):
        self.nx, self.ny, self.nz = int(nx), int(ny), int(nz)
        self.N = self.nx * self.ny * self.nz
        self.precision = precision
        self._omega = np.ascontiguousarray(omega, np.int32)
        self._gm = np.ascontiguousarray(grain_mat, np.int32)
        self._tr = np.ascontiguousarray(TR, np.float64)
        self._fl = None if is_interface is None else np.ascontiguousarray(is_interface, np.int32)
        if self._omega.size != self.N:
            raise ValueError("omega has %d cells, grid has %d" % (self._omega.size, self.N))
        d = _lib.FilmDesc()
        d.nx, d.ny, d.nz = self.nx, self.ny, self.nz
        d.del_h, d.del_t = float(del_h), float(del_t)
        d.dep_flag, d.zbc, d.eps_0_nd = int(dep_flag), int(zbc), float(eps_0_nd)
        d.n_grains = int(self._gm.size)
        d.omega, d.grain_mat, d.TR = _i(self._omega), _i(self._gm), _d(self._tr)
        d.is_interface = _i(self._fl) if self._fl is not None else None
        m = np.asarray(mats, np.float64).reshape(3, 8)
        for q in range(3):
            for c, n in enumerate(MAT_COLS):
                setattr(d.mats[q], n, float(m[q, c]))
        d.precision, d.pcg_crit = int(precision), int(pcg_crit)
        d.tol_abs, d.tol_rel, d.max_iter = float(tol_abs), float(tol_rel), int(max_iter)
        d.refine_tol, d.max_refine = float(refine_tol), int(max_refine)
        d.inner_tol, d.inner_max_iter = float(inner_tol), int(inner_max_iter)
        d.warm_start = int(warm_start)
        d.inner_solver = int(inner_solver)
        self.d = d


def _oracle_kw(f):
    return dict(nx=f.nx, ny=f.ny, nz=f.nz, omega=f.omega, grain_mat=f.grain_mat, TR=f.TR, mats=f.mats,
                del_h=f.del_h, del_t=f.del_t, dep_flag=f.dep_flag, zbc=f.zbc, eps_0_nd=f.eps_0_nd,
                is_interface=f.is_interface, tol_abs=f.tol_abs, tol_rel=f.tol_rel, max_iter=f.max_iter,
                pcg_crit=f.crit)


def _tile_config(fn, h):
    cfg = (C.c_int32 * 4)()
    check(fn(h, cfg))
    names = ("cp.async ring", "tensor copies")
    return {"x": int(cfg[0]), "y": int(cfg[1]), "z_chunk": int(cfg[2]),
            "tdgl_staging": names[cfg[3] & 1], "residual_staging": names[(cfg[3] >> 2) & 1]}


class Film:
    """One film on the GPU.

    mats: [3, 8] array, rows AFE, FE, DE; columns alpha, beta, gamma, g, a0,
    kappa, L, eps_r (non-dimensional, as make_nd_wrt_reference gives them).
    """

    def __init__(self, nx, ny, nz, omega, grain_mat, TR, mats, **kw):
        L = lib()
        self._desc = _Desc(nx, ny, nz, omega, grain_mat, TR, mats, **kw)
        self.nx, self.ny, self.nz, self.N = self._desc.nx, self._desc.ny, self._desc.nz, self._desc.N
        self.precision = self._desc.precision
        h = C.c_void_p()
        check(L.cmsl_film_create(C.byref(self._desc.d), C.byref(h)))
        self._h = h
        self._n_rows = 0
        self._n_steps = 0

    @classmethod
    def from_oracle_film(cls, f, **kw):
        """Builds the GPU film for an oracle.Film description (tests, bench)."""
        return cls(**{**_oracle_kw(f), **kw})

    def close(self):
        if getattr(self, "_h", None):
            lib().cmsl_film_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- state -----------------------------------------------------------
    def set_state(self, P, phi=None):
        P = [np.ascontiguousarray(p, np.float64) for p in P]
        arr = (_dp * 6)(*[_d(p) for p in P])
        ph = None if phi is None else np.ascontiguousarray(phi, np.float64)
        check(lib().cmsl_film_set_state(self._h, arr, _d(ph) if ph is not None else None))

    def get_state(self, out=None):
        """(P, phi) as float64 arrays; ``out=(P, phi)`` fills the caller's
        arrays instead (page-locked ones from ``pinned_empty`` are written by
        the GPU directly)."""
        P, phi = _state_out(out, self.N)
        arr = (_dp * 6)(*[_d(p) for p in P])
        check(lib().cmsl_film_get_state(self._h, arr, _d(phi)))
        return P, phi

    # -- the P-E loop driver ----------------------------------------------
    def run(self, Ez, rows=None, stream=None, sync=True):
        Ez = np.ascontiguousarray(Ez, np.float64)
        n = int(Ez.size)
        r = None if rows is None else np.ascontiguousarray(rows, np.int32)
        check(lib().cmsl_film_run(self._h, n, _d(Ez), _i(r) if r is not None else None,
                                  C.c_void_p(stream) if stream else None))
        self._n_steps = n
        self._n_rows = int(r.max()) + 1 if r is not None and n and r.max() >= 0 else 0
        if sync:
            self.sync()

    def sync(self):
        check(lib().cmsl_film_sync(self._h))

    def rows(self, first=0, n=None):
        n = self._n_rows - first if n is None else n
        out = np.zeros((max(n, 0), 11))
        if n > 0:
            check(lib().cmsl_film_get_rows(self._h, first, n, _d(out)))
        return out

    def iters(self, n=None):
        n = self._n_steps if n is None else n
        it = np.zeros(max(n, 1), np.int32)
        rf = np.zeros(max(n, 1), np.int32)
        if n > 0:
            check(lib().cmsl_film_get_iters(self._h, n, _i(it), _i(rf)))
        return it[:n], rf[:n]

    # -- single pieces (parity tests) --------------------------------------
    def tdgl_step(self, Ez):
        check(lib().cmsl_film_tdgl_step(self._h, float(Ez)))

    def depol(self):
        it = np.zeros(2, np.int32)
        st = np.zeros(1, np.int32)
        check(lib().cmsl_film_depol(self._h, _i(it), _i(st)))
        return {"iters": int(it[0]), "refine": int(it[1]), "status": int(st[0])}

    def apply_operator(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(self.N)
        check(lib().cmsl_film_apply_operator(self._h, _d(x), _d(y)))
        return y

    def efield(self):
        E = [np.zeros(self.N) for _ in range(3)]
        check(lib().cmsl_film_efield(self._h, _d(E[0]), _d(E[1]), _d(E[2])))
        return E

    def diag_inv(self):
        y = np.zeros(self.N)
        check(lib().cmsl_film_diag_inv(self._h, _d(y)))
        return y

    def write_checkpoint(self, path, peloop=0, count=0, Ez_ext=0.0, incEz=0.0):
        """The reference's checkpoint file of the current state (P, E)."""
        check(lib().cmsl_film_checkpoint_write(self._h, str(path).encode(), int(peloop), int(count), float(Ez_ext),
                                               float(incEz)))

    def read_checkpoint(self, path):
        """Restart from a reference checkpoint file; returns its loop counters."""
        pe, cnt = C.c_int(), C.c_int()
        ez, inc = np.zeros(1), np.zeros(1)
        check(lib().cmsl_film_checkpoint_read(self._h, str(path).encode(), C.byref(pe), C.byref(cnt), _d(ez),
                                              _d(inc)))
        return {"peloop": pe.value, "count": cnt.value, "Ez_ext": float(ez[0]), "incEz": float(inc[0])}

    def loop_gradient(self, Ez, rows, target, checkpoint_every=200):
        """Loss (1/R) sum_r (<Pm_z>_r - target_r)^2 of the loop run from the
        current state, and its gradient [3, 5]: per material (AFE, FE, DE),
        d loss / d (alpha, beta, gamma, g, kappa) non-dimensional (adjoint of
        TDGL + PCG, cmsl_film_loop_gradient)."""
        Ez = np.ascontiguousarray(Ez, np.float64)
        r = np.ascontiguousarray(rows, np.int32)
        t = np.ascontiguousarray(target, np.float64)
        loss = np.zeros(1)
        grad = np.zeros(15)
        check(lib().cmsl_film_loop_gradient(self._h, int(Ez.size), _d(Ez), _i(r), _d(t), int(t.size),
                                            int(checkpoint_every), _d(loss), _d(grad)))
        return float(loss[0]), grad.reshape(3, 5)

    def time_kernels(self, reps=20, stream=None):
        """Average ms per launch of [tdgl, solve set-up, spmv, update]."""
        ms = np.zeros(4)
        check(lib().cmsl_film_time_kernels(self._h, int(reps), C.c_void_p(stream) if stream else None,
                                           _d(ms)))
        return ms

    def device_bytes(self):
        b = C.c_size_t()
        check(lib().cmsl_film_device_bytes(self._h, C.byref(b)))
        return int(b.value)

    @property
    def inner_solver(self):
        """INNER_DIRECT (spectral direct solve) or INNER_PCG."""
        v = C.c_int()
        check(lib().cmsl_film_inner_solver(self._h, C.byref(v)))
        return v.value

    def autotune(self):
        """Times the stencil passes for several work-item z chunks (and both
        stagings where tensor copies apply), keeps the fastest and returns
        the z chunk (cmsl_film_autotune)."""
        v = C.c_int32()
        check(lib().cmsl_film_autotune(self._h, C.byref(v)))
        return int(v.value)

    def tile_config(self):
        """The stencil passes' tile, z chunk and staging (cmsl_film_tile_config)."""
        return _tile_config(lib().cmsl_film_tile_config, self._h)


class Batch:
    """Many independent films on the GPU advancing together (cmsl_batch_*).

    films: a list of dicts of Film's constructor arguments (nx, ny, nz, omega,
    grain_mat, TR, mats, del_h, del_t, ...), one per film; all with the same
    precision.  The campaign loop of the reference (HZO_Code_github/src/
    main.cu:455-498) runs such films one after another.
    """

    def __init__(self, films):
        L = lib()
        self._descs = [_Desc(**f) for f in films]
        if not self._descs:
            raise ValueError("empty batch")
        self.n_films = len(self._descs)
        self.N = [d.N for d in self._descs]
        self.precision = self._descs[0].precision
        arr = (_lib.FilmDesc * self.n_films)(*[d.d for d in self._descs])
        self._arr = arr
        h = C.c_void_p()
        check(L.cmsl_batch_create(arr, self.n_films, C.byref(h)))
        self._h = h
        self._n_rows = 0
        self._n_steps = 0

    @classmethod
    def from_oracle_films(cls, films, **kw):
        return cls([{**_oracle_kw(f), **kw} for f in films])

    def close(self):
        if getattr(self, "_h", None):
            lib().cmsl_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_state(self, film, P, phi=None):
        P = [np.ascontiguousarray(p, np.float64) for p in P]
        if any(p.size != self.N[film] for p in P):
            raise ValueError("P of film %d needs %d cells" % (film, self.N[film]))
        arr = (_dp * 6)(*[_d(p) for p in P])
        ph = None if phi is None else np.ascontiguousarray(phi, np.float64)
        check(lib().cmsl_batch_set_state(self._h, int(film), arr, _d(ph) if ph is not None else None))

    def get_state(self, film, out=None):
        """Film ``film``'s (P, phi), as ``Film.get_state``."""
        P, phi = _state_out(out, self.N[film])
        arr = (_dp * 6)(*[_d(p) for p in P])
        check(lib().cmsl_batch_get_state(self._h, int(film), arr, _d(phi)))
        return P, phi

    def run(self, Ez, rows=None, stream=None, sync=True):
        """Ez, rows: [n_films, n_steps].  Returns the per-film PCG status when
        sync (raises CmslError only for errors other than a film's PCG failure)."""
        Ez = np.ascontiguousarray(Ez, np.float64)
        if Ez.ndim != 2 or Ez.shape[0] != self.n_films:
            raise ValueError("Ez must be [n_films, n_steps]")
        n = int(Ez.shape[1])
        r = None if rows is None else np.ascontiguousarray(rows, np.int32)
        if r is not None and r.shape != Ez.shape:
            raise ValueError("rows must have Ez's shape")
        check(lib().cmsl_batch_run(self._h, n, _d(Ez), _i(r) if r is not None else None,
                                   C.c_void_p(stream) if stream else None))
        self._n_steps = n
        self._n_rows = int(r.max()) + 1 if r is not None and n and r.max() >= 0 else 0
        if sync:
            return self.sync()

    def sync(self):
        st = np.zeros(self.n_films, np.int32)
        s = lib().cmsl_batch_sync(self._h, _i(st))
        if s not in (_lib.CMSL_OK, 4):
            check(s)
        return st

    def rows(self, film, first=0, n=None):
        n = self._n_rows - first if n is None else n
        out = np.zeros((max(n, 0), 11))
        if n > 0:
            check(lib().cmsl_batch_get_rows(self._h, int(film), first, n, _d(out)))
        return out

    def iters(self, film, n=None):
        n = self._n_steps if n is None else n
        it = np.zeros(max(n, 1), np.int32)
        rf = np.zeros(max(n, 1), np.int32)
        if n > 0:
            check(lib().cmsl_batch_get_iters(self._h, int(film), n, _i(it), _i(rf)))
        return it[:n], rf[:n]

    def time_kernels(self, reps=20, stream=None):
        ms = np.zeros(4)
        check(lib().cmsl_batch_time_kernels(self._h, int(reps), C.c_void_p(stream) if stream else None, _d(ms)))
        return ms

    @property
    def inner_solver(self):
        """INNER_DIRECT (spectral direct solve) or INNER_PCG."""
        v = C.c_int()
        check(lib().cmsl_batch_inner_solver(self._h, C.byref(v)))
        return v.value

    def autotune(self):
        """The batch's tile-shape autotuner (cmsl_batch_autotune); returns the z chunk."""
        v = C.c_int32()
        check(lib().cmsl_batch_autotune(self._h, C.byref(v)))
        return int(v.value)

    def tile_config(self):
        """The stencil passes' tile, z chunk and staging (cmsl_batch_tile_config)."""
        return _tile_config(lib().cmsl_batch_tile_config, self._h)

    def device_bytes(self):
        b = C.c_size_t()
        check(lib().cmsl_batch_device_bytes(self._h, C.byref(b)))
        return int(b.value)
