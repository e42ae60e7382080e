"""CPU checks of the C ABI: the library builds, loads without a GPU and
exports every function include/cmsl.h declares."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header="cmsl.h"):
    txt = open(os.path.join(ROOT, "include", header)).read()
    decl = r"^\s*(?:cmsl_status|const char \*|void)\s*(cmsl_[a-z_0-9]+)\s*\("
    return sorted(set(re.findall(decl, txt, flags=re.M)))


def _all_declared():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            names += _declared(h)
    return sorted(set(names))


def test_header_and_binding_agree():
    from cmsl_gb300 import _lib
    assert _declared() == sorted(_lib.EXPORTS)


def test_io_header_functions_are_bound():
    from cmsl_gb300 import formats
    L = formats._bind()
    for name in _declared("cmsl_io.h"):
        assert getattr(L, name).argtypes is not None, name


def test_library_exports_every_symbol():
    from cmsl_gb300 import build, _lib
    build.build()
    L = _lib.lib()
    for name in _all_declared():
        assert hasattr(L, name), name
    assert b"sm_103a" in L.cmsl_version()


def test_create_rejects_bad_descriptors_without_gpu():
    """Argument checks run before any CUDA call."""
    import numpy as np
    import cmsl_gb300 as cg
    with pytest.raises(cg.CmslError) as e:
        cg.Film(4, 4, 2, np.zeros(32, np.int32), np.zeros(1, np.int32), np.eye(3).ravel(),
                np.zeros((3, 8)), del_h=0.5, del_t=1e-3)
    assert e.value.status == 1
    with pytest.raises(cg.CmslError):
        cg.Film(4, 4, 4, np.full(64, 3, np.int32), np.zeros(1, np.int32), np.eye(3).ravel(),
                np.zeros((3, 8)), del_h=0.5, del_t=1e-3)


def test_batch_rejects_bad_descriptors_without_gpu():
    """Batch argument checks (film index in the message, one precision for
    all films) run before any CUDA call."""
    import numpy as np
    import cmsl_gb300 as cg
    from cmsl_gb300 import _lib

    def film(**kw):
        d = dict(nx=4, ny=4, nz=4, omega=np.zeros(64, np.int32), grain_mat=np.ones(1, np.int32),
                 TR=np.eye(3).ravel(), mats=np.ones((3, 8)), del_h=0.5, del_t=1e-3)
        d.update(kw)
        return d
    with pytest.raises(cg.CmslError) as e:
        cg.Batch([film(), film(precision=cg.FP32_REFINED)])
    assert e.value.status == 1 and "film 1" in str(e.value)
    with pytest.raises(cg.CmslError) as e:
        cg.Batch([film(), film(), film(omega=np.full(64, 2, np.int32))])
    assert e.value.status == 1 and "film 2" in str(e.value)
    with pytest.raises(cg.CmslError) as e:
        cg.Batch([film(), film(nz=2, omega=np.zeros(32, np.int32))])
    assert "film 1" in str(e.value)
    h = _lib.C.c_void_p()
    assert _lib.lib().cmsl_batch_create(None, 1, _lib.C.byref(h)) == 1
    with pytest.raises(ValueError):
        cg.Batch([])


def test_state_out_arrays_checked_without_gpu():
    """get_state(out=...) validates the caller's arrays on the host (shape,
    dtype, contiguity, count) before any CUDA call; cmsl_host_alloc rejects a
    NULL out pointer, and cmsl_host_free(NULL) is a no-op."""
    import numpy as np
    from cmsl_gb300 import _lib
    from cmsl_gb300.film import _state_out
    n = 10
    P, phi = _state_out(None, n)
    assert len(P) == 6 and all(p.shape == (n,) and p.dtype == np.float64 for p in P) and phi.shape == (n,)
    ok = ([np.zeros(n) for _ in range(6)], np.zeros(n))
    P2, phi2 = _state_out(ok, n)
    assert P2[3] is ok[0][3] and phi2 is ok[1]
    bad = [([np.zeros(n)] * 5, np.zeros(n)),
           ([np.zeros(n)] * 6, np.zeros(n + 1)),
           ([np.zeros(n, np.float32)] * 6, np.zeros(n)),
           ([np.zeros(2 * n)[::2]] * 6, np.zeros(n))]
    ro = np.zeros(n)
    ro.flags.writeable = False
    bad.append(([ro] * 6, np.zeros(n)))
    for out in bad:
        with pytest.raises(ValueError):
            _state_out(out, n)
    L = _lib.lib()
    assert L.cmsl_host_alloc(16, None) == 1
    assert L.cmsl_host_free(None) == 0


def test_noalloc_argument_checks_without_gpu():
    """The allocation-free solve rejects grids it cannot tile before any CUDA
    call: a side above 32767 (the work items pack z ranges into 16 bits),
    more than 131072 cells, or nz < 3."""
    import ctypes as C
    import numpy as np
    from cmsl_gb300 import _lib
    L = _lib.lib()
    eps = (C.c_double * 3)(30.0, 30.0, 30.0)
    it = np.zeros(1, np.int32)
    st = np.zeros(1, np.int32)
    buf = np.zeros(8)
    p = C.c_void_p(buf.ctypes.data)
    ip = it.ctypes.data_as(C.POINTER(C.c_int32))
    sp = st.ctypes.data_as(C.POINTER(C.c_int32))
    for (nx, ny, nz), msg in (((1, 1, 70000), b"32767"), ((70000, 1, 3), b"32767"), ((1, 40000, 3), b"32767"),
                              ((128, 128, 16), b"131072"), ((4, 4, 2), b"nz >= 3")):
        rc = L.cmsl_depol_solve_noalloc(nx, ny, nz, 0.5, 0, 1.0, p, eps, p, p, p, p, 1e-3, 1e-2, 10, 0, None, ip, sp)
        assert rc == 1, (nx, ny, nz)
        assert msg in L.cmsl_last_error(), (nx, ny, nz, L.cmsl_last_error())
