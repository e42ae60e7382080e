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
