"""The C-ABI library loads (no GPU needed) and exports every entry point that
include/*.h declares; calls without a device fail with an error code, never
a crash."""
import glob
import os
import re

import pytest

from conftest import ROOT


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"\b(ember_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "ember_diffusion_integrate" in names and "ember_tridiag_step" in names


def test_library_exports_every_declared_symbol():
    from ember_gb300 import _lib
    lib = _lib.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared in include/*.h but not exported: {missing}"


def test_version_and_error_text():
    from ember_gb300 import _lib
    lib = _lib.lib()
    assert lib.ember_version() >= 100
    assert isinstance(_lib.last_error(), str)


def test_bad_arguments_are_rejected_without_device():
    import ctypes as C
    from ember_gb300 import _lib
    lib = _lib.lib()
    h = C.c_void_p()
    assert lib.ember_tridiag_create(0, None, C.byref(h)) == _lib.EINVAL
    assert "n_systems" in _lib.last_error()
    assert lib.ember_diffusion_integrate(0, None, 1, None, None, None, None, None, None, None, 0, None) \
        == _lib.EINVAL
    # entry points of the transport model, the split state and the tuning query
    assert lib.ember_transport_create(None, None, C.byref(h)) == _lib.EINVAL
    assert lib.ember_transport_eval(None, 1, 101325.0, 1e-5, None, None, None, 0, None) == _lib.EINVAL
    assert lib.ember_split_load_state(None, None, 0, None) == _lib.EINVAL
    assert lib.ember_split_set_transport_model(None, None, 1e-5, 1) == _lib.EINVAL
    assert lib.ember_mech_get_tuning(None, None, None, None, None, None, None) == _lib.EINVAL
    assert lib.ember_source_autotune(None, 0, 1, None, None, None, 0.0, None, None, None, None, 0, None) \
        == _lib.EINVAL
    assert lib.ember_convection_integrate(1, None, 10, None, None, None, None, None, None, None, None, None, 0,
                                          None) == _lib.EINVAL
    assert "null" in _lib.last_error()
    # the QSS adjoint: null mechanism, then missing arrays
    assert lib.ember_source_adjoint_qss(None, 1, None, None, None, 0.0, None, None, None, 0, None, None, None, None,
                                        0, None) == _lib.EINVAL
    assert "mechanism" in _lib.last_error()
    from ember_gb300.split import _lib as split_lib
    assert split_lib().ember_split_set_convection(None, None, None, None) == _lib.EINVAL
    assert lib.ember_math_eval(4, None, None, 1) == _lib.EINVAL
    assert lib.ember_math_eval(0, None, None, 1) == _lib.EINVAL
    assert lib.ember_math_eval(0, None, None, 0) == 0  # nothing to do: no device needed


def test_no_device_is_reported_not_crashed():
    from ember_gb300 import _lib
    lib = _lib.lib()
    if lib.ember_device_count() > 0:
        pytest.skip("a GPU is present")
    import numpy as np
    import ctypes as C
    off = np.array([0, 4], dtype=np.int64)
    h = C.c_void_p()
    rc = lib.ember_tridiag_create(1, off.ctypes.data_as(_lib.i64p), C.byref(h))
    assert rc == _lib.ECUDA
