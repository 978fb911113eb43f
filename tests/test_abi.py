"""C ABI: the library loads, exports every declared entry point, and rejects bad input
before touching a GPU."""
import ctypes
import os
import re

import pytest

from gandalf_gb300 import _native
from gandalf_gb300.sph import GandalfError, GradhSphTree, make_config

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "gsph_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(gsph_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(native_lib):
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(native_lib, n), n
    assert set(names) == set(_native.SIGNATURES)


def test_abi_version_and_defaults(native_lib):
    assert native_lib.gsph_abi_version() == _native.ABI_VERSION == 3
    cfg = _native.Config()
    native_lib.gsph_config_defaults(ctypes.byref(cfg))
    assert cfg.ndim == 3 and cfg.nleafmax == 8 and cfg.h_fac == 1.2 and cfg.h_converge == 0.01
    assert cfg.alpha_visc == 1.0 and cfg.beta_visc == 2.0 and cfg.multipole == 1


@pytest.mark.parametrize("bad,code", [
    (dict(ndim=2), -3), (dict(nleafmax=0), -1), (dict(nleafmax=64), -1), (dict(eos=7), -3),
    (dict(self_gravity=1, periodic=1), -3), (dict(h_fac=0.0), -1), (dict(precision=5), -1),
    (dict(periodic=1, boxmin=(0, 0, 0), boxmax=(1, 0, 1)), -1)])
def test_create_rejects_bad_config(native_lib, bad, code):
    cfg = make_config(**bad)
    ctx = native_lib.gsph_create(ctypes.byref(cfg), 0)
    assert not ctx
    assert native_lib.gsph_create_error() == code


def test_create_without_gpu_fails_cleanly(native_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(GandalfError):
        GradhSphTree()
