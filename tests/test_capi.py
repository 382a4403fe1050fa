"""The C ABI library builds, loads and exports every symbol include/vxg.h
declares; without a GPU the product path fails loudly (no CPU fallback)."""

import re
from pathlib import Path

import pytest
import torch

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    text = (ROOT / "include" / "vxg.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(vxg_[a-z_0-9]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from voltax_gb300 import _lib, build
    build.build()
    return _lib.load()


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert "vxg_newton" in names and "vxg_factor" in names
    for name in names:
        assert hasattr(lib, name), name


def test_binding_covers_the_header():
    from voltax_gb300 import _lib
    assert set(declared_functions()) == set(_lib.exported_symbols())


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-GPU behaviour")
def test_no_cpu_fallback_without_gpu(lib):
    import voltax_gb300 as vx
    from voltax_gb300 import _lib, workloads
    with pytest.raises(_lib.VxgError, match="CUDA GPU"):
        vx.dc(workloads.power_grid(4))


def _zero(argtype):
    import ctypes as C
    if argtype in (C.c_double, C.c_float):
        return 0.0
    if isinstance(argtype, type) and issubclass(argtype, (C.c_int32, C.c_int64, C.c_uint64,
                                                          C.c_size_t)):
        return 0
    return None  # every pointer, handle and struct pointer


def test_every_entry_point_rejects_null_arguments(lib):
    """The boundary's error behaviour: each entry point checks its handle,
    sizes and buffers before anything reaches CUDA, so null / zero
    arguments return VXG_ERR_INVALID (no crash, no device call)."""
    from voltax_gb300 import _lib
    # no status to return; NULL is vxg_fused_set_profile's "off" argument
    skip = {"vxg_last_error", "vxg_launch_count", "vxg_fused_set_profile"}
    checked = 0
    for name, (argtypes, restype) in _lib.SIGNATURES.items():
        if name in skip:
            continue
        fn = getattr(lib, name)
        rc = fn(*[_zero(t) for t in argtypes])
        assert rc == _lib.VXG_ERR_INVALID, (name, rc)
        checked += 1
    assert checked == len(declared_functions()) - len(skip)
