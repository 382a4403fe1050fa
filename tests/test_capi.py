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
