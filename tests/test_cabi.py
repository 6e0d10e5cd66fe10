"""The C-ABI library builds, loads and exports every entry point of include/smuthi_gb300.h."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_symbols():
    src = open(os.path.join(ROOT, "include", "smuthi_gb300.h")).read()
    return sorted(set(re.findall(r"\b(sg_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from smuthi_gb300.build import build
    from smuthi_gb300 import _lib
    build()
    L = _lib.lib()
    syms = _header_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(L, s), s
    assert set(_lib.EXPORTS) == set(syms)
    assert b"sm_103a" in L.sg_version()


def test_no_device_is_an_error_not_a_fallback():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from smuthi_gb300 import _lib
    with pytest.raises(_lib.SmuthiGB300Error) as e:
        _lib.Context(0)
    assert e.value.code in (_lib.SG_ERR_NO_DEVICE, _lib.SG_ERR_CUDA)


def test_product_does_not_import_oracle():
    pkg = os.path.join(ROOT, "smuthi_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith(".py"):
                text = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in text and "from oracle" not in text, f
