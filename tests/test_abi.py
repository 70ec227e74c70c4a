"""The C-ABI library builds, loads and exports every symbol its header
declares (no GPU calls)."""
import os
import re

from conftest import ROOT


def _declared():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            names += re.findall(r"^GRT_API\s+[\w\s\*]*?\b(\w+)\s*\(", src, re.M)
    return names


def test_header_declares_reference_entry_point():
    names = _declared()
    assert "green" in names and "grt_green" in names and "grt_run" in names


def test_library_exports_every_declared_symbol():
    import grtm_cuda_gb300 as g
    L = g.lib()
    for name in _declared():
        assert hasattr(L, name), name
    assert set(_declared()) <= set(g.EXPORTS) | set(_declared())


def test_status_strings_without_gpu():
    import grtm_cuda_gb300 as g
    assert g.lib().grt_status_string(0) == b"ok"
    assert g.lib().grt_status_string(g.ERR_MODEL) == b"unsupported layered model"
