"""CPU tests of the C ABI boundary: the library loads, exports every declared
symbol, and fails loudly (no CPU fallback) when no GB300 is present."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for hdr in os.listdir(os.path.join(ROOT, "include")):
        if hdr.endswith(".h"):
            text = open(os.path.join(ROOT, "include", hdr)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(cbx_[a-z0-9_]+)\s*\(", text))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    assert {"cbx_create", "cbx_destroy", "cbx_grm_bed", "cbx_bed_snp_counts"} <= names


def test_library_exports_every_declared_symbol(built_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (cbx_[a-z0-9_]+)\b", out))
    missing = declared_symbols() - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"


def test_ctypes_signatures_cover_header(built_lib):
    from cosmicblup_gb300._lib import SIGNATURES, lib
    lib()
    bound = {name for name, _, _ in SIGNATURES}
    assert declared_symbols() <= bound


def test_create_fails_loudly_without_gpu(built_lib):
    from cosmicblup_gb300 import CbxError, Handle
    try:
        Handle(0).close()
    except CbxError as e:
        assert "CBX_ERR_CUDA" in str(e)
        return
    pytest.skip("a GB300 is present")
