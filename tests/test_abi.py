"""The C-ABI library builds for sm_103a, loads, and exports every entry point
that include/*.h declares (no GPU needed: nothing is called)."""
import glob
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = set()
    for hdr in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(hdr).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(?:int|const char \*)\s*(phn_\w+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from phinum_gb300 import build
    build.build()
    from phinum_gb300 import _lib
    return _lib.load()


def test_header_declares_entry_points():
    names = declared()
    assert "phn_create" in names and "phn_evolve" in names and len(names) >= 20


def test_library_exports_every_declared_symbol(lib):
    from phinum_gb300 import build
    out = subprocess.run(["nm", "-D", "--defined-only", build.LIB], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (phn_\w+)", out))
    missing = [n for n in declared() if n not in exported]
    assert not missing, missing
    for n in declared():
        assert hasattr(lib, n)


def test_binding_covers_header(lib):
    from phinum_gb300 import _lib
    assert set(_lib.exported_symbols()) <= set(declared())
    import re
    hdr = open(os.path.join(ROOT, "include", "phinum_gpu.h")).read()
    version = int(re.search(r"#define PHN_ABI_VERSION (\d+)", hdr).group(1))
    assert lib.phn_abi_version() == version == _lib.ABI_VERSION

