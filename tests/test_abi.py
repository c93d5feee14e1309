"""The C-ABI library loads and exports every symbol declared in include/*.h (no GPU needed:
nothing here launches a kernel)."""
import ctypes
import os
import re

from conftest import ROOT


def declared_symbols():
    syms = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        txt = open(os.path.join(inc, f)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        syms |= set(re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(pmgb_\w+)\s*\(", txt, re.M))
    return syms


def test_library_builds_and_exports_declared_symbols():
    from particlesimulation_gb300 import _lib, build
    build.build()
    lib = ctypes.CDLL(_lib.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert set(_lib.EXPORTS) <= syms
    assert lib.pmgb_version


def test_version_string():
    from particlesimulation_gb300 import _lib
    v = _lib.lib().pmgb_version().decode()
    assert "sm_103a" in v

