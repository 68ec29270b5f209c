"""The C-ABI library loads and exports every entry point include/svgpu.h declares
(no GPU needed: nothing is called)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(svgpu_[a-z0-9_]+)\s*\(", src, re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from svfsiplus_gb300 import api, build
    if not os.path.exists(api.LIB_PATH):
        build.build()
    return ctypes.CDLL(api.LIB_PATH)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "svgpu_fsils_solve" in names and "svgpu_construct_fluid" in names
    assert len(names) >= 15


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_product_has_no_oracle_dependency():
    import subprocess
    pkg = os.path.join(ROOT, "svfsiplus_gb300")
    out = subprocess.run(["grep", "-rl", "oracle", pkg, "--include=*.py", "--include=*.cu",
                          "--include=*.cpp", "--include=*.h"], capture_output=True, text=True).stdout
    offenders = [l for l in out.split() if "pyoracle" in open(l).read() or "svoracle" in open(l).read()]
    assert not offenders, offenders
