"""The C ABI library loads and exports every function the headers declare
(no GPU needed: nothing is computed)."""
import ctypes
import os
import re

import pytest

from conftest import REPO

import cilia_gpu


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(REPO, "include"))):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(REPO, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*[A-Za-z_][\w\s\*]*?\b((?:mpcd|cilia)_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def library():
    if not os.path.exists(cilia_gpu.LIB_PATH):
        import __graft_entry__

        __graft_entry__.build()
    return ctypes.CDLL(cilia_gpu.LIB_PATH)


def test_headers_declare_entry_points():
    names = declared_functions()
    assert "mpcd_step" in names and "cilia_sim_create" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol(library):
    missing = [n for n in declared_functions() if not hasattr(library, n)]
    assert not missing, missing


def test_binding_signatures_cover_headers():
    lib = cilia_gpu.lib()
    for n in declared_functions():
        assert getattr(lib, n).argtypes is not None, n


def test_cilia_executable_built():
    exe = os.path.join(REPO, "multi-ciliated-microswimmers_gb300", "_build", "cilia")
    assert os.path.exists(exe) and os.access(exe, os.X_OK)
