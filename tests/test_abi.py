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


@pytest.mark.parametrize("lang", ["c99", "c++11"])
def test_headers_compile_and_link_from_c(lang, tmp_path, library):
    """Every header compiles on its own as C99 and as C++11 (the reference is
    C++11, its FFI callers may be C), and a program that takes the address of
    every declared entry point links against the library."""
    import shutil
    import subprocess

    cc = shutil.which("gcc" if lang == "c99" else "g++")
    if cc is None:
        pytest.skip("no host compiler")
    inc = os.path.join(REPO, "include")
    headers = sorted(h for h in os.listdir(inc) if h.endswith(".h"))
    names = declared_functions()
    src = "".join(f'#include "{h}"\n' for h in headers)
    src += "typedef void (*fp)(void);\nstatic const fp table[] = {\n"
    src += "".join(f"  (fp){n},\n" for n in names)
    src += "};\nint main(void) { return table[0] == 0; }\n"
    path = tmp_path / ("abi.c" if lang == "c99" else "abi.cpp")
    path.write_text(src)
    flags = ["-std=c99", "-pedantic"] if lang == "c99" else ["-std=c++11"]
    for h in headers:  # each header alone
        one = tmp_path / ("one.c" if lang == "c99" else "one.cpp")
        one.write_text(f'#include "{h}"\nint main(void) {{ return 0; }}\n')
        r = subprocess.run([cc, *flags, "-Wall", "-Werror", "-fsyntax-only", "-I", inc, str(one)],
                           capture_output=True, text=True)
        assert r.returncode == 0, (h, r.stderr)
    build = os.path.dirname(cilia_gpu.LIB_PATH)
    r = subprocess.run([cc, *flags, "-Wall", "-I", inc, str(path), "-o", str(tmp_path / "abi"), "-L", build,
                        "-lmpcd_gpu", f"-Wl,-rpath,{build}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
