"""The `cilia` executable's error reports, which match the reference's
src/main.cpp:56-93 (usage, I/O error, parse error with file and line, a
missing setting); they come before any GPU work, so they run on the CPU."""
import os
import subprocess

import pytest

from conftest import REPO

EXE = os.path.join(REPO, "multi-ciliated-microswimmers_gb300", "_build", "cilia")


def run(*args, cwd):
    return subprocess.run([EXE, *args], capture_output=True, text=True, timeout=60, cwd=cwd)


@pytest.fixture
def exe():
    if not os.path.exists(EXE):
        import __graft_entry__

        __graft_entry__.build()
    return EXE


def test_usage(exe, tmp_path):
    r = run(cwd=tmp_path)
    assert r.returncode == 1 and "usage" in r.stderr and "<configfile>" in r.stderr


def test_missing_file(exe, tmp_path):
    r = run(str(tmp_path / "none.cfg"), cwd=tmp_path)
    assert r.returncode == 1 and "I/O error while reading file." in r.stderr


def test_parse_error_names_file_and_line(exe, tmp_path):
    cfg = tmp_path / "bad.cfg"
    cfg.write_text('name = "x";\nsizex = 8;\nsizey = ;\n')
    r = run(str(cfg), cwd=tmp_path)
    assert r.returncode == 1 and f"Parse error at {cfg}:3" in r.stderr


def test_missing_setting(exe, tmp_path):
    cfg = tmp_path / "noname.cfg"
    cfg.write_text("sizex = 8;\n")
    r = run(str(cfg), cwd=tmp_path)
    assert r.returncode == 1 and "No name setting in configuration file." in r.stderr
    assert not (tmp_path / "inital_randi.dat").exists()  # nothing written
