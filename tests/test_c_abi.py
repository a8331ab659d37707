"""The C ABI from plain C (tests/c_abi_smoke.c), the way a foreign-function
binding calls it: the header compiles as C99 against the library, argument
and state errors come back as codes without a GPU, and on a GPU a plan runs
end to end into a host buffer."""
import os
import subprocess

import pytest

from conftest import ROOT


def _build(tmp_path):
    from geosgs import _abi, _build

    _build.build()
    lib = os.path.dirname(_abi.LIB_PATH)
    exe = str(tmp_path / "c_abi_smoke")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c_abi_smoke.c"), "-o", exe, "-L", lib, "-lgeosgs",
                    "-Wl,-rpath," + lib, "-lm"], check=True)
    return exe


def test_c_abi_errors_from_c(tmp_path):
    r = subprocess.run([_build(tmp_path), "nogpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "ok" in r.stdout


@pytest.mark.gpu
def test_c_abi_plan_from_c(tmp_path, geosgs_lib):
    r = subprocess.run([_build(tmp_path), "gpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "ok" in r.stdout
