"""The qtnh C++ API (include/qtnh.hpp, libqtnh.so) driven by tests/cpp/api_test.cpp:
the reference's test scenarios (indexing, construction, accessors, golden contractions
incl. rescattered operands, networks, QFT with distributed qubits) on the GB300 engine."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BIN = os.path.join(HERE, "cpp", "_build", "api_test")
GOLDEN = os.path.join(HERE, "golden")


@pytest.fixture(scope="module", autouse=True)
def _built():
    from qtnh_gb300 import build
    build.build()


def _run(mode):
    r = subprocess.run([BIN, mode, GOLDEN], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok")
    return r.stdout


def test_api_host_only():
    _run("cpu")


@pytest.mark.gpu
def test_api_on_gpu():
    out = _run("gpu")
    # every reference scenario ran: hundreds of checks
    assert int(out.split()[1].split("/")[1]) > 200
