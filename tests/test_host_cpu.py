"""The C++ drivers on the host, before any GPU work: command-line and
parameters.txt errors end them with a message and a non-zero status, where
the reference threw std::invalid_argument (admin.cpp catch_parameter,
geometry.cpp, modeling.cu set_properties). Without a CUDA device the engine's
context creation fails with its status message: there is no CPU fallback."""
import os
import subprocess

import numpy as np
import pytest

from helpers import write_case

NAMES = ["modeling.exe", "inversion.exe", "traveltime_tables.exe", "migration.exe"]


def _run(exe, *args):
    return subprocess.run([exe, *args], capture_output=True, text=True, timeout=120)


def _case(d):
    m = np.full((40, 20), 1.0 / 2000.0, np.float32)
    return write_case(str(d), 40, 20, 10.0, 10.0, m, [(100.0, 0.0)], [(50.0, 0.0), (300.0, 0.0)])


@pytest.mark.parametrize("name", NAMES)
def test_usage_without_arguments(exes, name):
    r = _run(exes[name])
    assert r.returncode == 1
    assert f"usage: {name} parameters.txt" in r.stderr


@pytest.mark.parametrize("name", NAMES)
def test_missing_parameter_file(exes, name, tmp_path):
    r = _run(exes[name], str(tmp_path / "none.txt"))
    assert r.returncode == 2
    assert "none.txt could not be opened" in r.stderr


@pytest.mark.parametrize("name", NAMES)
def test_missing_model_file(exes, name, tmp_path):
    p = _case(tmp_path)
    os.remove(tmp_path / "slowness.bin")
    r = _run(exes[name], p)
    assert r.returncode == 2
    assert "slowness.bin could not be opened" in r.stderr


def test_missing_geometry_file(exes, tmp_path):
    p = _case(tmp_path)
    os.remove(tmp_path / "sps.txt")
    r = _run(exes["modeling.exe"], p)
    assert r.returncode == 2
    assert "sps.txt could not be opened" in r.stderr


def test_context_creation_fails_without_a_gpu(exes, tmp_path):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = _run(exes["modeling.exe"], _case(tmp_path))
    assert r.returncode == 2
    assert "sf_ctx_create" in r.stderr
