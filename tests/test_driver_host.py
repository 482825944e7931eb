"""The C++ host driver without a GPU: it is built, prints its usage and turns
missing or malformed input files into an error exit before touching CUDA
(the reference's paramRead would dereference a NULL FILE*)."""
from __future__ import annotations

import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
DRIVER = ROOT / "lbm_bench_gpu_gb300" / "bin" / "lbm_zsc"


@pytest.fixture(scope="module")
def driver(lib):
    assert DRIVER.exists(), "lbm_zsc is built with the library"
    return DRIVER


def test_usage(driver):
    r = subprocess.run([str(driver), "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "properties.in" in r.stdout


def test_bad_option(driver):
    r = subprocess.run([str(driver), "--storage", "fp8"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "unknown storage" in r.stderr


def test_missing_inputs(driver, tmp_path):
    r = subprocess.run([str(driver), str(tmp_path)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "properties.in" in r.stderr


def test_malformed_inputs(driver, tmp_path):
    (tmp_path / "properties.in").write_text("maxStep relaxStep save stat\n10 x\n")
    (tmp_path / "discrete.in").write_text("nBubbles\n0\n\nxc yc zc Rc\n")
    r = subprocess.run([str(driver), str(tmp_path)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "ERROR" in r.stderr


def test_bad_objective(driver):
    r = subprocess.run([str(driver), "--adjoint", "drag"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "unknown objective" in r.stderr
