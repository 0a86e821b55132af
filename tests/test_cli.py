"""Drop-in command-line drivers (wavefiber3d_gb300/cli/wavepo_cli.cpp): argv
handling and input errors, checked without a GPU (they fail before any CUDA
call)."""
import subprocess

import numpy as np
import pytest

from conftest import ROOT

BUILD = ROOT / "wavefiber3d_gb300" / "_build"


@pytest.fixture(scope="module")
def clis():
    from wavefiber3d_gb300 import build
    build.build()
    return {p.name: p for p in build.build_cli()}


def run(exe, args, cwd):
    return subprocess.run([str(exe), *map(str, args)], cwd=cwd, capture_output=True, text=True, timeout=60)


def test_usage_and_argument_errors(clis, tmp_path):
    for name, nargs in (("wavepo_sphere", 3), ("wavepo_ellipsoid", 1), ("wavepo_treepo", 8)):
        r = run(clis[name], [], tmp_path)
        assert r.returncode == 2 and "usage" in r.stderr
    assert run(clis["wavepo_sphere"], ["0", "x", "2"], tmp_path).returncode == 1
    assert run(clis["wavepo_sphere"], ["0", "1", "-1"], tmp_path).returncode == 1
    r = run(clis["wavepo_treepo"], [0, 1, 90, 0, 4, 2, 0, 10], tmp_path)
    assert r.returncode == 1 and "FIBER" in r.stderr
    r = run(clis["wavepo_treepo"], [0, 1, 90, 0, 0, 2, 10, 3000], tmp_path)
    assert r.returncode == 1 and "ring" in r.stderr
    r = run(clis["wavepo_sphere"], [0, 1, 2, "--theta-mode", "sideways"], tmp_path)
    assert r.returncode == 1 and "theta-mode" in r.stderr


def test_missing_and_short_inputs(clis, tmp_path):
    r = run(clis["wavepo_sphere"], [0, 1, 2], tmp_path)
    assert r.returncode == 1 and "cannot open" in r.stderr and "sphere10um" in r.stderr
    mesh = tmp_path / "mesh"
    mesh.mkdir()
    np.zeros(10, np.float32).tofile(mesh / "sphere10um_area_float.binary")
    np.zeros(29, np.float32).tofile(mesh / "sphere10um_float.binary")  # needs 3 x 10
    np.zeros(30, np.float32).tofile(mesh / "sphere10um_normal_float.binary")
    r = run(clis["wavepo_sphere"], [0, 1, 2], tmp_path)
    assert r.returncode == 1 and "short read" in r.stderr
    r = run(clis["wavepo_treepo"], [0, 1, 90, 0, 0, 2, 0, 10], tmp_path)
    assert r.returncode == 1 and "fiber0.binary" in r.stderr
    assert (tmp_path / "output").is_dir()  # created like the reference drivers do
