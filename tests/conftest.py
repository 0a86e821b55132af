import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the C ABI library")


@pytest.fixture(scope="session")
def cases():
    import json
    return {c["name"]: c for c in json.loads((GOLDEN / "cases.json").read_text())}


def load_case_geometry(case):
    from wavefiber3d_gb300.geometry import PointCloud
    return PointCloud.load(GOLDEN / case["geom"]["file"])


def case_illum(case):
    import oracle
    il = case["illum"]
    return oracle.make_illum(il["lambda_m"], il["theta_i"], il["phi_i"], il["mode"], complex(*il["eta"]), il["sigma"])


def load_case_height_field(case):
    """(HeightField, ring_begin, ring_end) of a height-field case."""
    from wavefiber3d_gb300.geometry import HeightField
    h = case["height"]
    hf = HeightField.load(GOLDEN / h["file"], h["numel"], h["numelvert"], h["period"])
    assert hf.unitz == h["unitz"]
    end = case["ring"][1] if case["ring"][1] >= 0 else h["numel"] - 1
    return hf, case["ring"][0], end
