"""Generates the golden fixtures of the PO path.

Two steps, because the reference's only implementation is CUDA:

  python tests/golden/gen_ref_fixtures.py inputs
      writes the seeded input geometries / patterns below into tests/golden/
      and the case table tests/golden/cases.json (runs anywhere);

  python tests/golden/gen_ref_fixtures.py run OUTDIR
      runs the reference's own CUDA build (oracle/_ref/ref_harness, built with
      `make -C oracle stage-ref` here and `make -C oracle ref-harness` on the
      GPU host) on every case and writes OUTDIR/<case>.bin.  Those files are
      copied into tests/golden/ unchanged and committed.

The parameters of every case live in cases.json so that the tests read the
same values that produced the fixtures.
"""
from __future__ import annotations

import json
import math
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from wavefiber3d_gb300 import geometry, grids  # noqa: E402

SPHERE = dict(file="geom_sphere_r1um_n2000.bin", n=2000)
ELLIPSOID = dict(file="geom_ellipsoid_n3000.bin", n=3000)
HEIGHT = dict(file="hf_fiber_small.bin", radii=[2.0e-6, 1.6e-6], length=1.2e-6, spacing=0.1e-6, seed=7)
SPHERE_BOX = [-1.1e-6, -1.1e-6, -1.1e-6, 1.1e-6, 1.1e-6, 1.1e-6]
ELL_BOX = [-1.65e-6, -1.1e-6, -0.88e-6, 1.65e-6, 1.1e-6, 0.88e-6]
KZ = dict(theta_i=math.pi / 2, phi_i=math.pi)  # incidence along +z, E along x in mode M


def _cases():
    sph_d3 = grids.level_grids(48, 96, 3, 2e-6, 2e-6, 1.3)
    ell_d2 = grids.level_grids(48, 96, 2, 1.6e-6, 3.0e-6, 1.2)
    illum_a = dict(lambda_m=500e-9, mode="M", eta=[1.55, 0.0], sigma=1e-2, **KZ)
    illum_b = dict(lambda_m=640e-9, theta_i=0.3, phi_i=1.1, mode="E", eta=[1.55, 0.1], sigma=1.5e-6)
    return [
        dict(name="ref_currents_sphere_M", kind="currents", geom=SPHERE, illum=illum_a),
        dict(name="ref_currents_ellipsoid_E", kind="currents", geom=ELLIPSOID, illum=illum_b),
        dict(name="ref_octree_ellipsoid_d3", kind="octree", geom=ELLIPSOID, box=ELL_BOX, depth=3),
        dict(name="ref_solve_sphere_d0", kind="solve", geom=SPHERE, box=SPHERE_BOX, depth=0,
             n_theta=[48], n_phi=[96], illum=illum_a),
        dict(name="ref_solve_sphere_d3", kind="solve", geom=SPHERE, box=SPHERE_BOX, depth=3,
             n_theta=sph_d3[0], n_phi=sph_d3[1], illum=illum_a),
        dict(name="ref_solve_ellipsoid_d2", kind="solve", geom=ELLIPSOID, box=ELL_BOX, depth=2,
             n_theta=ell_d2[0], n_phi=ell_d2[1], illum=illum_b),
        dict(name="ref_solve_sphere_quirk_d1", kind="solve", geom=SPHERE, box=SPHERE_BOX, depth=1,
             n_theta=[48, 40], n_phi=[300, 40], illum=illum_a),
        dict(name="ref_interp_even", kind="interp", input="interp_in_20x30.bin", src=[20, 30], dst=[33, 300]),
        dict(name="ref_interp_odd", kind="interp", input="interp_in_21x25.bin", src=[21, 25], dst=[40, 64]),
        dict(name="ref_average_leftover", kind="average", input="avg_in_45x88.bin", src=[45, 88], dst=[18, 36]),
        dict(name="ref_average_even", kind="average", input="avg_in_90x144.bin", src=[90, 144], dst=[18, 36]),
        dict(name="ref_average_ragged", kind="average", input="avg_in_7x13.bin", src=[7, 13], dst=[3, 4]),
        dict(name="ref_heightfield_full", kind="heightfield", height=HEIGHT, ring=[0, -1]),
        dict(name="ref_heightfield_segment", kind="heightfield", height=HEIGHT, ring=[20, 70]),
        dict(name="ref_heightfield_wrap", kind="heightfield", height=HEIGHT, ring=[90, -1]),
    ]


def small_height_field():
    """The seeded fiber-like height field of the height-field cases."""
    h = HEIGHT
    return geometry.fiber_height_field(radii=h["radii"], length=h["length"], spacing=h["spacing"],
                                       scale_spacing=0.5e-6, scale_step=0.04e-6, noise_sigma=0.01e-6,
                                       noise_corr=0.2e-6, seed=h["seed"])


def make_inputs():
    geometry.fibonacci_sphere(1e-6, SPHERE["n"]).save(HERE / SPHERE["file"])
    geometry.ellipsoid((1.5e-6, 1.0e-6, 0.8e-6), ELLIPSOID["n"]).save(HERE / ELLIPSOID["file"])
    rng = np.random.default_rng(20231203)
    for c in _cases():
        if c["kind"] == "interp":
            th, ph = c["src"]
            z = (rng.standard_normal((th, ph)) + 1j * rng.standard_normal((th, ph))).astype(np.complex64)
            z.tofile(HERE / c["input"])
    rng = np.random.default_rng(20231204)
    for c in _cases():
        if c["kind"] == "average":
            th, ph = c["src"]
            rng.exponential(1.0, (th, ph)).astype(np.float32).tofile(HERE / c["input"])
    hf = small_height_field()
    hf.save(HERE / HEIGHT["file"])
    HEIGHT["numel"], HEIGHT["numelvert"], HEIGHT["period"], HEIGHT["unitz"] = hf.numel, hf.numelvert, hf.period, hf.unitz
    (HERE / "cases.json").write_text(json.dumps(_cases(), indent=1) + "\n")


def _harness_args(c):
    g = c.get("geom")
    args = []
    if c["kind"] == "currents":
        il = c["illum"]
        args = ["currents", str(HERE / g["file"]), str(g["n"]), repr(il["lambda_m"]), repr(il["theta_i"]),
                repr(il["phi_i"]), il["mode"], repr(il["eta"][0]), repr(il["eta"][1]), repr(il["sigma"])]
    elif c["kind"] == "octree":
        args = ["octree", str(HERE / g["file"]), str(g["n"])] + [repr(v) for v in c["box"]] + [str(c["depth"])]
    elif c["kind"] == "interp":
        args = ["interp", str(HERE / c["input"])] + [str(v) for v in c["src"] + c["dst"]]
    elif c["kind"] == "average":
        args = ["average", str(HERE / c["input"])] + [str(v) for v in c["src"] + c["dst"]]
    elif c["kind"] == "heightfield":
        h = c["height"]
        end = c["ring"][1] if c["ring"][1] >= 0 else h["numel"] - 1
        args = ["heightfield", str(HERE / h["file"]), str(h["numel"]), str(h["numelvert"]), repr(h["period"]),
                repr(h["unitz"]), str(c["ring"][0]), str(end)]
    elif c["kind"] == "solve":
        il = c["illum"]
        args = ["solve", str(HERE / g["file"]), str(g["n"])] + [repr(v) for v in c["box"]] + [str(c["depth"])]
        for t, p in zip(c["n_theta"], c["n_phi"]):
            args += [str(t), str(p)]
        args += [repr(il["lambda_m"]), repr(il["theta_i"]), repr(il["phi_i"]), il["mode"], repr(il["eta"][0]),
                 repr(il["eta"][1]), repr(il["sigma"])]
    return args


def run(outdir: Path, kinds=None):
    """Runs the harness on every case (or the cases of the given kinds; the
    height-field cases are host code and run without a GPU)."""
    outdir.mkdir(parents=True, exist_ok=True)
    exe = ROOT / "oracle" / "_ref" / "ref_harness"
    for c in json.loads((HERE / "cases.json").read_text()):
        if kinds and c["kind"] not in kinds:
            continue
        out = outdir / (c["name"] + ".bin")
        cmd = [str(exe)] + _harness_args(c) + [str(out)]
        print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True, timeout=600)


if __name__ == "__main__":
    if len(sys.argv) >= 2 and sys.argv[1] == "inputs":
        make_inputs()
    elif len(sys.argv) >= 3 and sys.argv[1] == "run":
        run(Path(sys.argv[2]), sys.argv[3:])
    else:
        print(__doc__)
        sys.exit(2)
