"""CPU checks of the FP64 oracle: its own invariants, an independent numpy
restatement, the Mie series, and the pins against the reference's own CUDA
outputs (tests/golden/ref_*.bin, generated by tests/golden/gen_ref_fixtures.py)."""
import math

import numpy as np
import pytest

from conftest import GOLDEN, case_illum, load_case_geometry

import oracle
from oracle import mie
from wavefiber3d_gb300 import geometry, grids


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300))


def fixture(name, dtype=np.float32):
    p = GOLDEN / f"{name}.bin"
    assert p.exists(), f"golden fixture {p.name} missing"
    return np.fromfile(p, dtype=dtype)


# ---------------------------------------------------------- oracle invariants
def test_fresnel_limits():
    eta = 1.55 + 0.1j
    rs, rp = oracle.fresnel(0.0, 1.0 + 0j, eta)
    assert abs(rs - (1 - eta) / (1 + eta)) < 1e-12
    assert abs(rp - (eta - 1) / (eta + 1)) < 1e-12
    rs, rp = oracle.fresnel(math.pi / 2 - 1e-9, 1.0 + 0j, eta)
    assert abs(rs + 1) < 1e-6 and abs(rp + 1) < 1e-6  # util.h:378-382 sign convention


def test_currents_are_tangential_and_zero_in_shadow():
    cloud = geometry.ellipsoid((1.5e-6, 1.0e-6, 0.8e-6), 3000)
    il = oracle.make_illum(600e-9, 0.4, -0.7, "E", 1.55 + 0.1j, 3e-6)
    cur = oracle.currents(cloud, il, scale=False)
    n = np.stack([cloud.nx, cloud.ny, cloud.nz], 1).astype(np.float64)
    assert np.abs(np.einsum("pc,pc->p", cur[:, :3], n)).max() < 1e-9 * np.abs(cur).max()
    assert np.abs(np.einsum("pc,pc->p", cur[:, 3:], n)).max() < 1e-9 * np.abs(cur).max()
    k = np.array([math.cos(0.4) * math.cos(-0.7), math.cos(0.4) * math.sin(-0.7), math.sin(0.4)])
    shadow = (n @ k).astype(np.float32) > 0
    assert shadow.any() and np.all(cur[shadow] == 0) and np.all(np.abs(cur[~shadow]).sum(1) > 0)


def test_far_field_matches_numpy_restatement():
    cloud = geometry.fibonacci_sphere(0.7e-6, 300)
    il = oracle.make_illum(450e-9, 0.1, 0.2, "M", 1.55, 1e-2)
    cur = oracle.currents(cloud, il)
    k = 2 * math.pi / 450e-9
    ctr = np.array([0.05e-6, 0.0, -0.1e-6])
    f = oracle.far_field(cloud, cur, k, ctr, 9, 14)
    s = grids.directions(9, 14)
    x = np.stack([cloud.x, cloud.y, cloud.z], 1).astype(np.float64) - ctr
    ref = np.exp(1j * k * (s @ x.T)) @ cur
    assert rel(f, ref) < 1e-12
    inten = oracle.intensity(f, 9, 14).ravel()
    z0 = oracle.z0()
    E = f[:, :3] - (np.einsum("dc,dc->d", f[:, :3], s))[:, None] * s
    H = f[:, 3:] - (np.einsum("dc,dc->d", f[:, 3:], s))[:, None] * s
    Ep = E - z0 * np.cross(s, H)
    assert rel(inten, (np.abs(Ep) ** 2).sum(1)) < 1e-12


def test_octree_structure():
    cloud = geometry.ellipsoid((1.5e-6, 1.0e-6, 0.8e-6), 3000)
    box = [-1.65e-6, -1.1e-6, -0.88e-6, 1.65e-6, 1.1e-6, 0.88e-6]
    perm, rng, bx = oracle.octree(cloud, box[:3], box[3:], 3)
    assert sorted(perm.tolist()) == list(range(cloud.n))
    off = [(8 ** l - 1) // 7 for l in range(5)]
    for l in range(3):
        for h in range(off[l], off[l + 1]):
            kids = off[l + 1] + 8 * (h - off[l]) + np.arange(8)
            assert rng[kids[0], 0] == rng[h, 0] and rng[kids[-1], 1] == rng[h, 1]
            assert np.all(rng[kids[1:], 0] == rng[kids[:-1], 1])
    p = np.stack([cloud.x, cloud.y, cloud.z], 1)[perm]
    for h in range(off[3], off[4]):
        b, e = rng[h]
        if e > b:
            assert np.all(perm[b:e][1:] > perm[b:e][:-1])  # stable
            inside = np.all((p[b:e] >= bx[h, :3]) & (p[b:e] < bx[h, 3:]), axis=1)
            assert inside.all()


def test_interp_is_exact_for_band_limited_patterns():
    rng = np.random.default_rng(5)
    for (tc, pc), (tp, pp) in [((15, 21), (40, 64)), ((16, 20), (33, 300)), ((9, 9), (9, 9))]:
        kt = np.fft.fftfreq(tc) * tc
        kp = np.fft.fftfreq(pc) * pc
        C = np.zeros((tc, pc), complex)
        mt, mp = (tc - 1) // 2, (pc - 1) // 2
        sel = (np.abs(kt)[:, None] <= mt) & (np.abs(kp)[None, :] <= mp)
        C[sel] = rng.standard_normal(sel.sum()) + 1j * rng.standard_normal(sel.sum())

        def ev(nt, np_):
            t = np.arange(nt)[:, None, None, None] / nt
            p = np.arange(np_)[None, :, None, None] / np_
            return (C[None, None] * np.exp(2j * np.pi * (kt[:, None] * t + kp[None, :] * p))).sum((2, 3))

        out = oracle.interp(ev(tc, pc), tp, pp, nyquist_quirk=False)
        assert rel(out, ev(tp, pp)) < 1e-11


def test_interp_quirk_only_touches_unreached_columns():
    rng = np.random.default_rng(9)
    z = rng.standard_normal((20, 30)) + 1j * rng.standard_normal((20, 30))
    a = oracle.interp(z, 33, 300, nyquist_quirk=True)
    b = oracle.interp(z, 33, 300, nyquist_quirk=False)
    assert np.array_equal(a[:, :256], b[:, :256])
    assert rel(a[:, 256:], b[:, 256:]) > 1e-6


def _numpy_tree(cloud, il, box, depth, nth, nph):
    """Independent restatement of the hierarchical solve (cover = pi, quirk-free
    Nyquist split) with numpy FFTs."""
    perm, rngs, bx = oracle.octree(cloud, box[:3], box[3:], depth)
    cur = oracle.currents(cloud, il)[perm]
    x = np.stack([cloud.x, cloud.y, cloud.z], 1).astype(np.float64)[perm]
    k0 = 2 * math.pi / il.lambda_m
    off = [(8 ** l - 1) // 7 for l in range(depth + 2)]
    ctr = lambda h: (0.5 * (bx[h, :3] + bx[h, 3:])).astype(np.float64)

    def up(X, n_out, axis):
        n = X.shape[axis]
        F = np.fft.fft(X, axis=axis)
        F = np.moveaxis(F, axis, 0)
        Y = np.zeros((n_out,) + F.shape[1:], complex)
        h = (n + 2) // 2
        Y[:h] = F[:h]
        Y[h + n_out - n:] = F[h:]
        if n % 2 == 0:
            Y[h - 1] /= 2
            Y[h - 1 + n_out - n] = Y[h - 1]
        return np.moveaxis(np.fft.ifft(Y, axis=0) * (n_out / n), 0, axis)

    s = grids.directions(nth[depth], nph[depth])
    pats = {}
    for h in range(off[depth], off[depth + 1]):
        b, e = rngs[h]
        if e > b:
            pats[h] = (np.exp(1j * k0 * (s @ (x[b:e] - ctr(h)).T)) @ cur[b:e]).reshape(nth[depth], nph[depth], 6)
    for l in range(depth - 1, -1, -1):
        s = grids.directions(nth[l], nph[l]).reshape(nth[l], nph[l], 3)
        new = {}
        for h in range(off[l], off[l + 1]):
            for o in range(8):
                hc = off[l + 1] + 8 * (h - off[l]) + o
                if hc in pats:
                    v = up(up(pats[hc], nph[l], 1), nth[l], 0) * np.exp(1j * k0 * (s @ (ctr(hc) - ctr(h))))[..., None]
                    new[h] = new.get(h, 0) + v
        pats = new
    return oracle.intensity(pats[0].reshape(-1, 6), nth[0], nph[0])


def test_oracle_tree_matches_numpy_restatement(cases):
    c = cases["ref_solve_ellipsoid_d2"]
    cloud, il = load_case_geometry(c), case_illum(c)
    a = oracle.solve_tree(cloud, il, c["box"][:3], c["box"][3:], c["depth"], c["n_theta"], c["n_phi"],
                          nyquist_quirk=False)
    b = _numpy_tree(cloud, il, c["box"], c["depth"], c["n_theta"], c["n_phi"])
    # the oracle takes every level's child offsets from the level's first node
    # as sphere.cu:499-539 does; the restatement uses each node's own float
    # centres.  The two differ by float rounding of the centres (~1e-13 m).
    assert rel(a, b) < 1e-6


def test_reference_tree_is_inaccurate_near_poles(cases):
    """The reference's pi-periodic theta interpolation (interpolation.h:48-77)
    is far from the direct sum when the pattern peaks at a pole: the reason the
    engine defaults to the double-cover theta grid."""
    c = cases["ref_solve_sphere_d3"]
    cloud, il = load_case_geometry(c), case_illum(c)
    d0 = oracle.solve_direct(cloud, il, 48, 96)
    tr = oracle.solve_tree(cloud, il, c["box"][:3], c["box"][3:], 3, c["n_theta"], c["n_phi"])
    assert rel(tr, d0) > 0.1


def test_mie_forward_lobe():
    """PO vs the Mie series on the 2 um sphere (20,000 Fibonacci points,
    n = 1.55, 500 nm): normalised theta = 0 ring (compareMie/mie.ipynb cell 4),
    forward diffraction lobe 0-10 degrees.  PO neglects the transmitted light,
    so only the diffraction lobe is compared."""
    cloud = geometry.fibonacci_sphere(2e-6, 20000)
    il = oracle.make_illum(500e-9, 0.0, 0.0, "M", 1.55, 1e-2)
    nth, nph = 180, 720
    dirs = np.arange(nph) + (nth // 2) * nph
    cur = oracle.currents(cloud, il)
    f = oracle.far_field_sampled(cloud, cur, 2 * math.pi / 500e-9, [0, 0, 0], nth, nph, dirs)
    po = oracle.intensity_sampled(f, nth, nph, dirs)
    ang = 2 * np.pi * np.arange(nph) / nph
    s = np.stack([np.cos(ang), np.sin(ang), np.zeros(nph)], 1)
    mi = mie.polarised_intensity(2e-6, 500e-9, 1.55, [1, 0, 0], [0, 0, 1], s)
    lobe = slice(0, int(10 / 360 * nph))
    assert rel(po[lobe] / po[0], mi[lobe] / mi[0]) < 0.1


def test_mie_coefficients_small_sphere_rayleigh_limit():
    # for x << 1 the phase function tends to the Rayleigh form |S1|^2 ~ const, |S2|^2 ~ cos^2
    s1, s2 = mie.amplitudes(0.01, 1.5, np.array([0.0, math.pi / 2]))
    assert abs(abs(s2[1]) / abs(s2[0])) < 1e-3
    assert abs(abs(s1[1]) / abs(s1[0]) - 1) < 1e-3


# ---------------------------------------------- pins against the reference build
@pytest.mark.parametrize("name", ["ref_currents_sphere_M", "ref_currents_ellipsoid_E"])
def test_oracle_currents_pinned_to_reference(cases, name):
    c = cases[name]
    cloud, il = load_case_geometry(c), case_illum(c)
    r = fixture(name).reshape(-1, 12).astype(np.float64).view(np.complex128)
    assert rel(oracle.currents(cloud, il, scale=False), r) < 1e-5


def test_oracle_octree_pinned_to_reference(cases):
    c = cases["ref_octree_ellipsoid_d3"]
    cloud = load_case_geometry(c)
    raw = fixture(c["name"], np.uint8)
    n = cloud.n
    geo = np.frombuffer(raw[: 28 * n].tobytes(), dtype=np.float32).reshape(7, n)
    rng = np.frombuffer(raw[28 * n:].tobytes(), dtype=np.int32).reshape(-1, 2)
    perm, orng, _ = oracle.octree(cloud, c["box"][:3], c["box"][3:], c["depth"])
    assert np.array_equal(cloud.soa()[:, perm], geo)
    assert np.array_equal(orng, rng)


@pytest.mark.parametrize("name", ["ref_interp_even", "ref_interp_odd"])
def test_oracle_interp_pinned_to_reference(cases, name):
    c = cases[name]
    z = np.fromfile(GOLDEN / c["input"], dtype=np.complex64).reshape(c["src"]).astype(np.complex128)
    r = fixture(name).view(np.complex64).reshape(c["dst"])
    assert rel(oracle.interp(z, *c["dst"], nyquist_quirk=True), r) < 1e-5


@pytest.mark.parametrize("name", ["ref_solve_sphere_d0", "ref_solve_sphere_d3", "ref_solve_ellipsoid_d2",
                                  "ref_solve_sphere_quirk_d1"])
def test_oracle_solve_pinned_to_reference(cases, name):
    c = cases[name]
    cloud, il = load_case_geometry(c), case_illum(c)
    r = fixture(name).reshape(c["n_theta"][0], c["n_phi"][0])
    o = oracle.solve_tree(cloud, il, c["box"][:3], c["box"][3:], c["depth"], c["n_theta"], c["n_phi"], True)
    assert rel(o, r) < 1e-4


# ------------------------------------------------- height field (geometry.h)
@pytest.mark.parametrize("name", ["ref_heightfield_full", "ref_heightfield_segment", "ref_heightfield_wrap"])
def test_height_field_oracle_vs_reference_build(cases, name):
    """The float restatement equals the reference's own set_sourcepoint bit for bit."""
    from conftest import load_case_height_field
    hf, b, e = load_case_height_field(cases[name])
    out, bad = oracle.height_field(hf, b, e)
    ref = fixture(name).reshape(7, -1)
    assert not bad
    assert out.shape == ref.shape
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))


def test_height_field_oracle_geometry():
    """Independent float64 check: samples on the surface, unit normals pointing
    outwards, areas summing to the lateral area of the segment."""
    hf = geometry.fiber_height_field(radii=(2e-6, 1.6e-6), length=1.0e-6, spacing=0.02e-6, scale_step=0.0,
                                     noise_sigma=1e-12, seed=1)
    out, bad = oracle.height_field(hf)
    assert not bad
    x, y, z, nx, ny, nz, a = out.astype(np.float64)
    assert np.allclose(np.sqrt(nx * nx + ny * ny + nz * nz), 1.0, atol=1e-6)
    assert np.all(nx * x / 4e-12 + ny * y / 2.56e-12 > 0)  # outward (ellipse gradient)
    # the last axial row of quads repeats row numelvert-1 (geometry.h:100-103): the band is numelvert*unitz high
    lateral = geometry.ellipse_perimeter(2e-6, 1.6e-6) * hf.numelvert * hf.unitz
    assert abs(a.sum() / lateral - 1) < 2e-3
    assert abs(z.min() - (-hf.period / 2 + hf.unitz / 2)) < 1e-12


def test_height_field_origin_vertex_flagged():
    hf = geometry.fiber_height_field(radii=(2e-6, 1.6e-6), length=0.5e-6, spacing=0.1e-6, seed=2)
    hf.xy[:, 5, 3] = 0.0
    _, bad = oracle.height_field(hf)
    assert bad
    _, bad = oracle.height_field(hf, 20, 40)  # the zero vertex is outside the segment
    assert not bad


# ------------------------------------------------ pattern averaging (fields.h)
@pytest.mark.parametrize("name", ["ref_average_leftover", "ref_average_even", "ref_average_ragged"])
def test_average_oracle_vs_reference_build(cases, name):
    c = cases[name]
    inp = np.fromfile(GOLDEN / c["input"], dtype=np.float32).reshape(c["src"])
    out = oracle.average(inp, *c["dst"])
    ref = fixture(name).reshape(c["dst"])
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))


def test_average_oracle_uses_leading_samples_only():
    """Integer ratios (fields.h:210-211): 45 -> 18 rows averages rows 0..35 in pairs."""
    p = np.zeros((45, 88), np.float32)
    p[36:, :] = 1e9
    p[:, 72:] = 1e9
    out = oracle.average(p, 18, 36)
    assert np.all(out == 0)
    q = np.arange(45 * 88, dtype=np.float32).reshape(45, 88)
    want = q[:36, :72].reshape(18, 2, 36, 2).mean(axis=(1, 3))
    assert np.allclose(oracle.average(q, 18, 36), want, rtol=1e-6)


# ------------------------------------- pattern statistics (fittingutil.py)
def test_acf_oracle_shifted_fft_matches_definition():
    """numpy stands in for FFTW in the restatement of ForwardFFT_shifted; pin it
    to the transform's definition (odd and even sizes)."""
    from oracle import acf
    rng = np.random.default_rng(3)
    for shape in ((6, 10), (7, 9), (5, 8)):
        a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        assert np.allclose(acf.forward_fft_shifted(a), acf.shifted_dft_direct(a), rtol=1e-12, atol=1e-12)
        assert np.allclose(acf.inverse_fft_shifted(a), acf.shifted_idft_direct(a), rtol=1e-12, atol=1e-12)
        # unnormalised pair: inverse(forward(a)) = N a when both sizes are even
        # (for an odd size the two rolls differ by one sample, as in the reference)
        n = shape[0] * shape[1]
        if shape[0] % 2 == 0 and shape[1] % 2 == 0:
            assert np.allclose(acf.inverse_fft_shifted(acf.forward_fft_shifted(a)), n * a, rtol=1e-10,
                               atol=1e-10)


def test_acf_oracle_pipeline_properties():
    """The ACF of the mean spectrum peaks at the shifted origin and is symmetric."""
    from oracle import acf
    rng = np.random.default_rng(4)
    raw = rng.standard_normal((16, 20, 12, 3))
    noisemat, mean = acf.weightedsum(raw, [0.5, 1.0, 2.0])
    f, a = acf.acf_from_ft(noisemat, mean)
    assert a.shape == (16, 20) and np.argmax(a) == np.ravel_multi_index((8, 10), (16, 20))
    assert np.allclose(a[1:, 1:], a[1:, 1:][::-1, ::-1], rtol=1e-9, atol=1e-9 * np.abs(a).max())


def test_point_gradient_fd_matches_brute_force_differences():
    """oracle.point_gradient_fd (central differences taken on one point's own
    field) equals the plain central differences of the whole FP64 loss."""
    cloud = geometry.ellipsoid((1.5e-6, 1.0e-6, 0.8e-6), 2000)
    s64 = cloud.soa().astype(np.float64)
    th, ph = 0.4, -0.7
    il = oracle.make_illum(600e-9, th, ph, "E", 1.55 + 0.1j, 3e-6)
    nth, nph = 24, 48
    dirs = np.arange(nth * nph)
    w = np.random.default_rng(5).standard_normal(dirs.size)
    k = np.array([math.cos(th) * math.cos(ph), math.cos(th) * math.sin(ph), math.sin(th)])
    lit = np.flatnonzero(s64[3:6].T @ k < -0.05)
    pts = lit[[3, 50, 400]]
    steps = [2e-10] * 3 + [1e-6] * 3 + [1e-6]
    g = oracle.point_gradient_fd(s64, il, nth, nph, dirs, w, pts, steps)
    fd = np.zeros((7, pts.size))
    for j, p in enumerate(pts):
        for q in range(7):
            h = steps[q] * (s64[6, p] if q == 6 else 1.0)
            a, b = s64.copy(), s64.copy()
            a[q, p] += h
            b[q, p] -= h
            fd[q, j] = (float(w @ oracle.solve_direct_f64(a, il, nth, nph).ravel()) -
                        float(w @ oracle.solve_direct_f64(b, il, nth, nph).ravel())) / (2 * h)
    assert np.all(np.linalg.norm(g - fd, axis=1) / np.linalg.norm(fd, axis=1) < 1e-6)
