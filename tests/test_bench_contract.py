"""Host-side pieces of bench.py's JSON contract that need no GPU."""
import bench


def test_clock_parser_reads_clocks_and_slowdown_reasons():
    lines = [
        "0, 2070, 2070, 900.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 2055, 2070, 1100.5, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 1980, 2070, 1350.0, 0x0000000000000008, Active, Not Active, Not Active, Not Active",
        "garbage line",
        "0, [N/A], 2070, 0.0, 0x0, Not Active, Not Active, Not Active, Not Active",
    ]
    sm, mx, reasons = bench.ClockSampler.parse(lines)
    assert sm == [2070.0, 2055.0, 1980.0]
    assert mx == [2070.0, 2070.0, 2070.0]
    assert reasons == {"sw_power_cap", "hw_slowdown"}


def test_clock_sampler_without_nvidia_smi_reports_unavailable(monkeypatch):
    def no_smi(*a, **k):
        raise FileNotFoundError("nvidia-smi")

    monkeypatch.setattr(bench.subprocess, "Popen", no_smi)
    c = bench.ClockSampler(0)
    assert c.stop() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}


def test_point_dirs_per_step_is_the_headline_unit():
    from wavefiber3d_gb300 import api
    illum = api.Illumination(bench.LAMBDAS, [0.0], [0.0], api.PO_POL_TM, bench.ETA, bench.SIGMA)
    # N points x 180 x 360 directions x 25 wavelengths x 1 incidence x 1 polarisation
    assert bench.point_dirs_per_step(illum) == 400000 * 180 * 360 * 25


def test_ellipsoid_workload_in_the_reference_theta_mode():
    # --theta-mode reference: the reference's own grids, whose odd levels
    # (197 and 37 columns) run on the tensor path with a phantom partner column
    from wavefiber3d_gb300 import api
    _, cfg, illum = bench.make_workload("split_bf16", "tensor", 0, 1, 1, "reference")
    assert cfg.theta_mode == api.PO_THETA_REFERENCE and cfg.interp_method == api.PO_INTERP_TENSOR
    assert list(cfg.n_phi) == [360, 197, 108, 62, 37, 24]
    assert illum.n_patterns == 1
