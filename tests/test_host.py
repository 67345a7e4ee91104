"""Host-side logic: synthetic inputs, the config_hpc.cfg layout, file formats."""
import os

import numpy as np
import pytest

from soap_gpu_gb300 import config, synth


def test_cases_match_the_workload_definitions():
    c0, c1 = synth.make_case(0), synth.make_case(1)
    assert (c0.grid, c0.n, c0.n_eff, c0.n_mu, c0.n_phase, len(c0.velocities)) == (100, 20000, 19968, 10, 25, 81)
    assert (c1.grid, c1.n, c1.n_eff, c1.n_mu, c1.n_phase, len(c1.velocities)) == (300, 310000, 309760, 20, 100, 161)
    assert abs(c0.sigma_v - 1107.0446527883928) < 1e-9
    # vsini 2 km/s at the equator, inclination 90
    v_eq = 2 * np.pi * c0.radius_km / (c0.period * 86400.0)
    assert abs(v_eq - 2.0) < 1e-12
    # 1 % of the hemisphere for s = 0.1, 3 % for s = 0.1732
    assert abs(c1.regions[1, 2] ** 2 - 0.01) < 1e-12 and abs(c1.regions[0, 2] ** 2 - 0.03) < 1e-4


def test_generator_is_deterministic_and_sane():
    case = synth.small_case(seed=5, grid=20, n=3000, n_phase=2, n_mu=4)
    a, b = synth.generate(case), synth.generate(case)
    assert np.array_equal(a.q_norm, b.q_norm) and np.array_equal(a.mask_wave, b.mask_wave)
    assert a.q_norm.shape == (4, 3000)
    assert np.all(a.q_norm <= 1.0 + 1e-12) and np.all(a.q_norm >= 0.0)
    assert np.all(np.diff(a.mu_boundary) < 0)
    assert np.allclose(np.diff(a.wave), case.step)


def test_reference_layout_round_trip(tmp_path):
    case = synth.small_case(seed=2, grid=24, n=2600, n_phase=3, n_mu=4)
    inp = synth.generate(case)
    cfg_path = synth.write_reference_layout(inp, str(tmp_path))
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        rc = config.load_config(cfg_path)
        assert rc.grid == case.grid and rc.nrho == case.nrho
        assert abs(rc.inst_sigma - case.sigma_v) < 1e-9
        assert np.allclose(rc.regions, case.regions)
        assert len(rc.phases) == case.n_phase
        assert np.allclose(rc.velocities, case.velocities)
        for key, path in rc.cube_paths.items():
            arr = np.fromfile(path, dtype=np.float64).reshape(case.n_mu, case.n)
            assert np.array_equal(arr, getattr(inp, key)), key
        wave = np.fromfile(rc.input_dir + rc.wave_array_name)
        assert np.array_equal(wave, inp.wave)
        mu = np.fromfile(rc.input_dir + rc.mu_array_name)
        assert mu.size == case.n_mu - 1
        lbf = np.load(rc.input_dir + "Limb_brightening_info.npz")
        lb = config.lb_params(rc.t_star, lbf["LB_G2"], lbf["LB_K0"], lbf["LB_M0"], lbf["Temp_array"])
        assert np.allclose(lb, inp.lb)
        mask = np.loadtxt(rc.input_prefix + rc.mask_prefix + config.mask_template_name(rc.t_star))
        assert mask.shape[1] == 2
    finally:
        os.chdir(cwd)


def _narrow_rne(v):
    """The integer-pipe FP64 -> FP32 rounding of the FP32 cube conversion (fir.cu,
    soap_f64_to_f32), restated with numpy integers for normal-range results."""
    u = v.view(np.uint64)
    e = ((u >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    frac = u & np.uint64(0xFFFFFFFFFFFFF)
    keep = (frac >> np.uint64(29)).astype(np.uint64)
    rest = frac & np.uint64(0x1FFFFFFF)
    bits = (((e - 1023 + 127).astype(np.uint64)) << np.uint64(23)) | keep
    half = np.uint64(0x10000000)
    up = (rest > half) | ((rest == half) & ((keep & np.uint64(1)) == np.uint64(1)))
    bits = bits + up.astype(np.uint64)
    bits = bits | ((u >> np.uint64(32)) & np.uint64(0x80000000))
    return bits.astype(np.uint32).view(np.float32)


def test_fp32_narrowing_rounds_to_nearest_even():
    rng = np.random.default_rng(3)
    v = rng.uniform(-2.0, 2.0, 200000) * 10.0 ** rng.integers(-30, 30, 200000)
    # exact halfway cases (odd and even kept bit) and one below / above half
    base = rng.uniform(1.0, 2.0, 1000).astype(np.float32).astype(np.float64)
    ulp = np.spacing(base.astype(np.float32)).astype(np.float64)
    v = np.concatenate([v, base + ulp / 2, base + ulp * 1.5, np.nextafter(base + ulp / 2, 0),
                        np.nextafter(base + ulp / 2, 10), -(base + ulp / 2),
                        [np.float64(np.finfo(np.float32).max) * (1 + 2.0 ** -25)]])
    e = (v.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)
    v = v[(e >= 1023 - 126) & (e <= 1023 + 127)]
    with np.errstate(over="ignore"):
        ref = v.astype(np.float32)
    assert np.array_equal(_narrow_rne(v).view(np.uint32), ref.view(np.uint32))


def test_evolving_sizes_follow_the_evolution_driver():
    """run_all_SOAP_evo.py:16-20,213-230: t = (phase - phase_min) P, area = size^2 -
    rate t (spot_evo), size = sqrt(area)."""
    from soap_gpu_gb300.driver import evolving_sizes
    phases = np.arange(0.0, 2.0, 0.25)
    sizes = np.array([0.1, 0.17])
    got = evolving_sizes(phases, sizes, 25.0, -0.002)
    t = (phases - phases.min()) * 25.0
    for r, s0 in enumerate(sizes):
        amax = s0 ** 2
        assert np.array_equal(got[:, r], (amax - (-0.002) * t) ** 0.5)


def test_torch_default_stream_maps_to_the_legacy_handle(monkeypatch):
    torch = pytest.importorskip("torch")
    from soap_gpu_gb300 import api

    class _S:
        def __init__(self, h):
            self.cuda_stream = h

    monkeypatch.setattr(torch.cuda, "current_stream", lambda device=None: _S(0))
    assert api.torch_stream_handle(0) == 0x1      # cudaStreamLegacy, never the null handle
    monkeypatch.setattr(torch.cuda, "current_stream", lambda device=None: _S(0x5678))
    assert api.torch_stream_handle(0) == 0x5678
