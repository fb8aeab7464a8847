"""GPU library vs the CPU FP64 oracle, through the C-ABI (host entry points).

Tolerances: the FP64 form must match the oracle within 1e-4 K in brightness
temperature and 1e-6 relative (to the largest Jacobian of the case) in the
K-matrix; the mixed form within 0.01 K and 1e-3 relative.
"""
import numpy as np
import pytest

from crtmv3_gb300 import synthetic as sy

pytestmark = pytest.mark.gpu

BT_TOL = {0: 1e-4, 1: 1e-2}
JAC_TOL = {0: 1e-6, 1: 1e-3}


def _case(sensor, P, nl, seed):
    return sy.clear_sky_workload(sensor, P, nl, seed)


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("sensor,nl", [("mwsynth_c22", 100), ("irsynth_c616", 101),
                                       ("mwsynth_c16", 90)])
def test_forward_matches_oracle(gpu_lib, coeff_dir, sensor, nl, precision):
    from oracle.pyoracle import Oracle
    atm, sfc, geo, opt = _case(sensor, 5, nl, 1234)
    h = gpu_lib.CRTM([sensor], coeff_dir, precision)
    rts = h.forward(atm, sfc, geo, opt)
    rad, bt = Oracle(coeff_dir, sensor).forward(atm, sfc, geo, opt)
    assert np.abs(rts.brightness_temperature - bt).max() < BT_TOL[precision]
    assert (rts.status == 0).all()


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("sensor,nl", [("mwsynth_c22", 100), ("irsynth_c616", 101),
                                       ("mwsynth_c16", 90)])
def test_k_matrix_matches_oracle(gpu_lib, coeff_dir, sensor, nl, precision):
    from oracle.pyoracle import Oracle
    atm, sfc, geo, opt = _case(sensor, 4, nl, 99)
    rng = np.random.default_rng(5)
    h = gpu_lib.CRTM([sensor], coeff_dir, precision)
    seed = rng.uniform(0.5, 1.5, (4, h.n_channels[0]))
    km, rts = h.k_matrix(atm, sfc, geo, opt, seed)
    ref = Oracle(coeff_dir, sensor).k_matrix(atm, sfc, geo, opt, seed)
    assert np.abs(rts.brightness_temperature - ref["bt"]).max() < BT_TOL[precision]
    assert _rel(km.temperature, ref["temperature_k"]) < JAC_TOL[precision]
    assert _rel(km.absorber, ref["absorber_k"]) < JAC_TOL[precision] * 10
    for j in range(atm.n_absorbers):
        assert _rel(km.absorber[:, :, j], ref["absorber_k"][:, :, j]) < JAC_TOL[precision] * 10
    assert _rel(km.water_temperature, ref["water_temperature_k"]) < JAC_TOL[precision]
    assert _rel(km.surface_emissivity, ref["surface_emissivity_k"]) < JAC_TOL[precision]


@pytest.mark.parametrize("precision", [0, 1])
def test_adjoint_matches_oracle(gpu_lib, coeff_dir, precision):
    from oracle.pyoracle import Oracle
    sensor = "irsynth_c616"
    atm, sfc, geo, opt = _case(sensor, 3, 101, 7)
    h = gpu_lib.CRTM([sensor], coeff_dir, precision)
    seed = np.random.default_rng(1).normal(size=(3, h.n_channels[0]))
    out, rts = h.adjoint(atm, sfc, geo, opt, seed)
    ref = Oracle(coeff_dir, sensor).adjoint(atm, sfc, geo, opt, seed)
    assert _rel(out["temperature"], ref["temperature_ad"]) < JAC_TOL[precision] * 10
    assert _rel(out["absorber"], ref["absorber_ad"]) < JAC_TOL[precision] * 10
    assert _rel(out["water_temperature"], ref["water_temperature_ad"]) < JAC_TOL[precision] * 10


def test_ragged_layers_and_surface_pressure(gpu_lib, coeff_dir):
    """Uneven layer counts in one batch and a surface above the ODPS surface level."""
    from oracle.pyoracle import Oracle
    sensor = "irsynth_c616"
    nl = np.array([60, 137, 101, 75, 120])
    atm, sfc, geo = sy.generate_profiles(5, nl, sy.absorber_set(1), 77, p_sfc=1013.0)
    opt = sy.OptionsBatch(emissivity=sy.emissivity_for(2, 5, 616, 3))
    h = gpu_lib.CRTM([sensor], coeff_dir, 0)
    km, rts = h.k_matrix(atm, sfc, geo, opt)
    ref = Oracle(coeff_dir, sensor).k_matrix(atm, sfc, geo, opt)
    assert np.abs(rts.brightness_temperature - ref["bt"]).max() < 1e-4
    assert _rel(km.temperature, ref["temperature_k"]) < 1e-6
    # padding layers are zero
    for m, n in enumerate(nl):
        assert np.all(km.temperature[m, :, n:] == 0.0)


def test_odd_sizes(gpu_lib, coeff_dir):
    """One profile, and channel counts that are not multiples of the block size."""
    from oracle.pyoracle import Oracle
    for sensor in ("mwsynth_c22", "mwsynth_c16"):
        atm, sfc, geo, opt = _case(sensor, 1, 100, 3)
        h = gpu_lib.CRTM([sensor], coeff_dir, 0)
        km, rts = h.k_matrix(atm, sfc, geo, opt)
        ref = Oracle(coeff_dir, sensor).k_matrix(atm, sfc, geo, opt)
        assert np.abs(rts.brightness_temperature - ref["bt"]).max() < 1e-4
        assert _rel(km.temperature, ref["temperature_k"]) < 1e-6


def test_k_matrix_absorber_selection(gpu_lib, coeff_dir):
    """Only the selected absorber Jacobians are written, in the selected order."""
    from oracle.pyoracle import Oracle
    sensor = "irsynth_c616"
    atm, sfc, geo, opt = _case(sensor, 2, 101, 11)
    h = gpu_lib.CRTM([sensor], coeff_dir, 0)
    ids = list(atm.absorber_id)
    sel = [ids.index(3), ids.index(1)]
    km, rts = h.k_matrix(atm, sfc, geo, opt, k_absorbers=sel)
    ref = Oracle(coeff_dir, sensor).k_matrix(atm, sfc, geo, opt)
    assert km.absorber.shape[2] == 2
    for j, ja in enumerate(sel):
        assert _rel(km.absorber[:, :, j], ref["absorber_k"][:, :, ja]) < 1e-5


def test_device_entry_points_and_stage_times(gpu_lib, coeff_dir):
    """The device-resident K-matrix equals the host call; stage timing covers every stage."""
    import torch
    sensor = "irsynth_c616"
    atm, sfc, geo, opt = _case(sensor, 3, 101, 21)
    h = gpu_lib.CRTM([sensor], coeff_dir, 1)
    km, rts = h.k_matrix(atm, sfc, geo, opt)
    import bench
    b, keep, t = bench.device_batch(torch, h, atm, sfc, geo, opt, torch.device("cuda"))
    out = bench.k_outputs(torch, 3, h.n_channels[0], atm.max_layers, atm.n_absorbers, torch.device("cuda"))
    h.set_profiling(True)
    h.k_matrix_device(b, out, None, 0, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    st = h.stage_times()
    assert np.array_equal(out["bt"].cpu().numpy(), rts.brightness_temperature)
    assert np.array_equal(out["temperature_k"].cpu().numpy(), km.temperature)
    for s in ("prep", "absorb_fwd", "column", "absorb_ad", "map_out"):
        assert st[s][1] >= 1 and st[s][0] > 0.0


def test_mixed_against_fp64_on_many_profiles(gpu_lib, coeff_dir):
    """The mixed form against the FP64 form on 300 profiles (rare layer states,
    e.g. T within a few mK of the reference temperature, show up only in
    larger batches): 0.01 K in BT, 1e-3 relative in the Jacobians."""
    sensor = "irsynth_c616"
    atm, sfc, geo, opt = _case(sensor, 300, 101, 23)
    ref = gpu_lib.CRTM([sensor], coeff_dir, 0).k_matrix(atm, sfc, geo, opt)
    mix = gpu_lib.CRTM([sensor], coeff_dir, 1).k_matrix(atm, sfc, geo, opt)
    assert np.abs(mix[1].brightness_temperature - ref[1].brightness_temperature).max() <= BT_TOL[1]
    for f in ("temperature", "absorber", "water_temperature"):
        assert _rel(getattr(mix[0], f), getattr(ref[0], f)) <= JAC_TOL[1], f


@pytest.mark.parametrize("precision", [0, 1])
def test_k_matrix_c2211_bench_sensor_matches_oracle(gpu_lib, coeff_dir, precision):
    """The clear-sky IR workload's own sensor (2211 channels, ODPS group 1, 6
    absorbers, 101 layers) with the H2O and O3 Jacobians that its K-matrix
    returns, against the oracle computing the same two."""
    from crtmv3_gb300 import coefficients as co
    from oracle.pyoracle import Oracle
    sensor = "irsynth_c2211"
    atm, sfc, geo, opt = _case(sensor, 4, 101, 2211)
    ids = list(atm.absorber_id)
    sel = [ids.index(co.H2O_ID), ids.index(co.O3_ID)]
    h = gpu_lib.CRTM([sensor], coeff_dir, precision)
    km, rts = h.k_matrix(atm, sfc, geo, opt, k_absorbers=sel)
    ref = Oracle(coeff_dir, sensor).k_matrix(atm, sfc, geo, opt, n_threads=4, k_absorbers=sel)
    assert np.abs(rts.brightness_temperature - ref["bt"]).max() < BT_TOL[precision]
    assert (rts.status == 0).all()
    assert _rel(km.temperature, ref["temperature_k"]) < JAC_TOL[precision]
    for i, j in enumerate(sel):
        assert _rel(km.absorber[:, :, i], ref["absorber_k"][:, :, j]) < JAC_TOL[precision]
    others = [j for j in range(atm.n_absorbers) if j not in sel]
    assert not ref["absorber_k"][:, :, others].any()
    assert _rel(km.water_temperature, ref["water_temperature_k"]) < JAC_TOL[precision]
    assert _rel(km.surface_emissivity, ref["surface_emissivity_k"]) < JAC_TOL[precision]
