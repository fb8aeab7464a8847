"""Cloudy and aerosol K-matrix on the GPU against the oracle's cloudy
K-matrix (the CPU reverse mode of the reference's ADA adding, MOM, phase
normalisation, combine and LUT adjoints, itself pinned to central
differences of the oracle's forward in tests/test_oracle_scatter.py).

Tolerances, relative to the largest Jacobian of each output:
* FP64 form: brightness temperature within 1e-4 K, Jacobians within 1e-6;
* mixed form (FP32 gas optics and layer solver, FP64 adding): 0.01 K and 1e-3.
"""
import numpy as np
import pytest

from crtmv3_gb300 import coefficients as co, synthetic as sy

pytestmark = pytest.mark.gpu

BT_TOL = {0: 1e-4, 1: 1e-2}
JAC_TOL = {0: 1e-6, 1: 1e-3}
SPECIES = (("cloud_water_content", "cloud_water_content_k"), ("cloud_effective_radius", "cloud_effective_radius_k"),
           ("aerosol_concentration", "aerosol_concentration_k"),
           ("aerosol_effective_radius", "aerosol_effective_radius_k"))


@pytest.fixture(scope="module")
def cloud_dir(coeff_dir):
    sy.write_cloud_files(coeff_dir)
    sy.write_aerosol_files(coeff_dir)
    return coeff_dir


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _case(sensor, n_streams, aer, seed, P=3, nl=100):
    mw = sensor.startswith("mw")
    types = ((co.WATER_CLOUD, co.ICE_CLOUD, co.RAIN_CLOUD, co.SNOW_CLOUD, co.GRAUPEL_CLOUD) if mw
             else (co.WATER_CLOUD, co.ICE_CLOUD))
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, P, nl, seed, cloud_types=types, wc_scale=3.0,
                                            n_streams=n_streams)
    if aer:
        sy.add_aerosols(atm, sy.AEROSOL_TYPES, seed + 1, load_scale=5.0)
    return atm, sfc, geo, opt


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("sensor,n_streams,aer", [("irsynth_c616", None, True), ("mwsynth_c22", None, False),
                                                  ("irsynth_c616", 16, False), ("mwsynth_c16", 8, False),
                                                  ("irsynth_c2211", None, False)])
def test_cloudy_k_matrix_matches_oracle(gpu_lib, cloud_dir, sensor, n_streams, aer, precision):
    from oracle.pyoracle import Oracle
    atm, sfc, geo, opt = _case(sensor, n_streams, aer, 401, P=2 if sensor.endswith("2211") else 3)
    rng = np.random.default_rng(7)
    h = gpu_lib.CRTM([sensor], cloud_dir, precision)
    seed = rng.uniform(0.5, 1.5, (atm.n_profiles, h.n_channels[0]))
    km, rts = h.k_matrix(atm, sfc, geo, opt, seed)
    ref = Oracle(cloud_dir, sensor).k_matrix_scatter(atm, sfc, geo, opt, f"{cloud_dir}/CloudCoeff.bin",
                                                     f"{cloud_dir}/AerosolCoeff.bin" if aer else None,
                                                     bt_k=seed, n_threads=8)
    assert (rts.status == 0).all()
    assert np.abs(rts.brightness_temperature - ref["bt"]).max() < BT_TOL[precision]
    tol = JAC_TOL[precision]
    assert _rel(km.temperature, ref["temperature_k"]) < tol
    for j in range(atm.n_absorbers):
        assert _rel(km.absorber[:, :, j], ref["absorber_k"][:, :, j]) < tol * 10, j
    assert _rel(km.water_temperature, ref["water_temperature_k"]) < tol
    assert _rel(km.surface_emissivity, ref["surface_emissivity_k"]) < tol
    for field, key in SPECIES:
        got = getattr(km, field, None)
        if got is None or not ref[key].size:
            continue
        # relative to the largest Jacobian times the variable (the response to a relative change)
        x = getattr(atm, field)[:, None]
        scale = max(np.abs(ref[key] * x).max(), 1e-300)
        assert np.abs((got - ref[key]) * x).max() <= tol * scale, field


@pytest.mark.parametrize("precision", [0, 1])
def test_ragged_batch_buckets_match_oracle(gpu_lib, cloud_dir, precision):
    """A batch whose profiles alternate between clear, cloudy on the stream
    rule and cloudy with Options%n_Streams 16: the library runs each bucket as
    its own pipeline (clear-sky, 5-angle and 10-angle scattering kernels) in
    the batch's buffers.  Every profile's outputs match the oracle, the clear
    profiles' cloud Jacobians are zero, and the host entry point (outputs
    copied back after all buckets) agrees with the device one."""
    import torch
    from oracle.pyoracle import Oracle
    sensor = "irsynth_c616"
    P = 6
    atm, sfc, geo, opt = _case(sensor, None, False, 411, P=P, nl=90)
    atm.n_clouds[[0, 3]] = 0
    ns = np.array([0, 0, 16, 0, 0, 16], np.int32)
    opt.use_n_streams, opt.n_streams = ns > 0, ns
    h = gpu_lib.CRTM([sensor], cloud_dir, precision)
    km, rts = h.k_matrix(atm, sfc, geo, opt)
    ref = Oracle(cloud_dir, sensor).k_matrix_scatter(atm, sfc, geo, opt, f"{cloud_dir}/CloudCoeff.bin", None,
                                                     n_threads=8)
    assert (rts.status == 0).all()
    assert np.abs(rts.brightness_temperature - ref["bt"]).max() < BT_TOL[precision]
    tol = JAC_TOL[precision]
    assert _rel(km.temperature, ref["temperature_k"]) < tol
    assert _rel(km.water_temperature, ref["water_temperature_k"]) < tol
    x = atm.cloud_water_content[:, None]
    assert np.abs((km.cloud_water_content - ref["cloud_water_content_k"]) * x).max() <= \
        tol * np.abs(ref["cloud_water_content_k"] * x).max()
    for p in (0, 3):
        assert not km.cloud_water_content[p].any() and not km.cloud_effective_radius[p].any()
        assert not km.cloud_fraction[p].any()
    # the device entry point on the same batch
    dev = torch.device("cuda")
    t = {}
    for k in ("level_pressure", "pressure", "temperature", "absorber", "cloud_water_content",
              "cloud_effective_radius", "cloud_fraction"):
        t[k] = torch.from_numpy(np.ascontiguousarray(getattr(atm, k), np.float64)).to(dev)
    for k in ("n_layers", "n_clouds", "cloud_type"):
        t[k] = torch.from_numpy(np.ascontiguousarray(getattr(atm, k), np.int32)).to(dev)
    for f in ("land_coverage", "water_coverage", "snow_coverage", "ice_coverage", "land_temperature",
              "water_temperature", "snow_temperature", "ice_temperature"):
        t[f] = torch.from_numpy(np.ascontiguousarray(getattr(sfc, f))).to(dev)
    for f in ("sensor_zenith_angle", "source_zenith_angle", "surface_altitude"):
        t[f] = torch.from_numpy(np.ascontiguousarray(getattr(geo, f))).to(dev)
    t["emissivity"] = torch.from_numpy(np.ascontiguousarray(opt.emissivity)).to(dev)
    t["n_streams"] = torch.from_numpy(ns).to(dev)
    b, keep = h.device_batch(t, atm.absorber_id)
    L, K, NC = h.n_channels[0], atm.max_layers, atm.cloud_type.shape[1]
    f64 = dict(dtype=torch.float64, device=dev)
    o = dict(radiance=torch.full((P, L), np.nan, **f64), bt=torch.full((P, L), np.nan, **f64),
             temperature_k=torch.full((P, L, K), np.nan, **f64),
             absorber_k=torch.full((P, L, atm.n_absorbers, K), np.nan, **f64),
             water_temperature_k=torch.full((P, L), np.nan, **f64),
             surface_emissivity_k=torch.full((P, L), np.nan, **f64),
             cloud_water_content_k=torch.full((P, L, NC, K), np.nan, **f64),
             cloud_effective_radius_k=torch.full((P, L, NC, K), np.nan, **f64),
             cloud_fraction_k=torch.full((P, L, K), np.nan, **f64),
             status=torch.full((P,), -1, dtype=torch.int32, device=dev))
    h.k_matrix_device(b, o, None, 0, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(o["bt"].cpu().numpy(), rts.brightness_temperature)
    assert np.array_equal(o["temperature_k"].cpu().numpy(), km.temperature)
    assert np.array_equal(o["cloud_water_content_k"].cpu().numpy(), km.cloud_water_content)
    assert not o["cloud_fraction_k"].isnan().any()
