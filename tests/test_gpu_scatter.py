"""Cloudy forward (cloud LUT, combine, ADA) on the GPU against the oracle.

Tolerances: 1e-4 K in brightness temperature in the FP64 form.  In the mixed
form the gas layer optical depths come from the FP32 regression (the
scattering solver is FP64 in both forms), so 0.01 K as for clear sky.
"""
import copy

import numpy as np
import pytest

from crtmv3_gb300 import coefficients as co, synthetic as sy

pytestmark = pytest.mark.gpu

BT_TOL = {0: 1e-4, 1: 1e-2}


@pytest.fixture(scope="module")
def cloud_dir(coeff_dir):
    sy.write_cloud_files(coeff_dir)
    return coeff_dir


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("sensor,nl,n_streams,wc_scale", [
    ("mwsynth_c16", 100, None, 1.0),      # config C3 distributions, stream rule
    ("mwsynth_c16", 100, None, 300.0),    # thick clouds
    ("mwsynth_c16", 100, 8, 100.0),
    ("mwsynth_c16", 100, 16, 100.0),
    ("irsynth_c616", 101, None, 100.0),
    ("mwsynth_c22", 100, None, 100.0)])
def test_cloudy_forward_matches_oracle(gpu_lib, cloud_dir, precision, sensor, nl, n_streams, wc_scale):
    from oracle.pyoracle import Oracle
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 6, nl, 61, wc_scale=wc_scale, n_streams=n_streams)
    atm.n_clouds[2] = 0   # one clear profile in the batch
    _, ref = Oracle(cloud_dir, sensor).forward_scatter(atm, sfc, geo, opt, f"{cloud_dir}/CloudCoeff.bin")
    h = gpu_lib.CRTM([sensor], cloud_dir, precision)
    rts = h.forward(atm, sfc, geo, opt)
    assert np.abs(rts.brightness_temperature - ref).max() <= BT_TOL[precision]
    assert (rts.status == 0).all()


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("sensor,nl,n_streams", [("mwsynth_c16", 100, None), ("mwsynth_c16", 100, 16),
                                                 ("irsynth_c616", 101, None)])
def test_soi_forward_matches_oracle(gpu_lib, cloud_dir, precision, sensor, nl, n_streams):
    """Options%RT_Algorithm_Id = RT_SOI for half of the profiles, ADA for the rest."""
    from oracle.pyoracle import Oracle
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 6, nl, 67, wc_scale=100.0, n_streams=n_streams)
    opt.rt_algorithm_id = np.array([168, 56, 168, 56, 168, 168], np.int32)
    atm.n_clouds[4] = 0
    _, ref = Oracle(cloud_dir, sensor).forward_scatter(atm, sfc, geo, opt, f"{cloud_dir}/CloudCoeff.bin")
    rts = gpu_lib.CRTM([sensor], cloud_dir, precision).forward(atm, sfc, geo, opt)
    assert np.abs(rts.brightness_temperature - ref).max() <= BT_TOL[precision]


def test_ragged_cloudy_batch(gpu_lib, cloud_dir):
    from oracle.pyoracle import Oracle
    sensor = "mwsynth_c16"
    nl = np.array([60, 137, 101, 75, 120])
    atm, sfc, geo = sy.generate_profiles(5, nl, (co.H2O_ID,), 62, p_sfc=1013.0)
    opt = sy.OptionsBatch(emissivity=sy.emissivity_for(co.MICROWAVE_SENSOR, 5, 16, 63))
    sy.add_clouds(atm, (co.RAIN_CLOUD, co.SNOW_CLOUD, co.GRAUPEL_CLOUD), 64, wc_scale=200.0)
    _, ref = Oracle(cloud_dir, sensor).forward_scatter(atm, sfc, geo, opt, f"{cloud_dir}/CloudCoeff.bin")
    rts = gpu_lib.CRTM([sensor], cloud_dir, 0).forward(atm, sfc, geo, opt)
    assert np.abs(rts.brightness_temperature - ref).max() <= BT_TOL[0]


def test_isothermal_enclosure_on_gpu(gpu_lib, cloud_dir, tmp_path):
    """Kirchhoff check of the GPU solver itself: an isothermal scene whose
    cosmic background is B(T) gives BT = T for any cloud and stream count."""
    import shutil
    sensor = "mwsynth_c16"
    sc = co.read_spccoeff(f"{cloud_dir}/{sensor}.SpcCoeff.bin")
    te = sc.band_c1 + sc.band_c2 * 250.0
    sc.cosmic_background_radiance = sc.planck_c1 / (np.exp(sc.planck_c2 / te) - 1.0)
    co.write_spccoeff(str(tmp_path / f"{sensor}.SpcCoeff.bin"), sc)
    shutil.copy(f"{cloud_dir}/{sensor}.TauCoeff.bin", tmp_path / f"{sensor}.TauCoeff.bin")
    shutil.copy(f"{cloud_dir}/CloudCoeff.bin", tmp_path / "CloudCoeff.bin")
    for ns in (None, 16):
        atm, sfc, geo, opt = sy.cloudy_workload(sensor, 4, 100, 66, wc_scale=300.0, n_streams=ns)
        for m in range(4):
            atm.temperature[m, :atm.n_layers[m]] = 250.0
        sfc.water_temperature[:] = 250.0
        opt.emissivity[:] = 1.0
        rts = gpu_lib.CRTM([sensor], str(tmp_path), 0).forward(atm, sfc, geo, opt)
        assert np.abs(rts.brightness_temperature - 250.0).max() < 1e-8


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("clouds,soi", [(True, False), (False, False), (True, True)])
def test_aerosols_match_oracle(gpu_lib, cloud_dir, precision, clouds, soi):
    """Config C4 shape: IR sensor, liquid and ice clouds plus dust, sea salt and
    sulfate (AerosolCoeff scheme 'CRTM'); aerosol-only profiles too."""
    from oracle.pyoracle import Oracle
    sensor = "irsynth_c616"
    apath = sy.write_aerosol_files(cloud_dir)
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, 5, 101, 68)
    if clouds:
        sy.add_clouds(atm, (co.WATER_CLOUD, co.ICE_CLOUD), 69, wc_scale=50.0)
    sy.add_aerosols(atm, sy.AEROSOL_TYPES, 70, load_scale=20.0)
    atm.n_aerosols[3] = 0
    if soi:
        opt.rt_algorithm_id = np.array([168, 56, 168, 168, 56], np.int32)
    _, ref = Oracle(cloud_dir, sensor).forward_scatter(atm, sfc, geo, opt,
                                                       f"{cloud_dir}/CloudCoeff.bin" if clouds else None, apath)
    rts = gpu_lib.CRTM([sensor], cloud_dir, precision).forward(atm, sfc, geo, opt)
    assert np.abs(rts.brightness_temperature - ref).max() <= BT_TOL[precision]


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("scheme,soi", [("CMAQ", False), ("GOCART-GEOS5", False), ("NAAPS", True),
                                        ("CMAQ", True)])
def test_aerosol_schemes_match_oracle(gpu_lib, cloud_dir, precision, scheme, soi):
    """CRTM_Init's Aerosol_Model: 'CMAQ' interpolates the LUT in (frequency,
    radius, sigma) with Effective_Variance as sigma, 'GOCART-GEOS5' / 'NAAPS' in
    (frequency, RH) with the layers' Relative_Humidity; liquid and ice clouds
    beside the aerosols, one aerosol-only and one clear profile."""
    from oracle.pyoracle import Oracle
    sensor = "irsynth_c616"
    apath = sy.write_aerosol_files(cloud_dir, scheme)
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, 5, 101, 71)
    sy.add_clouds(atm, (co.WATER_CLOUD, co.ICE_CLOUD), 72, wc_scale=50.0)
    sy.add_aerosols(atm, sy.AEROSOL_TYPES, 73, load_scale=20.0)
    sy.add_aerosol_scheme_inputs(atm, 74)
    atm.n_clouds[1] = 0
    atm.n_aerosols[3] = atm.n_clouds[3] = 0
    if soi:
        opt.rt_algorithm_id = np.array([168, 56, 168, 168, 56], np.int32)
    _, ref = Oracle(cloud_dir, sensor).forward_scatter(atm, sfc, geo, opt, f"{cloud_dir}/CloudCoeff.bin", apath,
                                                       aerosol_scheme=scheme)
    h = gpu_lib.CRTM([sensor], cloud_dir, precision, aerosol_model=scheme,
                     aerosol_coeff_file=sy.aerosol_file_name(scheme))
    rts = h.forward(atm, sfc, geo, opt)
    assert np.abs(rts.brightness_temperature - ref).max() <= BT_TOL[precision]
    # the scheme's coordinate matters: without it the radiances move
    bare = copy.deepcopy(atm)
    bare.aerosol_effective_variance = bare.relative_humidity = None
    assert np.abs(h.forward(bare, sfc, geo, opt).brightness_temperature - rts.brightness_temperature).max() > 1e-3


def test_unknown_aerosol_model_is_refused(gpu_lib, cloud_dir):
    with pytest.raises(RuntimeError, match="Aerosol_Model"):
        gpu_lib.CRTM(["irsynth_c616"], cloud_dir, 0, aerosol_model="OPAC")


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("overlap", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("sensor", ["mwsynth_c16", "irsynth_c616"])
def test_fractional_cloud_cover_matches_oracle(gpu_lib, cloud_dir, precision, overlap, sensor):
    """Cloud_Fraction in (0.05, 0.95) in cloudy layers: the clear and the
    scaled cloudy column mixed by the overlap scheme's total cover; ADA and
    SOI profiles, one profile with fraction 1, one whose clouds are dropped
    (fraction below 1e-12), one clear."""
    from oracle.pyoracle import Oracle
    nl = 100 if sensor.startswith("mw") else 101
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 8, nl, 71, cloud_types=(co.WATER_CLOUD, co.ICE_CLOUD, co.RAIN_CLOUD),
                                            wc_scale=60.0)
    sy.add_clouds(atm, (co.WATER_CLOUD, co.ICE_CLOUD, co.RAIN_CLOUD), 72, wc_scale=60.0, cover=(0.05, 0.95))
    atm.cloud_fraction[1] = np.where(atm.cloud_fraction[1] > 0, 1.0, 0.0)
    atm.cloud_fraction[2] *= 1e-13
    atm.n_clouds[3] = 0
    opt.overlap_id = np.full(8, overlap, np.int32)
    opt.rt_algorithm_id = np.array([56, 56, 56, 56, 168, 168, 56, 168], np.int32)
    _, ref = Oracle(cloud_dir, sensor).forward_scatter(atm, sfc, geo, opt, f"{cloud_dir}/CloudCoeff.bin")
    rts = gpu_lib.CRTM([sensor], cloud_dir, precision).forward(atm, sfc, geo, opt)
    assert np.abs(rts.brightness_temperature - ref).max() <= BT_TOL[precision]


def test_null_cloud_fraction_is_one_cloudy_column(gpu_lib, cloud_dir):
    atm, sfc, geo, opt = sy.cloudy_workload("mwsynth_c16", 4, 100, 73, wc_scale=100.0)
    h = gpu_lib.CRTM(["mwsynth_c16"], cloud_dir, 0)
    bt1 = h.forward(atm, sfc, geo, opt).brightness_temperature
    atm.cloud_fraction = None
    bt0 = h.forward(atm, sfc, geo, opt).brightness_temperature
    assert np.abs(bt1 - bt0).max() == 0.0


def test_invalid_overlap_id_fails(gpu_lib, cloud_dir):
    atm, sfc, geo, opt = sy.cloudy_workload("mwsynth_c16", 3, 100, 74, wc_scale=100.0)
    sy.add_clouds(atm, (co.WATER_CLOUD,), 75, wc_scale=100.0, cover=(0.2, 0.8))
    opt.overlap_id = np.array([4, 0, 4], np.int32)
    h = gpu_lib.CRTM(["mwsynth_c16"], cloud_dir, 0)
    with pytest.raises(RuntimeError, match="Overlap_Id"):
        h.forward(atm, sfc, geo, opt)
    opt.overlap_id = None
    assert (h.forward(atm, sfc, geo, opt).status == 0).all()
