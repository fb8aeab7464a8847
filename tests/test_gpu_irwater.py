"""IR sea-surface emissivity model on the GPU (batch emissivity NULL:
CRTM_Compute_IR_Water_SfcOptics / CRTM_IRSSEM at the sensor zenith angle)
against the oracle: forward with the oracle's IRSSEM emissivities, the
wind-speed Jacobian and (for a 'Nalli2' table) the water-temperature one
against central differences, the adjoint as the seeded K-matrix summed over
channels, and the refusals (clouds, microwave sensors, partial water cover)."""
import copy
import os
import shutil

import numpy as np
import pytest

from crtmv3_gb300 import coefficients as co, synthetic as sy

pytestmark = pytest.mark.gpu
SENSOR = "irsynth_c616"


@pytest.fixture(scope="module", params=["Nalli", "Nalli2"])
def water_dir(coeff_dir, tmp_path_factory, request):
    d = str(tmp_path_factory.mktemp("irw_" + request.param))
    for f in os.listdir(coeff_dir):
        if f.startswith(SENSOR) or f.startswith("mwsynth_c16"):
            shutil.copy(os.path.join(coeff_dir, f), d)
    sy.write_irwater_file(d, request.param)
    sy.write_cloud_files(d)
    return d, request.param


def _case(seed=501):
    atm, sfc, geo, opt = sy.clear_sky_workload(SENSOR, 6, 101, seed)
    sfc.land_coverage[:] = sfc.snow_coverage[:] = sfc.ice_coverage[:] = 0.0
    sfc.water_coverage[:] = 1.0
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    sfc.wind_speed = rng.uniform(0.5, 14.5, 6)
    sfc.wind_speed[4] = 20.0          # beyond the table: clamped, no wind dependence
    geo.sensor_zenith_angle[:] = rng.uniform(0.0, 65.0, 6)
    opt.emissivity = None
    return atm, sfc, geo, opt


def _oracle_bt(d, atm, sfc, geo, opt):
    from oracle.pyoracle import Oracle, irwater_emissivity
    sc = co.read_spccoeff(f"{d}/{SENSOR}.SpcCoeff.bin")
    o = copy.deepcopy(opt)
    o.emissivity = irwater_emissivity(f"{d}/{sy.IRWATER_FILE}", sfc, geo, sc.wavenumber)
    return Oracle(d, SENSOR).forward(atm, sfc, geo, o)[1]


@pytest.mark.parametrize("precision", [0, 1])
def test_forward_with_emissivity_model_matches_oracle(gpu_lib, water_dir, precision):
    d, _ = water_dir
    atm, sfc, geo, opt = _case()
    rts = gpu_lib.CRTM([SENSOR], d, precision).forward(atm, sfc, geo, opt)
    ref = _oracle_bt(d, atm, sfc, geo, opt)
    assert np.abs(rts.brightness_temperature - ref).max() <= (1e-4 if precision == 0 else 1e-2)
    # the default wind speed is 5 m/s
    s5 = copy.deepcopy(sfc)
    s5.wind_speed = None
    s6 = copy.deepcopy(sfc)
    s6.wind_speed = np.full(6, 5.0)
    h = gpu_lib.CRTM([SENSOR], d, precision)
    assert np.array_equal(h.forward(atm, s5, geo, opt).brightness_temperature,
                          h.forward(atm, s6, geo, opt).brightness_temperature)


def test_wind_and_temperature_jacobians_match_oracle_differences(gpu_lib, water_dir):
    d, classification = water_dir
    atm, sfc, geo, opt = _case()
    h = gpu_lib.CRTM([SENSOR], d, 0)
    km, rts = h.k_matrix(atm, sfc, geo, opt)
    step = 1e-3
    sp, sm = copy.deepcopy(sfc), copy.deepcopy(sfc)
    sp.wind_speed = sfc.wind_speed + step
    sm.wind_speed = sfc.wind_speed - step
    fd = (_oracle_bt(d, atm, sp, geo, opt) - _oracle_bt(d, atm, sm, geo, opt)) / (2 * step)
    assert np.abs(km.wind_speed - fd).max() <= 2e-5 * np.abs(fd).max()
    assert np.abs(km.wind_speed[4]).max() == 0.0     # clamped
    assert np.abs(km.wind_speed).max() > 1e-3
    sp, sm = copy.deepcopy(sfc), copy.deepcopy(sfc)
    sp.water_temperature = sfc.water_temperature + step
    sm.water_temperature = sfc.water_temperature - step
    fd = (_oracle_bt(d, atm, sp, geo, opt) - _oracle_bt(d, atm, sm, geo, opt)) / (2 * step)
    assert np.abs(km.water_temperature - fd).max() <= 2e-5 * np.abs(fd).max()
    # the adjoint: the seeded K-matrix summed over channels
    seed = np.random.Generator(np.random.PCG64(503)).standard_normal((6, km.wind_speed.shape[1]))
    k2, _ = h.k_matrix(atm, sfc, geo, opt, seed)
    ad, _ = h.adjoint(atm, sfc, geo, opt, seed)
    for f in ("wind_speed", "water_temperature"):
        assert np.abs(ad[f] - getattr(k2, f).sum(axis=1)).max() <= 1e-10 * np.abs(ad[f]).max(), f
    assert np.abs(ad["temperature"] - k2.temperature.sum(axis=1)).max() <= 1e-10 * np.abs(ad["temperature"]).max()
    # tangent linear along a wind-speed perturbation
    dv = np.random.Generator(np.random.PCG64(504)).standard_normal(6)
    tl_sfc = copy.deepcopy(sfc)
    for f in ("land_temperature", "water_temperature", "snow_temperature", "ice_temperature"):
        setattr(tl_sfc, f, np.zeros(6))
    tl_sfc.wind_speed = dv
    bt_tl, _ = h.tangent_linear(atm, sfc, geo, opt, None, tl_sfc, None)
    assert np.abs(bt_tl - km.wind_speed * dv[:, None]).max() <= 1e-12 * np.abs(bt_tl).max()


def test_emissivity_model_refusals(gpu_lib, water_dir):
    d, _ = water_dir
    atm, sfc, geo, opt = _case()
    h = gpu_lib.CRTM([SENSOR], d, 0)
    cloudy = copy.deepcopy(atm)
    sy.add_clouds(cloudy, (co.WATER_CLOUD,), 505, wc_scale=30.0)
    with pytest.raises(RuntimeError, match="clear-sky"):
        h.forward(cloudy, sfc, geo, opt)
    mixed = copy.deepcopy(sfc)
    mixed.water_coverage[2] = 0.5
    mixed.land_coverage[2] = 0.5
    with pytest.raises(RuntimeError, match="13"):
        h.forward(atm, mixed, geo, opt)
    mw = gpu_lib.CRTM(["mwsynth_c16"], d, 0)
    a2, s2, g2, o2 = sy.clear_sky_workload("mwsynth_c16", 2, 100, 506)
    o2.emissivity = None
    with pytest.raises(RuntimeError, match="infrared"):
        mw.forward(a2, s2, g2, o2)
    # the handle stays usable
    assert (h.forward(atm, sfc, geo, opt).status == 0).all()
