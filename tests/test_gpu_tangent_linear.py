"""CRTM_Tangent_Linear on the GPU: against central differences of the forward
and, through the dot-product test, against the adjoint (<TL dx, y> = <dx, AD y>,
the reference's test_AD.f90:216-377 method).  Clear sky, clouds with
fractional cover, and aerosols (schemes 'CRTM', 'CMAQ' with Effective_Variance
and 'GOCART-GEOS5' with Relative_Humidity perturbed); FP64 form."""
import copy
import types

import numpy as np
import pytest

from crtmv3_gb300 import coefficients as co, synthetic as sy

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cloud_dir(coeff_dir):
    sy.write_cloud_files(coeff_dir)
    for scheme in co.AEROSOL_SCHEMES:
        sy.write_aerosol_files(coeff_dir, scheme)
    return coeff_dir


SCHEME = {"cmaq": "CMAQ", "gocart": "GOCART-GEOS5"}


def _handle(gpu_lib, cloud_dir, sensor, kind):
    scheme = SCHEME.get(kind)
    if scheme is None:
        return gpu_lib.CRTM([sensor], cloud_dir, 0)
    return gpu_lib.CRTM([sensor], cloud_dir, 0, aerosol_model=scheme, aerosol_coeff_file=sy.aerosol_file_name(scheme))


def _case(kind):
    if kind == "clear":
        return ("irsynth_c616",) + sy.clear_sky_workload("irsynth_c616", 5, 101, 401)
    if kind == "clouds":
        sensor = "mwsynth_c16"
        atm, sfc, geo, opt = sy.cloudy_workload(sensor, 5, 100, 402, wc_scale=100.0)
        sy.add_clouds(atm, (co.WATER_CLOUD, co.RAIN_CLOUD, co.SNOW_CLOUD), 403, wc_scale=100.0, cover=(0.2, 0.9))
        atm.n_clouds[3] = 0
        return (sensor, atm, sfc, geo, opt)
    sensor = "irsynth_c616"
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, 4, 101, 404)
    sy.add_clouds(atm, (co.WATER_CLOUD, co.ICE_CLOUD), 405, wc_scale=30.0)
    sy.add_aerosols(atm, sy.AEROSOL_TYPES, 406, load_scale=20.0)
    if kind in SCHEME:
        sy.add_aerosol_scheme_inputs(atm, 410)
    return (sensor, atm, sfc, geo, opt)


def _direction(atm, sfc, P, L, seed):
    """A random perturbation direction, relative to the inputs where that matters."""
    rng = np.random.Generator(np.random.PCG64(seed))
    d = types.SimpleNamespace()
    d.temperature = rng.standard_normal(atm.temperature.shape)
    d.absorber = rng.standard_normal(atm.absorber.shape) * atm.absorber * 0.05
    for f in ("cloud_water_content", "cloud_effective_radius", "aerosol_concentration", "aerosol_effective_radius",
              "aerosol_effective_variance", "relative_humidity"):
        v = getattr(atm, f)
        setattr(d, f, None if v is None else rng.uniform(-0.05, 0.05, v.shape) * v)
    d.cloud_fraction = None if atm.cloud_fraction is None else \
        np.where(atm.cloud_fraction > 0, rng.uniform(-0.02, 0.02, atm.cloud_fraction.shape), 0.0)
    s = types.SimpleNamespace(land_temperature=rng.standard_normal(P), water_temperature=rng.standard_normal(P),
                              snow_temperature=rng.standard_normal(P), ice_temperature=rng.standard_normal(P))
    e = rng.uniform(-0.01, 0.01, (P, L))
    return d, s, e


def _moved(atm, sfc, opt, d, s, e, h):
    a, f, o = copy.deepcopy(atm), copy.deepcopy(sfc), copy.deepcopy(opt)
    for name in ("temperature", "absorber", "cloud_water_content", "cloud_effective_radius", "cloud_fraction",
                 "aerosol_concentration", "aerosol_effective_radius", "aerosol_effective_variance",
                 "relative_humidity"):
        dv = getattr(d, name)
        if dv is not None and getattr(a, name) is not None:
            setattr(a, name, getattr(a, name) + h * dv)
    for name in ("land_temperature", "water_temperature", "snow_temperature", "ice_temperature"):
        setattr(f, name, getattr(f, name) + h * getattr(s, name))
    o.emissivity = o.emissivity + h * e
    return a, f, o


@pytest.mark.parametrize("kind", ["clear", "clouds", "aerosols", "cmaq", "gocart"])
def test_tangent_linear_matches_central_differences(gpu_lib, cloud_dir, kind):
    sensor, atm, sfc, geo, opt = _case(kind)
    h = _handle(gpu_lib, cloud_dir, sensor, kind)
    P, L = atm.n_profiles, h.n_channels[0]
    sfc.land_coverage[:] = 0.2
    sfc.water_coverage[:] = 0.6
    sfc.snow_coverage[:] = 0.1
    sfc.ice_coverage[:] = 0.1
    d, s, e = _direction(atm, sfc, P, L, 407)
    bt_tl, rts = h.tangent_linear(atm, sfc, geo, opt, d, s, e)
    fw = h.forward(atm, sfc, geo, opt)
    assert np.abs(rts.brightness_temperature - fw.brightness_temperature).max() < 1e-9
    # central differences with two steps; an element whose difference straddles a
    # kink of the model (an optical-depth clamp) disagrees at one step only
    errs = []
    for step in (1e-3, 1e-4):
        bp = h.forward(*_moved(atm, sfc, opt, d, s, e, step)[:2], geo, _moved(atm, sfc, opt, d, s, e, step)[2])
        bm = h.forward(*_moved(atm, sfc, opt, d, s, e, -step)[:2], geo, _moved(atm, sfc, opt, d, s, e, -step)[2])
        fd = (bp.brightness_temperature - bm.brightness_temperature) / (2 * step)
        errs.append(np.abs(bt_tl - fd))
    err = np.minimum(*errs)
    assert err.max() <= 2e-5 * np.abs(bt_tl).max(), (err.max() / np.abs(bt_tl).max(),
                                                      [x.max() / np.abs(bt_tl).max() for x in errs])


@pytest.mark.parametrize("kind", ["clear", "clouds", "aerosols", "cmaq", "gocart"])
def test_tangent_linear_adjoint_dot_product(gpu_lib, cloud_dir, kind):
    sensor, atm, sfc, geo, opt = _case(kind)
    h = _handle(gpu_lib, cloud_dir, sensor, kind)
    P, L = atm.n_profiles, h.n_channels[0]
    d, s, e = _direction(atm, sfc, P, L, 408)
    d.cloud_fraction = None if atm.cloud_fraction is None else np.where(atm.cloud_fraction > 0, d.cloud_fraction, 0)
    bt_tl, _ = h.tangent_linear(atm, sfc, geo, opt, d, s, None)
    y = np.random.Generator(np.random.PCG64(409)).standard_normal((P, L))
    ad, _ = h.adjoint(atm, sfc, geo, opt, y)
    lhs = float((bt_tl * y).sum())
    rhs = float((ad["temperature"] * d.temperature).sum() + (ad["absorber"] * d.absorber).sum())
    rhs += float(sum((ad[f] * getattr(s, f)).sum() for f in ("land_temperature", "water_temperature",
                                                             "snow_temperature", "ice_temperature")))
    for f in ("cloud_water_content", "cloud_effective_radius", "cloud_fraction", "aerosol_concentration",
              "aerosol_effective_radius", "aerosol_effective_variance", "relative_humidity"):
        if f in ad and getattr(d, f, None) is not None:
            rhs += float((ad[f] * getattr(d, f)).sum())
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), 1e-300), (lhs, rhs)
