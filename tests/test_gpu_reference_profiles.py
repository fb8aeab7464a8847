"""The reference's own unit-test profiles (tests/golden/reference_profiles.json:
two 92-layer profiles with 0.714 hPa tops, snow clouds and three aerosols
each, a four-cover surface, 30 degrees zenith) on the GPU against the oracle:

* clear sky through the reference-named CRTM_Forward / CRTM_K_Matrix (which
  add the climatology layers above the 0.714 hPa tops), as test_AD.f90 runs
  them (no clouds, no aerosols), infrared and microwave;
* with the file's clouds and aerosols: the forward of both profiles (the
  second one fractional, Cloud_Fraction 0.5) and the K-matrix of the first.

Tolerances as the other parity tests: FP64 form 1e-4 K and 1e-6 of the
largest Jacobian; mixed form 0.01 K and 1e-3."""
import numpy as np
import pytest

from conftest import reference_profiles
from crtmv3_gb300 import addlayers as al, synthetic as sy

pytestmark = pytest.mark.gpu

BT_TOL = {0: 1e-4, 1: 1e-2}
JAC_TOL = {0: 1e-6, 1: 1e-3}


@pytest.fixture(scope="module")
def cloud_dir(coeff_dir):
    sy.write_cloud_files(coeff_dir)
    sy.write_aerosol_files(coeff_dir)
    return coeff_dir


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("sensor", ["irsynth_c616", "mwsynth_c22"])
def test_clear_reference_profiles_match_oracle(gpu_lib, coeff_dir, sensor, precision):
    from oracle.pyoracle import Oracle
    api = gpu_lib
    atm, sfc, geo, opt = reference_profiles(sensor)
    ext, info = al.add_layers(atm)
    ci = []
    assert api.CRTM_Init([sensor], ci, coeff_dir, precision) == api.SUCCESS
    L = ci[0].n_channels
    ks, rts, fw = [], [], []
    assert api.CRTM_K_Matrix(atm, sfc, [np.ones((2, L))], geo, ci, ks, rts, opt) == api.SUCCESS
    assert api.CRTM_Forward(atm, sfc, geo, ci, fw, opt) == api.SUCCESS
    ref = Oracle(coeff_dir, sensor).k_matrix(ext, sfc, geo, opt)
    assert np.abs(rts[0].brightness_temperature - ref["bt"]).max() < BT_TOL[precision]
    assert np.abs(fw[0].brightness_temperature - ref["bt"]).max() < BT_TOL[precision]
    km, tol = ks[0], JAC_TOL[precision]
    assert km.temperature.shape == (2, L, 92)
    assert _rel(km.temperature, al.user_layers(info, ref["temperature_k"])) < tol
    ak = al.user_layers(info, ref["absorber_k"])
    for j in range(2):
        assert _rel(km.absorber[:, :, j], ak[:, :, j]) < tol * 10, j
    assert _rel(km.water_temperature, ref["water_temperature_k"]) < tol
    assert _rel(km.surface_emissivity, ref["surface_emissivity_k"]) < tol
    api.CRTM_Destroy(ci)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("sensor", ["irsynth_c616", "mwsynth_c22"])
def test_cloudy_reference_profiles_match_oracle(gpu_lib, cloud_dir, sensor, precision):
    from oracle.pyoracle import Oracle
    ir = sensor.startswith("ir")
    atm, sfc, geo, opt = reference_profiles(sensor, clouds=True, aerosols=ir)
    ext, info = al.add_layers(atm)
    cc = f"{cloud_dir}/CloudCoeff.bin"
    ac = f"{cloud_dir}/AerosolCoeff.bin" if ir else None
    o = Oracle(cloud_dir, sensor)
    h = gpu_lib.CRTM([sensor], cloud_dir, precision)
    _, bt = o.forward_scatter(ext, sfc, geo, opt, cc, ac)
    rts = h.forward(ext, sfc, geo, opt)
    assert (rts.status == 0).all()
    assert np.abs(rts.brightness_temperature - bt).max() < BT_TOL[precision]
    # K-matrix of the first profile (Cloud_Fraction 1)
    one = [0]
    e1, s1, g1, o1 = ext.subset(one), sfc.subset(one), geo.subset(one), opt.subset(one)
    km, r1 = h.k_matrix(e1, s1, g1, o1)
    ref = o.k_matrix_scatter(e1, s1, g1, o1, cc, ac, n_threads=8)
    assert np.abs(r1.brightness_temperature - ref["bt"]).max() < BT_TOL[precision]
    tol = JAC_TOL[precision]
    assert _rel(km.temperature, ref["temperature_k"]) < tol
    for j in range(2):
        assert _rel(km.absorber[:, :, j], ref["absorber_k"][:, :, j]) < tol * 10, j
    # under the file's 5 kg/m^2 snow cloud the surface is all but hidden: the
    # skin-temperature Jacobian is held to the temperature Jacobian's scale
    scale = max(np.abs(ref["water_temperature_k"]).max(), np.abs(ref["temperature_k"]).max())
    assert np.abs(km.water_temperature - ref["water_temperature_k"]).max() < tol * scale
    fields = [("cloud_water_content", "cloud_water_content_k"), ("cloud_effective_radius", "cloud_effective_radius_k")]
    if ir:
        fields += [("aerosol_concentration", "aerosol_concentration_k"),
                   ("aerosol_effective_radius", "aerosol_effective_radius_k")]
    for field, key in fields:
        x = getattr(e1, field)[:, None]
        scale = max(np.abs(ref[key] * x).max(), 1e-300)
        assert np.abs((getattr(km, field) - ref[key]) * x).max() <= tol * scale, field
