"""The oracle's further RTSolution components (or_forward_ext), checked
against relations the reference's definitions imply:

* clear profiles: R = Up_Radiance + exp(-sum(Layer_Optical_Depth) / mu) x
  Upwelling_Radiance at the surface, which is e Bs + (1 - e) Down_Radiance
  (Emission_Module.f90:140-172); the overcast radiance of the top layer is its
  Planck radiance; Tb_clear / R_clear are the brightness temperature and
  radiance (CRTM_Forward_Module.f90:1115-1119); the layer optical depths are
  the clear-sky forward's;
* fractional profiles: R_clear / Tb_clear are the clear-sky forward of the same
  profile, and the radiance mixes them with the cloudy column by the total
  cloud cover (:1086-1114);
* n_Full_Streams is n_Streams + 2, the stream rule's count + 2 for profiles
  with clouds, 0 otherwise; SOD is zero for clear profiles and positive for
  cloudy ones."""
import dataclasses

import numpy as np
import pytest

from crtmv3_gb300 import coefficients as co, synthetic as sy


@pytest.fixture(scope="module")
def cloud_dir(coeff_dir):
    sy.write_cloud_files(coeff_dir)
    return coeff_dir


def _planck(sc, l, t):
    return sc.planck_c1[l] / (np.exp(sc.planck_c2[l] / (sc.band_c1[l] + sc.band_c2[l] * t)) - 1.0)


@pytest.mark.parametrize("sensor", ["mwsynth_c22", "irsynth_c616"])
def test_clear_components(coeff_dir, sensor):
    from oracle.pyoracle import Oracle
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, 4, 100, 81)
    opt.n_streams = np.array([0, 8, 0, 16], np.int32)
    opt.use_n_streams = opt.n_streams > 0
    o = Oracle(coeff_dir, sensor)
    x = o.forward_components(atm, sfc, geo, opt)
    rad, bt, lod = o.forward(atm, sfc, geo, opt, layer_od=True)
    sc = co.read_spccoeff(f"{coeff_dir}/{sensor}.SpcCoeff.bin")
    assert np.array_equal(x["radiance"], rad) and np.array_equal(x["tb_clear"], bt) and np.array_equal(x["r_clear"], rad)
    assert np.abs(x["layer_optical_depth"] - lod).max() <= 1e-14 * np.abs(lod).max()
    assert not x["sod"].any() and not x["total_cloud_cover"].any()
    assert np.array_equal(x["n_full_streams"], np.broadcast_to(np.where(opt.n_streams > 0, opt.n_streams + 2, 0)[:, None],
                                                               rad.shape))
    mu = np.cos(np.deg2rad(geo.sensor_zenith_angle))
    for p in range(4):
        Ku = int(atm.n_layers[p])
        surf = x["upwelling_radiance"][p, :, Ku - 1]
        e = x["surface_emissivity"][p]
        assert np.allclose(surf, e * x["surface_planck_radiance"][p] + (1 - e) * x["down_radiance"][p], rtol=1e-13)
        # R = Up_Radiance + exp(-tau_total / u) x the surface's upwelling, u the
        # cosine of the (Earth-curvature) sensor angle: u from the channel
        # whose total optical depth is nearest 1, then every channel
        tot = x["layer_optical_depth"][p, :, :Ku].sum(axis=1)
        j = int(np.argmin(np.abs(tot - 1.0)))
        sec = -np.log((rad[p, j] - x["up_radiance"][p, j]) / surf[j]) / tot[j]
        assert abs(sec - 1.0 / mu[p]) < 0.05 / mu[p]
        assert np.allclose(rad[p], x["up_radiance"][p] + np.exp(-tot * sec) * surf, rtol=1e-9, atol=0)
        t0 = atm.temperature[p, 0]
        assert np.allclose(x["upwelling_overcast_radiance"][p, :, 0], [_planck(sc, l, t0) for l in range(sc.n_channels)],
                           rtol=1e-12)
        assert not x["upwelling_radiance"][p, :, Ku:].any() and not x["layer_optical_depth"][p, :, Ku:].any()


def test_fractional_components(cloud_dir):
    from oracle.pyoracle import Oracle
    sensor = "mwsynth_c16"
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 4, 100, 83, wc_scale=30.0)
    rng = np.random.default_rng(2)
    atm.cloud_fraction = np.where(atm.cloud_fraction > 0, rng.uniform(0.2, 0.9, atm.cloud_fraction.shape), 0.0)
    atm.n_clouds[3] = 0
    opt.overlap_id = np.full(4, 3, np.int32)
    o = Oracle(cloud_dir, sensor)
    x = o.forward_components(atm, sfc, geo, opt, f"{cloud_dir}/CloudCoeff.bin")
    clear = dataclasses.replace(atm, n_clouds=np.zeros(4, np.int32))
    rc, btc = o.forward(clear, sfc, geo, opt)
    tcc = x["total_cloud_cover"][:, 0]
    assert (tcc[:3] > 0).all() and (tcc[:3] < 1).all() and tcc[3] == 0
    assert np.allclose(x["r_clear"], rc, rtol=1e-13, atol=0) and np.allclose(x["tb_clear"], btc, rtol=1e-13, atol=0)
    assert (x["sod"][:3] >= 0).all() and x["sod"][:3].max() > 0 and not x["sod"][3].any()
    assert not x["up_radiance"][:3].any() and not x["upwelling_radiance"][:3].any()
    assert (x["up_radiance"][3] > 0).all()
    sc = co.read_spccoeff(f"{cloud_dir}/{sensor}.SpcCoeff.bin")
    for p in range(3):
        mie = 2 * np.pi * atm.cloud_effective_radius[p].max() * sc.wavenumber / 1e4
        nleg = np.where(mie < 0.01, 2, np.where(mie < 1.0, 4, 6))
        assert np.array_equal(x["n_full_streams"][p], nleg + 2)
    assert not x["n_full_streams"][3].any()
