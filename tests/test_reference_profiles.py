"""The reference's own unit-test profiles (tests/golden/reference_profiles.json,
read from test/mains/unit/Unit_Test/Load_Atm_Data.inc, Load_Sfc_Data.inc and
test_AD.f90 by tests/golden/make_reference_profiles.py) through the oracle:
the fixture's contents, AddLayers on their 0.714 hPa tops, and the oracle's
clear-sky and cloudy K-matrices against central differences of its own
forward on them (the reference's own check, test_TL_convergence.f90)."""
import dataclasses

import numpy as np
import pytest

from conftest import reference_profiles
from crtmv3_gb300 import addlayers as al, coefficients as co, synthetic as sy


@pytest.fixture(scope="module")
def cloud_dir(coeff_dir):
    sy.write_cloud_files(coeff_dir)
    sy.write_aerosol_files(coeff_dir)
    return coeff_dir


def test_fixture_contents():
    atm, sfc, geo, opt = reference_profiles("irsynth_c616", clouds=True, aerosols=True)
    assert atm.n_profiles == 2 and atm.max_layers == 92 and atm.level_pressure.shape == (2, 93)
    assert np.allclose(atm.level_pressure[:, 0], 0.714) and (np.diff(atm.level_pressure, axis=1) > 0).all()
    assert ((atm.pressure > atm.level_pressure[:, :-1]) & (atm.pressure < atm.level_pressure[:, 1:])).all()
    assert list(atm.absorber_id) == [co.H2O_ID, co.O3_ID] and list(atm.climatology) == [6, 1]
    assert (atm.cloud_type == co.SNOW_CLOUD).all()
    assert atm.cloud_water_content[0, 0, 59:80].min() == 5.0 and not atm.cloud_water_content[0, 0, 80:].any()
    assert list(atm.cloud_fraction[:, 0]) == [1.0, 0.5]
    assert atm.aerosol_type.tolist() == [[1, 8, 5], [2, 3, 4]]
    assert np.allclose(sfc.land_coverage + sfc.water_coverage + sfc.snow_coverage + sfc.ice_coverage, 1.0)
    assert geo.sensor_zenith_angle[0] == 30.0
    ext, info = al.add_layers(atm)
    assert list(info.n_added) == [8, 8] and np.allclose(ext.level_pressure[:, 0], 0.005)
    assert np.array_equal(ext.temperature[:, 8:], atm.temperature)
    assert not ext.cloud_water_content[:, :, :8].any()


def _fd_check(o, ext, sfc, geo, opt, ref, layers, n_added, forward, tol):
    """Central differences of `forward` in T (0.01 K) and H2O (1e-4 relative)
    at user layers `layers` against the K-matrix `ref`."""
    kt, ka = ref["temperature_k"], ref["absorber_k"]
    for k in layers:
        e = k + n_added
        for what in ("t", "q"):
            bts = []
            for sgn in (1, -1):
                a = dataclasses.replace(ext, temperature=ext.temperature.copy(), absorber=ext.absorber.copy())
                if what == "t":
                    a.temperature[:, e] += sgn * 0.01
                else:
                    a.absorber[:, 0, e] *= 1.0 + sgn * 1e-4
                bts.append(forward(a))
            if what == "t":
                fd, got, scale = (bts[0] - bts[1]) / 0.02, kt[:, :, e], np.abs(kt).max()
            else:
                q = ext.absorber[:, 0, e][:, None]
                fd, got = (bts[0] - bts[1]) / (2e-4 * q) * q, ka[:, :, 0, e] * q
                scale = np.abs(ka[:, :, 0] * ext.absorber[:, 0][:, None]).max()
            assert np.abs(fd - got).max() <= tol * scale, (what, k, np.abs(fd - got).max() / scale)


@pytest.mark.parametrize("sensor", ["irsynth_c616", "mwsynth_c22"])
def test_oracle_clear_k_matrix_on_reference_profiles(coeff_dir, sensor):
    from oracle.pyoracle import Oracle
    atm, sfc, geo, opt = reference_profiles(sensor)
    ext, info = al.add_layers(atm)
    o = Oracle(coeff_dir, sensor)
    ref = o.k_matrix(ext, sfc, geo, opt, n_threads=4)
    _, bt = o.forward(ext, sfc, geo, opt)
    assert np.abs(ref["bt"] - bt).max() < 1e-10
    _fd_check(o, ext, sfc, geo, opt, ref, (5, 40, 75, 90), 8, lambda a: o.forward(a, sfc, geo, opt)[1], 2e-5)


def test_oracle_cloudy_k_matrix_on_reference_profiles(cloud_dir):
    """The first profile (snow cloud in layers 60-80 at Cloud_Fraction 1, dust,
    sulfate and SSCM3 sea salt) on the infrared sensor through ADA: the
    oracle's reverse mode against central differences in T, H2O and the
    cloud's water content."""
    from oracle.pyoracle import Oracle
    sensor = "irsynth_c616"
    atm, sfc, geo, opt = reference_profiles(sensor, clouds=True, aerosols=True)
    atm, sfc, geo, opt = atm.subset([0]), sfc.subset([0]), geo.subset([0]), opt.subset([0])
    ext, info = al.add_layers(atm)
    o = Oracle(cloud_dir, sensor)
    cc, ac = f"{cloud_dir}/CloudCoeff.bin", f"{cloud_dir}/AerosolCoeff.bin"
    ref = o.k_matrix_scatter(ext, sfc, geo, opt, cc, ac, n_threads=4)
    fwd = lambda a: o.forward_scatter(a, sfc, geo, opt, cc, ac)[1]   # noqa: E731
    assert np.abs(ref["bt"] - fwd(ext)).max() < 1e-9
    _fd_check(o, ext, sfc, geo, opt, ref, (30, 62, 79, 88), 8, fwd, 2e-5)
    kw = ref["cloud_water_content_k"][:, :, 0]
    scale = np.abs(kw * ext.cloud_water_content[:, None, 0, :]).max()
    for k in (59, 66, 79):
        e = k + 8
        bts = []
        for sgn in (1, -1):
            a = dataclasses.replace(ext, cloud_water_content=ext.cloud_water_content.copy())
            a.cloud_water_content[:, 0, e] *= 1.0 + sgn * 1e-4
            bts.append(fwd(a))
        w = ext.cloud_water_content[0, 0, e]
        fd = (bts[0] - bts[1]) / 2e-4
        assert np.abs(fd - kw[:, :, e] * w).max() <= 2e-5 * scale, k
