"""The CPU FP64 oracle: finite differences, adjoint symmetry and known answers.

The reference publishes no golden vectors for this path (its data files are
LFS stubs), so the oracle is pinned by these properties, following the
reference's own test methods (test/mains/unit/Unit_Test/test_AD.f90,
test_TL_convergence.f90).
"""
import numpy as np
import pytest

from crtmv3_gb300 import coefficients as co, synthetic as sy


@pytest.fixture(scope="module")
def oracles(coeff_dir):
    from oracle.pyoracle import Oracle
    return {s: Oracle(coeff_dir, s) for s in ("mwsynth_c22", "irsynth_c616", "mwsynth_c16")}


CASES = [("mwsynth_c22", 100), ("irsynth_c616", 101), ("mwsynth_c16", 90)]


def _best_fd(o, atm, sfc, geo, opt, t_tl, a_tl, ts_tl, ref):
    """Central differences at three step sizes; the smallest error against ``ref``
    (large steps carry truncation error, small ones rounding error)."""
    return min(np.abs(o.tangent_fd(atm, sfc, geo, opt, t_tl, a_tl, ts_tl, step=h) - ref).max()
               for h in (1e-1, 1e-2, 1e-3))


@pytest.mark.parametrize("sensor,nl", CASES)
def test_k_matrix_temperature_matches_central_differences(oracles, sensor, nl):
    o = oracles[sensor]
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, 2, nl, 31)
    k = o.k_matrix(atm, sfc, geo, opt)
    P = atm.n_profiles
    za = np.zeros_like(atm.absorber)
    for lay in (nl // 3, nl - 2):
        tl = np.zeros_like(atm.temperature)
        tl[:, lay] = 1.0
        kk = k["temperature_k"][:, :, lay]
        assert _best_fd(o, atm, sfc, geo, opt, tl, za, np.zeros(P), kk) <= 1e-6 * np.abs(kk).max() + 5e-11
    kk = k["water_temperature_k"]
    assert _best_fd(o, atm, sfc, geo, opt, np.zeros_like(atm.temperature), za, np.ones(P), kk) \
        <= 1e-6 * np.abs(kk).max() + 5e-11


@pytest.mark.parametrize("sensor,nl", CASES)
def test_k_matrix_absorbers_match_central_differences(oracles, sensor, nl):
    o = oracles[sensor]
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, 2, nl, 32)
    k = o.k_matrix(atm, sfc, geo, opt)
    lay = nl // 2
    for j in range(atm.n_absorbers):
        al = np.zeros_like(atm.absorber)
        al[:, j, lay] = atm.absorber[:, j, lay] * 1e-3
        fd = o.tangent_fd(atm, sfc, geo, opt, np.zeros_like(atm.temperature), al,
                          np.zeros(atm.n_profiles), step=1.0)
        kk = k["absorber_k"][:, :, j, lay] * atm.absorber[:, j, lay][:, None] * 1e-3
        assert np.abs(fd - kk).max() <= 1e-4 * max(np.abs(kk).max(), 1e-12) + 1e-11


def test_adjoint_symmetry(oracles):
    """<K dx, y> == <dx, K^T y>: the adjoint equals the K-matrix summed with weights y
    (the reference's TL/AD check, test_AD.f90:216-377, tolerance there 1e-7)."""
    o = oracles["irsynth_c616"]
    atm, sfc, geo, opt = sy.clear_sky_workload("irsynth_c616", 2, 101, 33)
    rng = np.random.default_rng(0)
    y = rng.normal(size=(2, o.n_channels))
    k = o.k_matrix(atm, sfc, geo, opt)
    ad = o.adjoint(atm, sfc, geo, opt, y)
    lhs = np.einsum("pl,plk->pk", y, k["temperature_k"])
    assert np.abs(lhs - ad["temperature_ad"]).max() <= 1e-9 * np.abs(lhs).max()
    lhs = np.einsum("pl,pljk->pjk", y, k["absorber_k"])
    assert np.abs(lhs - ad["absorber_ad"]).max() <= 1e-9 * np.abs(lhs).max()
    k2 = o.k_matrix(atm, sfc, geo, opt, bt_k=y)
    ref = k["temperature_k"] * y[:, :, None]
    assert np.abs(k2["temperature_k"] - ref).max() <= 1e-12 * np.abs(ref).max()


def _zero_coefficient_sensor(d, sid):
    tc = sy.generate_odps(3, 5, 5, sid, co.MICROWAVE_SENSOR)
    tc.c = np.zeros_like(tc.c)
    sc = sy.generate_spccoeff(sid, co.MICROWAVE_SENSOR, 5, 6)
    co.write_odps(f"{d}/{sid}.TauCoeff.bin", tc)
    co.write_spccoeff(f"{d}/{sid}.SpcCoeff.bin", sc)
    return sc


def test_transparent_atmosphere_known_answer(tmp_path):
    """Zero optical depth: TOA radiance = e*B(Ts) + (1-e)*cosmic background."""
    from oracle.pyoracle import Oracle
    sc = _zero_coefficient_sensor(str(tmp_path), "z")
    atm, sfc, geo = sy.generate_profiles(3, 50, (co.H2O_ID,), 8)
    opt = sy.OptionsBatch(emissivity=sy.emissivity_for(1, 3, 5, 2))
    rad, bt = Oracle(str(tmp_path), "z").forward(atm, sfc, geo, opt)
    te = sc.band_c1 + sc.band_c2 * sfc.water_temperature[:, None]
    bs = sc.planck_c1 / (np.exp(sc.planck_c2 / te) - 1.0)
    e = opt.emissivity
    expect = e * bs + (1 - e) * sc.cosmic_background_radiance
    assert np.allclose(rad, expect, rtol=1e-13, atol=0)


def test_isothermal_blackbody_known_answer(oracles):
    """Isothermal atmosphere over a black surface at the same temperature: BT = T
    for any optical depth (Planck / inverse Planck round trip)."""
    o = oracles["irsynth_c616"]
    atm, sfc, geo, opt = sy.clear_sky_workload("irsynth_c616", 2, 101, 34)
    atm.temperature[:, :] = 250.0
    sfc.water_temperature[:] = 250.0
    opt.emissivity[:] = 1.0
    rad, bt = o.forward(atm, sfc, geo, opt)
    assert np.abs(bt - 250.0).max() < 1e-9


def test_padding_layers_are_ignored(oracles):
    """A ragged batch gives the same results as each profile run alone."""
    o = oracles["irsynth_c616"]
    nl = np.array([70, 101])
    atm, sfc, geo = sy.generate_profiles(2, nl, sy.absorber_set(1), 35)
    opt = sy.OptionsBatch(emissivity=sy.emissivity_for(2, 2, 616, 3))
    _, bt = o.forward(atm, sfc, geo, opt)
    one = atm.subset(slice(0, 1))
    one.level_pressure = np.ascontiguousarray(one.level_pressure[:, :71])
    one.pressure = np.ascontiguousarray(one.pressure[:, :70])
    one.temperature = np.ascontiguousarray(one.temperature[:, :70])
    one.absorber = np.ascontiguousarray(one.absorber[:, :, :70])
    _, bt1 = o.forward(one, sfc.subset(slice(0, 1)), geo.subset(slice(0, 1)), opt.subset(slice(0, 1)))
    assert np.array_equal(bt[0], bt1[0])
