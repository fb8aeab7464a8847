"""The oracle's cloud / ADA path (CPU).

The reference publishes no outputs for this path either.  These tests pin the
oracle by an independent eigensolver, by known answers and by limits:

* one ADA layer (MOM, ADA_Module.f90:262-354) against the same formulas
  evaluated with numpy's general eigensolver (the reference uses a general
  real eigensolver, ASYMTX);
* Kirchhoff: an isothermal atmosphere over a black surface at the same
  temperature gives BT = T for any cloud, any scattering and any stream count;
* clouds below the water-content threshold: the ADA path with no scattering
  layer equals the Emission solver;
* stream-count convergence.
"""
import ctypes as ct

import numpy as np
import pytest

from crtmv3_gb300 import coefficients as co, synthetic as sy

_dp = ct.POINTER(ct.c_double)


def _p(a):
    return a.ctypes.data_as(_dp)


@pytest.fixture(scope="module")
def cloud_path(coeff_dir):
    return sy.write_cloud_files(coeff_dir)


def _setup(nleg, mu_sensor, g):
    from oracle.pyoracle import lib
    pc = 0.5 * g ** np.arange(nleg + 1)
    n = 20
    mu, wt = np.zeros(n), np.zeros(n)
    ff, bb = np.zeros(n * n), np.zeros(n * n)
    nz = ct.c_int(0)
    lib().or_phase_setup(nleg, mu_sensor, _p(pc), _p(mu), _p(wt), _p(ff), _p(bb), ct.byref(nz))
    nZ = nz.value
    return mu[:nZ].copy(), wt[:nZ].copy(), ff[:nZ * nZ].reshape(nZ, nZ), bb[:nZ * nZ].reshape(nZ, nZ)


def _mom_numpy(mu, wt, ff, bb, w, tau):
    """MOM (ADA_Module.f90:262-354) with numpy's general eigensolver."""
    s = min(w, 0.999999)
    c = s / mu
    PM = c[:, None] * bb * wt[None, :]
    PP = c[:, None] * ff * wt[None, :] - np.diag(1.0 / mu)
    PPM, PPP = PP - PM, PP + PM
    HH = PPM @ PPP
    ev, E = np.linalg.eig(HH)
    assert np.abs(ev.imag).max() < 1e-9 * np.abs(ev).max()
    ev, E = ev.real, E.real
    lam = np.where(ev > 0, np.sqrt(np.maximum(ev, 0)), 0.0)
    EF = np.linalg.inv(PPM) @ (E * lam[None, :])
    Gp, Gm = (E + EF) / 2, (E - EF) / 2
    ex = np.exp(-lam * tau)
    A1, A4 = Gp * ex[None, :], Gm * ex[None, :]
    A2 = np.linalg.inv(Gm) @ A1
    A3, A5, A6 = Gp @ A2, A1 @ A2, A4 @ A2
    iGA = np.linalg.inv(Gm - A5)
    return (A4 - A3) @ iGA, (Gp - A6) @ iGA


@pytest.mark.parametrize("nleg,mu_sensor", [(2, 0.83), (4, 0.6), (6, 0.97), (8, 0.5), (16, 0.71)])
@pytest.mark.parametrize("w,tau,g", [(0.5, 0.3, 0.6), (0.95, 4.0, 0.85), (0.2, 0.01, 0.3)])
def test_mom_layer_matches_general_eigensolver(nleg, mu_sensor, w, tau, g):
    from oracle.pyoracle import lib
    mu, wt, ff, bb = _setup(nleg, mu_sensor, g)
    nZ = mu.size
    nS = (nleg + 2) // 2
    T, R, S = np.zeros(nZ * nZ), np.zeros(nZ * nZ), np.zeros(nZ)
    rc = lib().or_amom_layer(nS, nZ, w, tau, _p(mu), _p(wt), _p(np.ascontiguousarray(ff)),
                             _p(np.ascontiguousarray(bb)), 1.0, _p(T), _p(R), _p(S))
    assert rc == 0
    Tn, Rn = _mom_numpy(mu, wt, ff, bb, w, tau)
    assert np.abs(T.reshape(nZ, nZ) - Tn).max() < 1e-11
    assert np.abs(R.reshape(nZ, nZ) - Rn).max() < 1e-11


def test_normalised_phase_conserves_energy():
    """After Normalize_Phase the scattering out of each quadrature stream sums to 1."""
    for nleg in (2, 4, 6, 8, 16):
        mu, wt, ff, bb = _setup(nleg, 0.77, 0.7)
        nS = (nleg + 2) // 2
        rows = ((ff + bb)[:nS, :nS] * wt[None, :nS]).sum(axis=1)
        assert np.abs(rows - 1.0).max() < 1e-12
        assert np.allclose(ff, ff.T) and np.allclose(bb, bb.T)


def _isothermal(atm, sfc, opt, T=265.0):
    for m in range(atm.n_profiles):
        atm.temperature[m, :atm.n_layers[m]] = T
    sfc.water_temperature[:] = T
    opt.emissivity[:] = 1.0


def _isothermal_sensor(coeff_dir, tmp_path, sensor, T):
    """A copy of ``sensor`` whose cosmic background is B(T): with it the scene is
    an isothermal enclosure."""
    import shutil
    sc = co.read_spccoeff(f"{coeff_dir}/{sensor}.SpcCoeff.bin")
    te = sc.band_c1 + sc.band_c2 * T
    sc.cosmic_background_radiance = sc.planck_c1 / (np.exp(sc.planck_c2 / te) - 1.0)
    co.write_spccoeff(str(tmp_path / f"{sensor}.SpcCoeff.bin"), sc)
    shutil.copy(f"{coeff_dir}/{sensor}.TauCoeff.bin", tmp_path / f"{sensor}.TauCoeff.bin")
    return str(tmp_path)


@pytest.mark.parametrize("sensor,nl", [("mwsynth_c16", 100), ("irsynth_c616", 101)])
@pytest.mark.parametrize("n_streams", [None, 8, 16])
def test_kirchhoff_isothermal_enclosure(coeff_dir, cloud_path, tmp_path, sensor, nl, n_streams):
    """Isothermal atmosphere, black surface and a cosmic background all at the
    same temperature: BT = T for any cloud, scattering and stream count."""
    from oracle.pyoracle import Oracle
    d = _isothermal_sensor(coeff_dir, tmp_path, sensor, 265.0)
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 3, nl, 41, wc_scale=300.0, n_streams=n_streams)
    _isothermal(atm, sfc, opt)
    _, bt = Oracle(d, sensor).forward_scatter(atm, sfc, geo, opt, cloud_path)
    assert np.abs(bt - 265.0).max() < 1e-8


@pytest.mark.parametrize("sensor,nl", [("mwsynth_c16", 100), ("irsynth_c616", 101)])
def test_sub_threshold_clouds_equal_emission(coeff_dir, cloud_path, sensor, nl):
    """Water content below WATER_CONTENT_THRESHOLD: ADA runs (the profile has
    clouds) but no layer scatters, and the result equals the Emission solver."""
    from oracle.pyoracle import Oracle
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 3, nl, 42)
    atm.cloud_water_content[:] = np.where(atm.cloud_water_content > 0, 5e-7, 0.0)
    o = Oracle(coeff_dir, sensor)
    _, bt = o.forward_scatter(atm, sfc, geo, opt, cloud_path)
    _, bt0 = o.forward(atm, sfc, geo, opt)
    assert np.abs(bt - bt0).max() < 1e-9


def test_clear_profiles_in_a_cloudy_batch(coeff_dir, cloud_path):
    from oracle.pyoracle import Oracle
    sensor = "mwsynth_c16"
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 4, 100, 43, wc_scale=100.0)
    atm.n_clouds[1] = 0
    o = Oracle(coeff_dir, sensor)
    _, bt = o.forward_scatter(atm, sfc, geo, opt, cloud_path)
    _, bt0 = o.forward(atm, sfc, geo, opt)
    assert np.array_equal(bt[1], bt0[1])
    assert np.abs(bt[0] - bt0[0]).max() > 0.1


def test_stream_count_convergence(coeff_dir, cloud_path):
    from oracle.pyoracle import Oracle
    sensor = "mwsynth_c16"
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 3, 100, 44, wc_scale=100.0, n_streams=16)
    o = Oracle(coeff_dir, sensor)
    _, b16 = o.forward_scatter(atm, sfc, geo, opt, cloud_path)
    opt.n_streams[:] = 8
    _, b8 = o.forward_scatter(atm, sfc, geo, opt, cloud_path)
    assert np.abs(b16 - b8).max() < 1.0


@pytest.mark.parametrize("sensor,nl", [("mwsynth_c16", 100), ("irsynth_c616", 101)])
def test_soi_agrees_with_ada(coeff_dir, cloud_path, sensor, nl):
    """Two different solvers of the same scattering problem: at the config's
    cloud amounts SOI (successive orders, 1e-4 stopping rule, truncated
    doubling) and ADA (eigen-solution + adding) agree to 0.02 K."""
    from oracle.pyoracle import Oracle
    o = Oracle(coeff_dir, sensor)
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 4, nl, 45)
    _, ba = o.forward_scatter(atm, sfc, geo, opt, cloud_path)
    opt.rt_algorithm_id = np.full(4, 168, np.int32)
    _, bs = o.forward_scatter(atm, sfc, geo, opt, cloud_path)
    assert np.abs(bs - ba).max() < 0.02


# ---------------------------------------------------------------------------
# Cloud coverage (CRTM_Atmosphere_Coverage, Compute_CloudCover)
# ---------------------------------------------------------------------------

def _tcc(cf, lwc, overlap):
    """Total cloud cover of one profile (CRTM_CloudCover_Define.f90:522-638),
    restated for the test: cf and the summed cloud water per layer."""
    cf = np.where(cf < 1e-12, 0.0, cf)
    if overlap == 1:
        return cf.max()
    if overlap == 2:
        return 1.0 - np.prod(np.where(cf > 1e-12, 1.0 - cf, 1.0))
    if overlap == 3:
        prod = 1.0 - cf[0]
        for k in range(1, cf.size):
            mc = 1.0 - max(cf[k - 1], cf[k])
            prod = mc if (prod == 0.0 and cf[k - 1] == 1.0) else prod * mc / (1.0 - cf[k - 1])
        return 1.0 - prod
    if overlap == 4:
        w = np.where(lwc > 1e-6, lwc, 0.0)
        return (cf * w).sum() / w.sum()
    return 1.0


@pytest.mark.parametrize("overlap", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("sensor,nl", [("mwsynth_c16", 100), ("irsynth_c616", 101)])
def test_fractional_cover_mixes_clear_and_scaled_cloudy_columns(coeff_dir, cloud_path, sensor, nl, overlap):
    """FRACTIONAL profile = (1 - tcc) x the clear column (gas only) + tcc x the
    cloudy column with water content / tcc (CRTM_Forward_Module.f90:1086-1093,
    CRTM_CloudCover_Define.f90:512-519), tcc from the overlap scheme."""
    import copy
    from oracle.pyoracle import Oracle
    P = 4
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, P, nl, 301, cloud_types=(co.WATER_CLOUD, co.ICE_CLOUD),
                                            wc_scale=50.0)
    sy.add_clouds(atm, (co.WATER_CLOUD, co.ICE_CLOUD), 302, wc_scale=50.0, cover=(0.05, 0.95))
    opt.overlap_id = np.full(P, overlap, np.int32)
    orc = Oracle(coeff_dir, sensor)
    _, bt = orc.forward_scatter(atm, sfc, geo, opt, cloud_path)
    clear = copy.deepcopy(atm)
    clear.n_clouds = np.zeros(P, np.int32)
    r_clear, _ = orc.forward_scatter(clear, sfc, geo, opt, cloud_path)
    tcc = np.array([_tcc(atm.cloud_fraction[m, :nl], atm.cloud_water_content[m, :, :nl].sum(axis=0), overlap)
                    for m in range(P)])
    assert ((tcc > 0.04) & (tcc <= 1.0)).all()
    full = copy.deepcopy(atm)
    full.cloud_water_content = atm.cloud_water_content / tcc[:, None, None]
    full.cloud_fraction = np.where(atm.cloud_fraction > 0, 1.0, 0.0)
    r_cloudy, _ = orc.forward_scatter(full, sfc, geo, opt, cloud_path)
    mix = (1.0 - tcc[:, None]) * r_clear + tcc[:, None] * r_cloudy
    sc = co.read_spccoeff(f"{coeff_dir}/{sensor}.SpcCoeff.bin")
    te_inv = sc.planck_c2 / np.log(sc.planck_c1 / mix + 1.0)
    bt_mix = (te_inv - sc.band_c1) / sc.band_c2
    assert np.abs(bt - bt_mix).max() < 1e-9


def test_cloud_fraction_thresholds(coeff_dir, cloud_path):
    """Fraction below 1e-12 drops the cloud (CRTM_Forward_Module.f90:367-376);
    between 1e-12 and 1e-6 the profile is one cloudy column, as with fraction 1;
    an invalid overlap id fails."""
    import copy
    from oracle.pyoracle import Oracle
    sensor = "mwsynth_c16"
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 3, 100, 303, wc_scale=100.0)
    orc = Oracle(coeff_dir, sensor)
    _, bt1 = orc.forward_scatter(atm, sfc, geo, opt, cloud_path)
    small = copy.deepcopy(atm)
    small.cloud_fraction = atm.cloud_fraction * 1e-9
    _, bts = orc.forward_scatter(small, sfc, geo, opt, cloud_path)
    assert np.abs(bts - bt1).max() == 0.0
    gone = copy.deepcopy(atm)
    gone.cloud_fraction = atm.cloud_fraction * 1e-13
    _, btg = orc.forward_scatter(gone, sfc, geo, opt, cloud_path)
    _, btc = orc.forward(atm, sfc, geo, opt)
    assert np.abs(btg - btc).max() < 1e-9
    assert np.abs(bt1 - btc).max() > 1.0
    opt.overlap_id = np.array([4, 9, 4], np.int32)
    with pytest.raises(RuntimeError, match="Overlap"):
        orc.forward_scatter(atm, sfc, geo, opt, cloud_path)


@pytest.mark.parametrize("sensor,n_streams,aer", [("irsynth_c616", None, True), ("mwsynth_c22", None, False),
                                                  ("irsynth_c616", 16, True), ("mwsynth_c16", 8, False)])
def test_oracle_cloudy_kmatrix_matches_central_differences(coeff_dir, sensor, n_streams, aer):
    """The oracle's cloudy K-matrix (reverse mode of the ADA adding, MOM,
    phase normalisation, combine and LUT interpolation) against central
    differences of the oracle's own cloudy forward, for the temperature
    (1e-3 K), every absorber, each cloud's water content and effective
    radius, each aerosol's concentration and radius (1e-4 relative steps)
    and the surface temperature: within 2e-6 of each variable's largest
    Jacobian (the differences' truncation and rounding)."""
    import copy

    from oracle.pyoracle import Oracle
    sy.write_sensor_files(coeff_dir, sensor)
    cp, ap = sy.write_cloud_files(coeff_dir), sy.write_aerosol_files(coeff_dir)
    mw = sensor.startswith("mw")
    types = ((co.WATER_CLOUD, co.ICE_CLOUD, co.RAIN_CLOUD, co.SNOW_CLOUD, co.GRAUPEL_CLOUD) if mw
             else (co.WATER_CLOUD, co.ICE_CLOUD))
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 1, 60, 11, cloud_types=types, wc_scale=10.0,
                                            n_streams=n_streams)
    if aer:
        sy.add_aerosols(atm, sy.AEROSOL_TYPES, 12, load_scale=10.0)
    o = Oracle(coeff_dir, sensor)
    K = o.k_matrix_scatter(atm, sfc, geo, opt, cp, ap if aer else None, n_threads=8)

    def bt(a, s=sfc):
        return o.forward_scatter(a, s, geo, opt, cp, ap if aer else None, n_threads=8)[1]
    assert np.array_equal(bt(atm), K["bt"])

    def fd(field, idx, h, rel=True):
        a1, a2 = copy.deepcopy(atm), copy.deepcopy(atm)
        hh = h * abs(getattr(a1, field)[idx]) if rel else h
        getattr(a1, field)[idx] += hh
        getattr(a2, field)[idx] -= hh
        return (bt(a1) - bt(a2)) / (2 * hh)

    def check(name, got, want, scale):
        assert np.abs(got - want).max() <= 2e-6 * scale, (name, np.abs(got - want).max() / scale)
    m, tol_checked = 0, 0
    Ku = int(atm.n_layers[m])
    wc = atm.cloud_water_content
    cloudy = np.where((wc[m] > 1e-6).any(axis=0))[0]
    for k in [cloudy[0], cloudy[len(cloudy) // 2], Ku - 1]:
        check("T", fd("temperature", (m, k), 1e-3, rel=False)[m], K["temperature_k"][m, :, k],
              np.abs(K["temperature_k"][m]).max())
        for j in range(min(atm.n_absorbers, 2)):
            check(f"absorber {j}", fd("absorber", (m, j, k), 1e-4)[m], K["absorber_k"][m, :, j, k],
                  np.abs(K["absorber_k"][m, :, j]).max() * 3.0)
        for c in range(wc.shape[1]):
            if not wc[m, c, k] > 1e-6:
                assert not K["cloud_water_content_k"][m, :, c, k].any()
                continue
            for f, kf in (("cloud_water_content", "cloud_water_content_k"),
                          ("cloud_effective_radius", "cloud_effective_radius_k")):
                x = getattr(atm, f)
                check(f, fd(f, (m, c, k), 1e-4)[m] * x[m, c, k], K[kf][m, :, c, k] * x[m, c, k],
                      np.abs(K[kf][m, :, c] * x[m, c]).max())
                tol_checked += 1
        for a in (range(3) if aer and k == cloudy[0] else ()):
            for f, kf in (("aerosol_concentration", "aerosol_concentration_k"),
                          ("aerosol_effective_radius", "aerosol_effective_radius_k")):
                x = getattr(atm, f)
                check(f, fd(f, (m, a, k), 1e-4)[m] * x[m, a, k], K[kf][m, :, a, k] * x[m, a, k],
                      np.abs(K[kf][m, :, a] * x[m, a]).max())
    s1, s2 = copy.deepcopy(sfc), copy.deepcopy(sfc)
    s1.water_temperature[m] += 1e-3
    s2.water_temperature[m] -= 1e-3
    check("Ts", ((bt(atm, s1) - bt(atm, s2)) / 2e-3)[m], K["water_temperature_k"][m],
          np.abs(K["water_temperature_k"][m]).max())
    assert tol_checked >= 2
