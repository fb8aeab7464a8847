"""K-matrix and adjoint of scattering profiles (clouds, aerosols; ADA and SOI) on the GPU.

The oracle's cloudy forward is the checker: central finite differences of it
(FP64) give the Jacobians of one layer in every profile at a time, for the
temperature (step 1e-3 K) and each absorber (step 1e-4 of the amount), and of
the surface temperature and emissivity.  Central differences of a smooth FP64
forward carry about 1e-7 of the largest Jacobian, so the FP64 form must agree
within 2e-5 relative to the largest Jacobian of the variable (layer by layer);
the mixed form must agree with the FP64 form within 1e-3, as for clear sky.
"""
import copy

import numpy as np
import pytest

from crtmv3_gb300 import coefficients as co, synthetic as sy

pytestmark = pytest.mark.gpu

FD_TOL = 2e-5
MIX_TOL = 1e-3
RT_SOI = 168


@pytest.fixture(scope="module")
def cloud_dir(coeff_dir):
    sy.write_cloud_files(coeff_dir)
    sy.write_aerosol_files(coeff_dir)
    return coeff_dir


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _paths(d, atm):
    cp = f"{d}/CloudCoeff.bin" if atm.cloud_type is not None else None
    ap = f"{d}/AerosolCoeff.bin" if atm.aerosol_type is not None else None
    return cp, ap


def _fd_bt(orc, d, atm, sfc, geo, opt, perturb, step):
    """Central difference of the oracle's cloudy brightness temperatures:
    perturb(atm, sfc, opt, s) applies a signed step s (scalar or per profile;
    profiles with a zero step come out as zero)."""
    cp, ap = _paths(d, atm)
    out = []
    for sgn in (1.0, -1.0):
        a, s, o = copy.deepcopy(atm), copy.deepcopy(sfc), copy.deepcopy(opt)
        perturb(a, s, o, sgn * step)
        out.append(orc.forward_scatter(a, s, geo, o, cp, ap, n_threads=8)[1])
    st = np.asarray(step, np.float64)
    den = 2.0 * (st[:, None] if st.ndim else st)
    return (out[0] - out[1]) / np.where(den == 0.0, 1.0, den)


def _fd_best(orc, d, atm, sfc, geo, opt, perturb, step, got, mult):
    """_fd_bt for each step multiplier in mult, elementwise the one closest to
    got (SOI: the doubling's rounding noise asks for large steps, the LUT
    interpolation's curvature for small ones)."""
    best = None
    for m in mult:
        fd = _fd_bt(orc, d, atm, sfc, geo, opt, perturb, np.asarray(step) * m)
        best = fd if best is None else np.where(np.abs(fd - got) < np.abs(best - got), fd, best)
    return best


def _check_layers(km, orc, d, atm, sfc, geo, opt, layers, mult=(1.0,), tol=FD_TOL, absorbers=True):
    for k in layers:
        def pt(a, s, o, h, k=k):
            a.temperature[:, k] += h
        got = km.temperature[:, :, k]
        fd = _fd_best(orc, d, atm, sfc, geo, opt, pt, 1e-3, got, mult)
        assert np.abs(got - fd).max() <= tol * max(np.abs(km.temperature).max(), 1e-12), (k, _rel(got, fd))
        for j in range(atm.n_absorbers if absorbers else 0):
            step = 1e-4 * atm.absorber[:, j, k]

            def pa(a, s, o, h, k=k, j=j):
                a.absorber[:, j, k] += h
            got = km.absorber[:, :, j, k]
            fd = _fd_best(orc, d, atm, sfc, geo, opt, pa, step, got, mult)
            scale = max(np.abs(km.absorber[:, :, j]).max(), 1e-12)
            assert np.abs(got - fd).max() <= tol * scale, (k, j, _rel(got, fd))


def _check_species(km, orc, d, atm, sfc, geo, opt, layers, fraction=False, mult=(1.0,), tol=FD_TOL,
                   fraction_mult=(1.0,)):
    """Cloud water content / effective radius (and, for fractional profiles,
    cloud fraction) and aerosol concentration / effective radius Jacobians of
    the listed layers against central differences (steps 1e-4 of the value,
    1e-6 in the fraction), profile by profile where the species is present."""
    groups = []
    if atm.cloud_type is not None:
        groups += [("cloud_water_content", "cloud_water_content", c) for c in range(atm.cloud_type.shape[1])]
        groups += [("cloud_effective_radius", "cloud_effective_radius", c) for c in range(atm.cloud_type.shape[1])]
    if atm.aerosol_type is not None:
        groups += [("aerosol_concentration", "aerosol_concentration", a) for a in range(atm.aerosol_type.shape[1])]
        groups += [("aerosol_effective_radius", "aerosol_effective_radius", a)
                   for a in range(atm.aerosol_type.shape[1])]
    checked = 0
    for k in layers:
        for kname, aname, c in groups:
            amount = getattr(atm, "cloud_water_content" if kname.startswith("cloud") else "aerosol_concentration")
            on = amount[:, c, k] > (1e-6 if kname.startswith("cloud") else 1e-9)
            if kname.startswith("cloud") and atm.cloud_fraction is not None:
                on &= atm.cloud_fraction[:, k] >= 1e-12
            if not on.any():
                continue
            val = getattr(atm, aname)[:, c, k]
            step = np.where(on, 1e-4 * val, 0.0)

            def pert(a, s_, o, h, aname=aname, c=c, k=k):
                getattr(a, aname)[:, c, k] += h
            got = getattr(km, kname)[:, :, c, k]
            fd = _fd_best(orc, d, atm, sfc, geo, opt, pert, step, got, mult)
            scale = max(np.abs(getattr(km, kname)[:, :, c] * getattr(atm, aname)[:, None, c]).max(), 1e-12)
            err = np.abs((got - fd)[on] * val[on, None]).max()
            assert err <= tol * scale, (kname, c, k, err / scale)
            checked += 1
        if fraction:
            on = atm.cloud_fraction[:, k] > 0.0
            if on.any():
                def pf(a, s_, o, h, k=k):
                    a.cloud_fraction[:, k] += h
                got = km.cloud_fraction[:, :, k]
                fd = _fd_best(orc, d, atm, sfc, geo, opt, pf, np.where(on, 1e-6, 0.0), got, fraction_mult)
                scale = max(np.abs(km.cloud_fraction).max(), 1e-12)
                assert np.abs((got - fd)[on]).max() <= max(1e-4, tol) * scale, ("cloud_fraction", k)
                checked += 1
    assert checked > 0


def _check_surface(km, orc, d, atm, sfc, geo, opt, mult=(1.0,), tol=FD_TOL):
    def pw(a, s, o, h):
        s.water_temperature += h
    fd = _fd_best(orc, d, atm, sfc, geo, opt, pw, 1e-3, km.water_temperature, mult)
    assert np.abs(km.water_temperature - fd).max() <= tol * np.abs(fd).max()

    def pe(a, s, o, h):
        o.emissivity = o.emissivity + h
    fd = _fd_best(orc, d, atm, sfc, geo, opt, pe, 1e-5, km.surface_emissivity, mult)
    assert np.abs(km.surface_emissivity - fd).max() <= tol * np.abs(fd).max()


def _layers(atm, extra=(3, 30, 60, 90)):
    """Layers to difference: a few fixed ones plus the cloudy layers of profile 0."""
    ks = set(k for k in extra if k < int(atm.n_layers.min()))
    if atm.cloud_water_content is not None:
        ks |= set(np.nonzero(atm.cloud_water_content[0].max(axis=0) > 0)[0][:4].tolist())
    return sorted(ks)


@pytest.mark.parametrize("sensor,nl,n_streams,wc_scale,cover", [
    ("mwsynth_c16", 100, None, 100.0, None),     # stream rule
    ("mwsynth_c16", 100, 16, 100.0, None),       # Options%n_Streams = 16
    ("irsynth_c616", 101, None, 30.0, None),
    ("mwsynth_c16", 100, None, 100.0, (0.1, 0.9)),    # fractional cover, average overlap
    ("irsynth_c616", 101, 8, 30.0, (0.1, 0.9))])
def test_cloudy_k_matrix_matches_oracle_differences(gpu_lib, cloud_dir, sensor, nl, n_streams, wc_scale, cover):
    from oracle.pyoracle import Oracle
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 4, nl, 81, wc_scale=wc_scale, n_streams=n_streams)
    if cover is not None:
        sy.add_clouds(atm, (co.WATER_CLOUD, co.ICE_CLOUD, co.RAIN_CLOUD, co.SNOW_CLOUD), 80, wc_scale=wc_scale,
                      cover=cover)
        opt.overlap_id = np.array([4, 3, 4, 1], np.int32)
    atm.n_clouds[2] = 0   # one clear profile in the batch
    h = gpu_lib.CRTM([sensor], cloud_dir, 0)
    km, rts = h.k_matrix(atm, sfc, geo, opt)
    orc = Oracle(cloud_dir, sensor)
    _, bt = orc.forward_scatter(atm, sfc, geo, opt, f"{cloud_dir}/CloudCoeff.bin", n_threads=8)
    assert np.abs(rts.brightness_temperature - bt).max() <= 1e-4
    _check_layers(km, orc, cloud_dir, atm, sfc, geo, opt, _layers(atm))
    _check_surface(km, orc, cloud_dir, atm, sfc, geo, opt)
    _check_species(km, orc, cloud_dir, atm, sfc, geo, opt, _layers(atm, ())[:4], fraction=cover is not None)


def test_aerosol_k_matrix_matches_oracle_differences(gpu_lib, cloud_dir):
    """IR sensor, liquid and ice clouds plus dust, sea salt and sulfate; one
    profile with aerosols only, one clear."""
    from oracle.pyoracle import Oracle
    sensor = "irsynth_c616"
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, 4, 101, 82)
    sy.add_clouds(atm, (co.WATER_CLOUD, co.ICE_CLOUD), 83, wc_scale=30.0)
    sy.add_aerosols(atm, sy.AEROSOL_TYPES, 84, load_scale=20.0)
    atm.n_clouds[1] = 0
    atm.n_clouds[3] = 0
    atm.n_aerosols[3] = 0
    km, rts = gpu_lib.CRTM([sensor], cloud_dir, 0).k_matrix(atm, sfc, geo, opt)
    orc = Oracle(cloud_dir, sensor)
    _check_layers(km, orc, cloud_dir, atm, sfc, geo, opt, _layers(atm, (10, 50, 80, 100)))
    _check_surface(km, orc, cloud_dir, atm, sfc, geo, opt)
    _check_species(km, orc, cloud_dir, atm, sfc, geo, opt, _layers(atm, (30, 90))[:4])


@pytest.mark.parametrize("scheme", ["CMAQ", "GOCART-GEOS5", "NAAPS"])
def test_aerosol_scheme_k_matrix_matches_oracle_differences(gpu_lib, cloud_dir, scheme):
    """K-matrix under CRTM_Init's other aerosol models: concentration (and, for
    'CMAQ', radius and Effective_Variance; for 'GOCART-GEOS5' / 'NAAPS' the
    layers' Relative_Humidity, summed over the aerosols that read it) against
    central differences of the oracle's forward in the same scheme; the
    coordinates a scheme does not read have zero Jacobians.  The adjoint is
    the seeded K-matrix summed over channels."""
    from oracle.pyoracle import Oracle
    sensor = "irsynth_c616"
    apath = sy.write_aerosol_files(cloud_dir, scheme)
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, 4, 101, 97)
    sy.add_clouds(atm, (co.WATER_CLOUD, co.ICE_CLOUD), 98, wc_scale=30.0)
    sy.add_aerosols(atm, sy.AEROSOL_TYPES, 99, load_scale=20.0)
    sy.add_aerosol_scheme_inputs(atm, 100)
    atm.n_clouds[1] = 0
    atm.n_aerosols[3] = 0
    h = gpu_lib.CRTM([sensor], cloud_dir, 0, aerosol_model=scheme, aerosol_coeff_file=sy.aerosol_file_name(scheme))
    km, rts = h.k_matrix(atm, sfc, geo, opt)
    orc = Oracle(cloud_dir, sensor)
    _, bt = orc.forward_scatter(atm, sfc, geo, opt, f"{cloud_dir}/CloudCoeff.bin", apath, n_threads=8,
                                aerosol_scheme=scheme)
    assert np.abs(rts.brightness_temperature - bt).max() <= 1e-4

    def fd(perturb, step):
        out = []
        for sgn in (1.0, -1.0):
            a = copy.deepcopy(atm)
            perturb(a, sgn * step)
            out.append(orc.forward_scatter(a, sfc, geo, opt, f"{cloud_dir}/CloudCoeff.bin", apath, n_threads=8,
                                           aerosol_scheme=scheme)[1])
        st = np.asarray(step, np.float64)
        den = 2.0 * (st[:, None] if st.ndim else st)
        return (out[0] - out[1]) / np.where(den == 0.0, 1.0, den)
    layers = sorted(set([5, 40, 80, 95]) | set(np.nonzero(atm.aerosol_concentration[0].max(axis=0) > 1e-7)[0][-3:]))
    fields = [("aerosol_concentration", "aerosol_concentration")]
    if scheme == "CMAQ":
        fields += [("aerosol_effective_radius", "aerosol_effective_radius"),
                   ("aerosol_effective_variance", "aerosol_effective_variance")]
    checked = 0
    for k in layers:
        for kname, aname in fields:
            for c in range(atm.aerosol_type.shape[1]):
                val = getattr(atm, aname)[:, c, k]
                on = atm.aerosol_concentration[:, c, k] > 1e-9
                if not on.any():
                    continue

                def pert(a, hh, aname=aname, c=c, k=k):
                    getattr(a, aname)[:, c, k] += hh
                d = fd(pert, np.where(on, 1e-4 * val, 0.0))
                got = getattr(km, kname)[:, :, c, k]
                scale = max(np.abs(getattr(km, kname)[:, :, c] * getattr(atm, aname)[:, None, c]).max(), 1e-12)
                err = np.abs((got - d)[on] * val[on, None]).max()
                assert err <= FD_TOL * scale, (kname, c, k, err / scale)
                checked += 1
        if scheme != "CMAQ":
            on = (atm.aerosol_concentration[:, :, k] > 1e-9).any(axis=1) & (atm.relative_humidity[:, k] > 0.0)
            if on.any():
                def prh(a, hh, k=k):
                    a.relative_humidity[:, k] += hh
                d = fd(prh, np.where(on, 1e-4 * atm.relative_humidity[:, k], 0.0))
                got = km.relative_humidity[:, :, k]
                scale = max(np.abs(km.relative_humidity * atm.relative_humidity[:, None, :]).max(), 1e-12)
                err = np.abs((got - d)[on] * atm.relative_humidity[on, k][:, None]).max()
                assert err <= FD_TOL * scale, ("relative_humidity", k, err / scale)
                checked += 1
    assert checked > 0
    if scheme == "CMAQ":
        assert np.abs(km.aerosol_effective_variance).max() > 0
        assert getattr(km, "relative_humidity", None) is None
    else:
        assert np.abs(km.relative_humidity).max() > 0
        assert np.abs(km.aerosol_effective_radius).max() == 0.0
    # adjoint = seeded K-matrix summed over the channels
    seed = np.random.Generator(np.random.PCG64(101)).standard_normal((4, 616))
    km2, _ = h.k_matrix(atm, sfc, geo, opt, seed)
    ad, _ = h.adjoint(atm, sfc, geo, opt, seed)
    for f in ("aerosol_concentration", "aerosol_effective_radius",
              "aerosol_effective_variance" if scheme == "CMAQ" else "relative_humidity"):
        assert _rel(ad[f], getattr(km2, f).sum(axis=1)) <= 1e-10, f


@pytest.mark.parametrize("sensor,n_streams", [("mwsynth_c16", None), ("irsynth_c616", None),
                                              ("mwsynth_c16", 8)])
def test_mixed_cloudy_k_matrix_matches_fp64(gpu_lib, cloud_dir, sensor, n_streams):
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 24, 100, 85, wc_scale=100.0, n_streams=n_streams)
    atm.n_clouds[::5] = 0
    ref = gpu_lib.CRTM([sensor], cloud_dir, 0).k_matrix(atm, sfc, geo, opt)
    mix = gpu_lib.CRTM([sensor], cloud_dir, 1).k_matrix(atm, sfc, geo, opt)
    assert np.abs(mix[1].brightness_temperature - ref[1].brightness_temperature).max() <= 1e-2
    for f in ("temperature", "absorber", "water_temperature", "surface_emissivity", "cloud_water_content",
              "cloud_effective_radius"):
        assert _rel(getattr(mix[0], f), getattr(ref[0], f)) <= MIX_TOL, f


@pytest.mark.parametrize("precision", [0, 1])
def test_cloudy_k_matrix_radiance_matches_forward(gpu_lib, cloud_dir, precision):
    """The K-matrix returns the forward radiance.  In the mixed form the
    forward adds FP32 layer records in FP64 and the K-matrix adds them in FP32
    (with the (I - Rup R)^-1 inversions in FP64), so the two agree within the
    form's 0.01 K budget there; to 1e-6 K in the FP64 form."""
    atm, sfc, geo, opt = sy.cloudy_workload("mwsynth_c16", 12, 100, 86, wc_scale=300.0)
    h = gpu_lib.CRTM(["mwsynth_c16"], cloud_dir, precision)
    fw = h.forward(atm, sfc, geo, opt)
    _, rts = h.k_matrix(atm, sfc, geo, opt)
    assert np.abs(rts.brightness_temperature - fw.brightness_temperature).max() <= (1e-6 if precision == 0
                                                                                   else 1e-2)


@pytest.mark.parametrize("precision", [0, 1])
def test_cloudy_adjoint_is_seeded_k_matrix_sum(gpu_lib, cloud_dir, precision):
    """Adjoint of a BT seed = sum over channels of seed x K (CRTM_Adjoint vs
    CRTM_K_Matrix with the same seed)."""
    sensor = "irsynth_c616"
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 9, 101, 87, wc_scale=30.0)
    sy.add_clouds(atm, (co.WATER_CLOUD, co.ICE_CLOUD), 86, wc_scale=30.0, cover=(0.1, 1.0))
    opt.overlap_id = np.array([1, 2, 3, 4, 5, 4, 4, 3, 2], np.int32)
    sy.add_aerosols(atm, sy.AEROSOL_TYPES, 88, load_scale=20.0)
    atm.n_clouds[4] = 0
    atm.n_aerosols[7] = 0
    seed = np.random.Generator(np.random.PCG64(89)).standard_normal((9, 616))
    h = gpu_lib.CRTM([sensor], cloud_dir, precision)
    km, _ = h.k_matrix(atm, sfc, geo, opt, seed)
    ad, _ = h.adjoint(atm, sfc, geo, opt, seed)
    tol = 1e-10 if precision == 0 else 1e-5
    assert _rel(ad["temperature"], km.temperature.sum(axis=1)) <= tol
    assert _rel(ad["absorber"], km.absorber.sum(axis=1)) <= tol
    assert _rel(ad["water_temperature"], km.water_temperature.sum(axis=1)) <= tol
    for f in ("cloud_water_content", "cloud_effective_radius", "cloud_fraction", "aerosol_concentration",
              "aerosol_effective_radius"):
        assert _rel(ad[f], getattr(km, f).sum(axis=1)) <= tol, f


def test_clear_profile_in_cloudy_batch_keeps_clear_k_matrix(gpu_lib, cloud_dir):
    sensor = "mwsynth_c16"
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 5, 100, 90, wc_scale=100.0)
    atm.n_clouds[1] = 0
    h = gpu_lib.CRTM([sensor], cloud_dir, 0)
    km, _ = h.k_matrix(atm, sfc, geo, opt)
    clear = copy.deepcopy(atm)
    clear.n_clouds = clear.cloud_type = clear.cloud_water_content = None
    clear.cloud_effective_radius = clear.cloud_fraction = None
    kc, _ = h.k_matrix(clear, sfc, geo, opt)
    assert _rel(km.temperature[1], kc.temperature[1]) <= 1e-12
    assert _rel(km.absorber[1], kc.absorber[1]) <= 1e-12
    assert np.abs(km.temperature[0] - kc.temperature[0]).max() > 1e-6   # the clouds do matter


def test_isothermal_enclosure_k_matrix_sum_rule(gpu_lib, cloud_dir, tmp_path):
    """Isothermal scene at 250 K with cosmic background c = B(250 K): BT = 250 K
    whatever the clouds and absorbers.  Raising every temperature and c together
    by dT raises BT by dT, so sum_k K_T(k) + K_Ts + dR/dc = 1 for every channel
    (dBT/dR . dB/dT = 1 with the same band correction).  R is linear in c, so
    dR/dc comes exactly from a second forward run with c scaled by 1 + 1e-3."""
    import os
    import shutil
    sensor = "mwsynth_c16"
    sc = co.read_spccoeff(f"{cloud_dir}/{sensor}.SpcCoeff.bin")
    te = sc.band_c1 + sc.band_c2 * 250.0
    cosmic = sc.planck_c1 / (np.exp(sc.planck_c2 / te) - 1.0)
    dirs = []
    for i, c in enumerate((cosmic, cosmic * (1.0 + 1e-3))):
        d = tmp_path / f"c{i}"
        os.makedirs(d)
        sc.cosmic_background_radiance = c
        co.write_spccoeff(str(d / f"{sensor}.SpcCoeff.bin"), sc)
        shutil.copy(f"{cloud_dir}/{sensor}.TauCoeff.bin", d / f"{sensor}.TauCoeff.bin")
        shutil.copy(f"{cloud_dir}/CloudCoeff.bin", d / "CloudCoeff.bin")
        dirs.append(str(d))
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 64, 100, 91, wc_scale=300.0)
    for m in range(64):
        atm.temperature[m, :atm.n_layers[m]] = 250.0
    sfc.land_coverage[:] = sfc.snow_coverage[:] = sfc.ice_coverage[:] = 0.0
    sfc.water_coverage[:] = 1.0
    sfc.water_temperature[:] = 250.0
    km, rts = gpu_lib.CRTM([sensor], dirs[0], 0).k_matrix(atm, sfc, geo, opt)
    assert np.abs(rts.brightness_temperature - 250.0).max() < 1e-8
    r2 = gpu_lib.CRTM([sensor], dirs[1], 0).forward(atm, sfc, geo, opt).radiance
    dr_dc = (r2 - rts.radiance) / (cosmic * 1e-3)[None, :]
    total = km.temperature.sum(axis=2) + km.water_temperature + dr_dc
    assert np.abs(total - 1.0).max() < 1e-8
    assert dr_dc.max() > 1e-3   # the clouds reflect part of the cosmic background


@pytest.mark.parametrize("sensor,nl,n_streams,wc_scale,cover", [
    ("mwsynth_c16", 100, None, 300.0, None),
    ("mwsynth_c16", 100, 16, 100.0, None),
    ("mwsynth_c16", 100, None, 100.0, (0.1, 0.9)),
    ("irsynth_c616", 101, 8, 30.0, (0.1, 0.9))])
def test_soi_k_matrix_matches_oracle_differences(gpu_lib, cloud_dir, sensor, nl, n_streams, wc_scale, cover):
    """SOI profiles (Options%RT_Algorithm_Id = RT_SOI) next to an ADA and a
    clear one: the adjoint of the orders of interaction against central
    differences of the oracle's SOI forward.

    Microwave (4-5 orders): every Jacobian layer by layer, best of a 10x and
    a 1x step (the ADA test's steps; 1000x-10x for the cloud fraction, whose
    1e-6 step is below the doubling's rounding noise), within 3e-4 of the
    largest Jacobian of the variable.  Infrared (14-60 orders with these clouds): the forward is
    not smooth at the 1e-3 level there.  Its doubling (up to ~30 doublings of
    a 1e-8 thin layer) leaves rounding noise of ~1e-6 K in the brightness
    temperature, and its stopping rule (the newest order below 1e-4 of the
    radiance) jumps by up to ~0.01 K where a step changes the count of
    orders.  So temperature, surface and cloud Jacobians take the elementwise
    best of a ladder of steps (10x, 1x, 0.1x; 1000x-10x for the cloud
    fraction) within 1e-3; the absorbers, whose one-layer steps move the
    radiance by less than the noise and whose column steps cross the jumps,
    are checked on the microwave cases only.  The same physics code is held
    to 2e-5 of central differences with chosen steps on the CPU
    (tests/test_scatter_harness.py)."""
    from oracle.pyoracle import Oracle
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 4, nl, 93, wc_scale=wc_scale, n_streams=n_streams)
    if cover is not None:
        sy.add_clouds(atm, (co.WATER_CLOUD, co.ICE_CLOUD, co.RAIN_CLOUD, co.SNOW_CLOUD), 94, wc_scale=wc_scale,
                      cover=cover)
        opt.overlap_id = np.array([4, 3, 4, 2], np.int32)
    opt.rt_algorithm_id = np.array([RT_SOI, RT_SOI, 56, RT_SOI], np.int32)
    atm.n_clouds[1] = 0   # clear profile (SOI requested, clear-sky Emission)
    h = gpu_lib.CRTM([sensor], cloud_dir, 0)
    km, rts = h.k_matrix(atm, sfc, geo, opt)
    orc = Oracle(cloud_dir, sensor)
    _, bt = orc.forward_scatter(atm, sfc, geo, opt, f"{cloud_dir}/CloudCoeff.bin", n_threads=8)
    assert np.abs(rts.brightness_temperature - bt).max() <= 1e-4
    fw = h.forward(atm, sfc, geo, opt)
    assert np.abs(rts.brightness_temperature - fw.brightness_temperature).max() <= 1e-6
    mw = sensor.startswith("mw")
    mult, tol = ((10.0, 1.0), 3e-4) if mw else ((10.0, 1.0, 0.1), 1e-3)
    _check_layers(km, orc, cloud_dir, atm, sfc, geo, opt, _layers(atm), mult, tol, absorbers=mw)
    _check_surface(km, orc, cloud_dir, atm, sfc, geo, opt, mult, tol)
    _check_species(km, orc, cloud_dir, atm, sfc, geo, opt, _layers(atm, ())[:4], fraction=cover is not None,
                   mult=mult, tol=tol, fraction_mult=(1000.0, 100.0, 10.0))


def test_soi_k_matrix_checkpoints_match_kept_orders(gpu_lib, cloud_dir, monkeypatch):
    """With 17 order-field slots the IR orders beyond 17 are recomputed from
    checkpoints: the same K-matrix, bit for bit, as with all 75 kept; and the
    SOI adjoint is the seeded K-matrix summed over channels."""
    sensor = "irsynth_c616"
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 3, 101, 95, wc_scale=100.0, n_streams=8)
    opt.rt_algorithm_id = np.full(3, RT_SOI, np.int32)
    out = []
    for slots in ("17", "75"):
        monkeypatch.setenv("CRTM_GPU_SOI_SLOTS", slots)
        out.append(gpu_lib.CRTM([sensor], cloud_dir, 0).k_matrix(atm, sfc, geo, opt))
    for f in ("temperature", "absorber", "water_temperature", "surface_emissivity", "cloud_water_content",
              "cloud_effective_radius"):
        assert np.array_equal(getattr(out[0][0], f), getattr(out[1][0], f)), f
    assert np.array_equal(out[0][1].radiance, out[1][1].radiance)
    seed = np.random.Generator(np.random.PCG64(96)).standard_normal((3, 616))
    h = gpu_lib.CRTM([sensor], cloud_dir, 0)
    km, _ = h.k_matrix(atm, sfc, geo, opt, seed)
    ad, _ = h.adjoint(atm, sfc, geo, opt, seed)
    for f in ("temperature", "absorber", "water_temperature", "cloud_water_content", "cloud_effective_radius"):
        assert _rel(ad[f], getattr(km, f).sum(axis=1)) <= 1e-10, f
