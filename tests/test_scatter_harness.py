"""The GPU library's cloud/ADA physics header (scatter_physics.cuh), compiled
for the CPU, against the oracle: one ADA layer, and whole cloudy
(profile, channel) radiances given the oracle's gas layer optical depths."""
import ctypes as ct
import os
import shutil
import subprocess

import numpy as np
import pytest

from crtmv3_gb300 import coefficients as co, synthetic as sy

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
_dp = ct.POINTER(ct.c_double)
_ip = ct.POINTER(ct.c_int)


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


@pytest.fixture(scope="module")
def sx(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    out = str(tmp_path_factory.mktemp("sx") / "libsx.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I",
                    os.path.join(ROOT, "crtmv3_gb300", "csrc"), "-o", out,
                    os.path.join(HERE, "harness", "scatter_harness.cpp")], check=True)
    return ct.CDLL(out)


@pytest.mark.parametrize("nleg,mu_s", [(2, 0.9), (4, 0.55), (6, 0.8), (8, 0.66), (16, 0.93)])
@pytest.mark.parametrize("w,tau", [(0.6, 0.5), (0.98, 6.0), (0.3, 5e-9), (0.05, 0.02)])
def test_ada_layer_matches_oracle(sx, nleg, mu_s, w, tau):
    from oracle.pyoracle import lib
    pc = 0.5 * 0.8 ** np.arange(nleg + 1)
    mu, wt = np.zeros(20), np.zeros(20)
    ff, bb = np.zeros(400), np.zeros(400)
    nz = ct.c_int(0)
    lib().or_phase_setup(nleg, mu_s, _p(pc), _p(mu), _p(wt), _p(ff), _p(bb), ct.byref(nz))
    nZ, nS = nz.value, (nleg + 2) // 2
    outs = [[np.zeros(nZ * nZ), np.zeros(nZ * nZ), np.zeros(nZ)] for _ in range(2)]
    assert lib().or_amom_layer(nS, nZ, w, tau, _p(mu), _p(wt), _p(ff), _p(bb), 1.7,
                               *[_p(x) for x in outs[0]]) == 0
    assert sx.sx_ada_layer(nS, nZ, ct.c_double(w), ct.c_double(tau), _p(mu), _p(wt), _p(ff), _p(bb),
                           ct.c_double(1.7), *[_p(x) for x in outs[1]]) == 0
    for a, b in zip(*outs):
        assert np.abs(a - b).max() < 1e-12


@pytest.mark.parametrize("sensor,nl,n_streams,soi,aer,scheme", [
    ("mwsynth_c16", 100, None, 0, 0, "CRTM"), ("mwsynth_c16", 100, 16, 0, 0, "CRTM"),
    ("irsynth_c616", 101, None, 0, 0, "CRTM"), ("mwsynth_c22", 100, 8, 0, 0, "CRTM"),
    ("mwsynth_c16", 100, None, 1, 0, "CRTM"), ("mwsynth_c16", 100, 16, 1, 0, "CRTM"),
    ("irsynth_c616", 101, None, 1, 0, "CRTM"), ("mwsynth_c16", 100, None, 2, 0, "CRTM"),
    ("irsynth_c616", 101, None, 2, 0, "CRTM"), ("irsynth_c616", 101, None, 0, 1, "CRTM"),
    ("irsynth_c616", 101, 8, 1, 1, "CRTM"), ("irsynth_c616", 101, None, 0, 2, "CRTM"),
    ("mwsynth_c16", 100, None, 0, 1, "CRTM"), ("mwsynth_c16", 100, None, 3, 0, "CRTM"),
    ("irsynth_c616", 101, None, 3, 1, "CRTM"), ("irsynth_c616", 101, None, 3, 2, "CRTM"),
    ("irsynth_c616", 101, None, 0, 1, "CMAQ"), ("irsynth_c616", 101, 8, 1, 2, "CMAQ"),
    ("irsynth_c616", 101, None, 0, 1, "GOCART-GEOS5"), ("irsynth_c616", 101, None, 1, 2, "NAAPS")])
def test_cloudy_radiance_matches_oracle(sx, coeff_dir, sensor, nl, n_streams, soi, aer, scheme):
    """aer 1: clouds and aerosols; aer 2: aerosols only.  soi 2 / 3: layered
    ADA as the GPU kernels run it, with the layer optics in FP64 / in
    double-float (the mixed form).  scheme: the AerosolCoeff scheme
    (CRTM_Init's Aerosol_Model) with its effective variance and relative
    humidity inputs."""
    from oracle.pyoracle import Oracle
    path = sy.write_cloud_files(coeff_dir)
    apath = sy.write_aerosol_files(coeff_dir, scheme)
    cc = co.read_cloudcoeff(path)
    ac = co.read_aerosolcoeff(apath, scheme)
    sc = co.read_spccoeff(f"{coeff_dir}/{sensor}.SpcCoeff.bin")
    o = Oracle(coeff_dir, sensor)
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 3, nl, 51, wc_scale=200.0, n_streams=n_streams)
    if soi == 1:
        opt.rt_algorithm_id = np.full(atm.n_profiles, 168, np.int32)
    if aer:
        sy.add_aerosols(atm, sy.AEROSOL_TYPES, 52, load_scale=30.0)
        sy.add_aerosol_scheme_inputs(atm, 53)
    if aer == 2:
        atm.n_clouds[:] = 0
    rad_ref, _ = o.forward_scatter(atm, sfc, geo, opt, path, apath if aer else None, aerosol_scheme=scheme)
    _, _, lod = o.forward(atm, sfc, geo, opt, layer_od=True)
    f = lambda a: np.ascontiguousarray(np.ravel(a, order="F"))   # noqa: E731
    arrs = [f(x) for x in (cc.frequency_mw, cc.reff_mw, cc.temperature, cc.frequency_ir, cc.reff_ir,
                           cc.ke_l_mw, cc.w_l_mw, cc.pcoeff_l_mw, cc.ke_s_mw, cc.w_s_mw, cc.pcoeff_s_mw,
                           cc.ke_ir, cc.w_ir, cc.pcoeff_ir)]
    dims = np.array([cc.frequency_mw.size, cc.reff_mw.size, cc.temperature.size, cc.density_mw.size,
                     cc.frequency_ir.size, cc.reff_ir.size, cc.n_legendre_terms], np.int32)
    mw = sc.sensor_type == co.MICROWAVE_SENSOR
    adims = np.array([ac.wavelength.size, ac.ke.shape[1], ac.ke.shape[2], ac.ke.shape[3], ac.ke.shape[4],
                      ac.pcoeff.shape[5] - 1, co.AEROSOL_SCHEMES.index(scheme), ac.rh.size], np.int32)
    aarrs = [np.ascontiguousarray(ac.type_id, np.int32)] + [f(x) for x in (
        1.0e4 / ac.wavelength, ac.reff, ac.rsig, ac.rh, ac.ke, ac.w, ac.pcoeff[..., 0])]
    L = sc.n_channels
    chans = range(0, L, max(1, L // 40))
    worst = 0.0
    for m in range(atm.n_profiles):
        Ku = int(atm.n_layers[m])
        ts = sfc.water_temperature[m]
        mu = np.cos(np.deg2rad(geo.sensor_zenith_angle[m]))
        temp = np.ascontiguousarray(atm.temperature[m, :Ku])
        NC = atm.cloud_type.shape[1]
        wc = np.ascontiguousarray(atm.cloud_water_content[m])
        re = np.ascontiguousarray(atm.cloud_effective_radius[m])
        ctype = np.ascontiguousarray(atm.cloud_type[m], np.int32)
        nc = int(atm.n_clouds[m])
        na = int(atm.n_aerosols[m]) if aer else 0
        atype = np.ascontiguousarray(atm.aerosol_type[m] if aer else np.zeros(1), np.int32)
        conc = np.ascontiguousarray(atm.aerosol_concentration[m] if aer else np.zeros((1, atm.max_layers)))
        areff = np.ascontiguousarray(atm.aerosol_effective_radius[m] if aer else np.zeros((1, atm.max_layers)))
        avar = np.ascontiguousarray(atm.aerosol_effective_variance[m] if aer else np.zeros((1, atm.max_layers)))
        rhl = np.ascontiguousarray(atm.relative_humidity[m] if aer else np.zeros(atm.max_layers))
        for l in chans:
            planck = np.array([sc.planck_c1[l], sc.planck_c2[l], sc.band_c1[l], sc.band_c2[l]])
            te = sc.band_c1[l] + sc.band_c2[l] * ts
            bs = sc.planck_c1[l] / (np.exp(sc.planck_c2[l] / te) - 1.0)
            if n_streams:
                nleg = n_streams
            else:
                mr = max(re[:nc, :Ku].max() if nc else 0.0, areff[:na, :Ku].max() if na else 0.0)
                nleg = sx.sx_stream_rule(ct.c_double(mr), ct.c_double(sc.wavenumber[l]))
            od = np.ascontiguousarray(lod[m, l, :Ku])
            r = ct.c_double(0.0)
            rc = sx.sx_cloudy_radiance(
                _p(dims, _ip), *[_p(a) for a in arrs], Ku, nc, nleg, int(mw),
                ct.c_double(sc.frequency[l] if mw else sc.wavenumber[l]), ct.c_double(mu),
                ct.c_double(opt.emissivity[m, l]), ct.c_double(bs),
                ct.c_double(sc.cosmic_background_radiance[l]), _p(planck), _p(temp), _p(ctype, _ip),
                _p(wc), _p(re), atm.max_layers, _p(od), soi, na, _p(atype, _ip), _p(conc), _p(areff),
                _p(avar), _p(rhl), _p(adims, _ip), _p(aarrs[0], _ip), *[_p(a) for a in aarrs[1:]],
                ct.c_double(sc.wavenumber[l]), ct.byref(r))
            assert rc == 0
            worst = max(worst, abs(r.value - rad_ref[m, l]) / abs(rad_ref[m, l]))
    assert worst < 1e-11


@pytest.mark.parametrize("sensor,nleg,wc_scale", [("mwsynth_c16", 6, 300.0), ("mwsynth_c16", 16, 100.0),
                                                  ("irsynth_c616", 6, 100.0), ("mwsynth_c16", 2, 50.0)])
def test_layer_derivatives_match_finite_differences(sx, coeff_dir, sensor, nleg, wc_scale):
    """d(layer T, R, source, optical depth) / d(gas optical depth) and / d(temperature)
    from derivative numbers through the cloud LUT, combine, phase blocks and
    MOM (eigen-perturbation), against central differences of the FP64 forward."""
    path = sy.write_cloud_files(coeff_dir)
    cc = co.read_cloudcoeff(path)
    sc = co.read_spccoeff(f"{coeff_dir}/{sensor}.SpcCoeff.bin")
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 2, 100, 53, wc_scale=wc_scale,
                                            cloud_types=(co.WATER_CLOUD, co.RAIN_CLOUD, co.SNOW_CLOUD))
    f = lambda a: np.ascontiguousarray(np.ravel(a, order="F"))   # noqa: E731
    arrs = [f(x) for x in (cc.frequency_mw, cc.reff_mw, cc.temperature, cc.frequency_ir, cc.reff_ir,
                           cc.ke_l_mw, cc.w_l_mw, cc.pcoeff_l_mw, cc.ke_s_mw, cc.w_s_mw, cc.pcoeff_s_mw,
                           cc.ke_ir, cc.w_ir, cc.pcoeff_ir)]
    dims = np.array([cc.frequency_mw.size, cc.reff_mw.size, cc.temperature.size, cc.density_mw.size,
                     cc.frequency_ir.size, cc.reff_ir.size, cc.n_legendre_terms], np.int32)
    mw = sc.sensor_type == co.MICROWAVE_SENSOR
    m = 0
    wc = np.ascontiguousarray(atm.cloud_water_content[m])
    re = np.ascontiguousarray(atm.cloud_effective_radius[m])
    ctype = np.ascontiguousarray(atm.cloud_type[m], np.int32)
    NC = ctype.size
    cloudy = np.where((wc > 1e-6).any(axis=0))[0]
    n = 30 * 30
    checked = 0
    for k in cloudy[:6]:
        for l in (0, sc.n_channels // 2):
            planck = np.array([sc.planck_c1[l], sc.planck_c2[l], sc.band_c1[l], sc.band_c2[l]])
            fr = sc.frequency[l] if mw else sc.wavenumber[l]

            def rec(gas, tk):
                outs = [np.zeros(2 * 20 * 20 + 40) for _ in range(3)]
                nz = ct.c_int(0)
                kind = sx.sx_layer_record(_p(dims, _ip), *[_p(a) for a in arrs], NC, nleg, int(mw),
                                          ct.c_double(fr), ct.c_double(0.83), _p(planck), _p(ctype, _ip),
                                          _p(wc), _p(re), atm.max_layers, int(k), ct.c_double(gas),
                                          ct.c_double(tk), *[_p(o) for o in outs], ct.byref(nz))
                nZ = nz.value
                ne = 1 + 2 * nZ * nZ + nZ
                return kind, [o[:ne] for o in outs]
            gas, tk = 0.05, float(atm.temperature[m, k])
            kind, (v, dg, dt) = rec(gas, tk)
            if kind != 1:
                continue
            for h, d, which in ((1e-6, dg, 0), (1e-4, dt, 1)):
                args_p = (gas + h, tk) if which == 0 else (gas, tk + h)
                args_m = (gas - h, tk) if which == 0 else (gas, tk - h)
                fd = (rec(*args_p)[1][0] - rec(*args_m)[1][0]) / (2 * h)
                scale = np.abs(fd).max() + 1e-12
                assert np.abs(fd - d).max() <= 1e-6 * scale + 1e-10, (k, l, which)
            checked += 1
    assert checked > 0


@pytest.mark.parametrize("sensor,nl,n_streams,wc_scale,soi", [("mwsynth_c16", 100, None, 300.0, 0),
                                                              ("mwsynth_c16", 100, 16, 100.0, 0),
                                                              ("irsynth_c616", 101, None, 100.0, 0),
                                                              ("mwsynth_c16", 100, None, 300.0, 75),
                                                              ("mwsynth_c16", 100, 16, 100.0, 75),
                                                              ("irsynth_c616", 101, None, 100.0, 75),
                                                              ("irsynth_c616", 101, 8, 100.0, 17)])
def test_cloudy_kmatrix_matches_finite_differences(sx, coeff_dir, sensor, nl, n_streams, wc_scale, soi):
    """K-matrix of one cloudy (profile, channel) against central differences
    of the FP64 cloudy radiance with respect to each layer's gas optical
    depth and temperature, each cloud's water content and effective radius,
    the surface emissivity and the surface Planck radiance.  soi 0: ADA
    (adjoint of the adding); soi > 0: SOI with that many order-field slots
    (the adjoint of the orders of interaction; 17 slots recompute from
    checkpoints once an IR channel needs more orders).  Both contract the
    record adjoints on derivative numbers through the layer optics."""
    path = sy.write_cloud_files(coeff_dir)
    cc = co.read_cloudcoeff(path)
    sc = co.read_spccoeff(f"{coeff_dir}/{sensor}.SpcCoeff.bin")
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 1, nl, 54, wc_scale=wc_scale, n_streams=n_streams)
    f = lambda a: np.ascontiguousarray(np.ravel(a, order="F"))   # noqa: E731
    arrs = [f(x) for x in (cc.frequency_mw, cc.reff_mw, cc.temperature, cc.frequency_ir, cc.reff_ir,
                           cc.ke_l_mw, cc.w_l_mw, cc.pcoeff_l_mw, cc.ke_s_mw, cc.w_s_mw, cc.pcoeff_s_mw,
                           cc.ke_ir, cc.w_ir, cc.pcoeff_ir)]
    dims = np.array([cc.frequency_mw.size, cc.reff_mw.size, cc.temperature.size, cc.density_mw.size,
                     cc.frequency_ir.size, cc.reff_ir.size, cc.n_legendre_terms], np.int32)
    mw = sc.sensor_type == co.MICROWAVE_SENSOR
    m, Ku = 0, int(atm.n_layers[0])
    temp0 = np.ascontiguousarray(atm.temperature[m, :Ku])
    wc = np.ascontiguousarray(atm.cloud_water_content[m])
    re = np.ascontiguousarray(atm.cloud_effective_radius[m])
    ctype = np.ascontiguousarray(atm.cloud_type[m], np.int32)
    od0 = np.full(Ku, 0.02) * (1.0 + 0.5 * np.sin(np.arange(Ku)))
    mu = np.cos(np.deg2rad(geo.sensor_zenith_angle[m]))
    orders = []
    for l in (0, sc.n_channels // 3):
        planck = np.array([sc.planck_c1[l], sc.planck_c2[l], sc.band_c1[l], sc.band_c2[l]])
        nleg = n_streams or sx.sx_stream_rule(ct.c_double(re[:, :Ku].max()), ct.c_double(sc.wavenumber[l]))
        fr = sc.frequency[l] if mw else sc.wavenumber[l]
        e, bs, cbr = float(opt.emissivity[m, l]), 1.5 * planck[0], float(sc.cosmic_background_radiance[l])

        def fwd(od, temp, e=e, bs=bs, wc=wc, re=re):
            r = ct.c_double()
            assert sx.sx_cloudy_radiance(_p(dims, _ip), *[_p(a) for a in arrs], Ku, ctype.size, nleg, int(mw),
                                         ct.c_double(fr), ct.c_double(mu), ct.c_double(e), ct.c_double(bs),
                                         ct.c_double(cbr), _p(planck), _p(temp), _p(ctype, _ip), _p(wc), _p(re),
                                         atm.max_layers, _p(od), 1 if soi else 0, 0, *([None] * 14),
                                         ct.c_double(sc.wavenumber[l]), ct.byref(r)) == 0
            return r.value
        dg, dT = np.zeros(Ku), np.zeros(Ku)
        dwc, dre = np.zeros_like(wc), np.zeros_like(re)
        rad, eb, bb = ct.c_double(), ct.c_double(), ct.c_double()
        kargs = (_p(dims, _ip), *[_p(a) for a in arrs], Ku, ctype.size, nleg, int(mw), ct.c_double(fr),
                 ct.c_double(mu), ct.c_double(e), ct.c_double(bs), ct.c_double(cbr), _p(planck), _p(temp0),
                 _p(ctype, _ip), _p(wc), _p(re), atm.max_layers, _p(od0), ct.byref(rad))
        n_ord = ct.c_int(0)
        assert sx.sx_cloudy_kmatrix(*kargs, _p(dg), _p(dT), ct.byref(eb), ct.byref(bb), _p(dwc), _p(dre), 0,
                                    soi, ct.byref(n_ord)) == 0
        if soi:
            orders.append(n_ord.value)
            if soi < 75:   # checkpointed reverse: the same numbers as with every order kept
                d2 = [np.zeros(Ku), np.zeros(Ku), np.zeros_like(wc), np.zeros_like(re)]
                eb2, bb2 = ct.c_double(), ct.c_double()
                assert sx.sx_cloudy_kmatrix(*kargs, _p(d2[0]), _p(d2[1]), ct.byref(eb2), ct.byref(bb2),
                                            _p(d2[2]), _p(d2[3]), 0, 75, None) == 0
                for x, y in zip((dg, dT, dwc, dre, [eb.value, bb.value]), (*d2, [eb2.value, bb2.value])):
                    assert np.array_equal(x, y)
        else:
            # the contraction on double-float derivative numbers (the mixed form) agrees to 1e-6
            # of the largest Jacobian (eigenvector derivatives divide by eigenvalue gaps, which
            # double-float resolves to ~1e-15 instead of FP64's 1e-16)
            d2 = [np.zeros(Ku), np.zeros(Ku), np.zeros_like(wc), np.zeros_like(re)]
            eb2, bb2 = ct.c_double(), ct.c_double()
            assert sx.sx_cloudy_kmatrix(*kargs, _p(d2[0]), _p(d2[1]), ct.byref(eb2), ct.byref(bb2), _p(d2[2]),
                                        _p(d2[3]), 1, 0, None) == 0
            for x, y in zip((dg, dT, dwc * wc, dre * re), (d2[0], d2[1], d2[2] * wc, d2[3] * re)):
                assert np.abs(x - y).max() <= 1e-6 * max(np.abs(x).max(), 1e-30)
        assert abs(rad.value - fwd(od0, temp0)) <= 1e-13 * abs(rad.value)
        cloudy = np.where((wc[:, :Ku] > 1e-6).any(axis=0))[0]
        # SOI's doubling (up to ~30 doublings from a 1e-8 thin layer) leaves ~1e-10 relative
        # noise in the radiance, and the LUT interpolation bends over the larger steps that
        # noise asks for: the best of three steps, against a looser bound
        if soi:
            h_od, h_t, h_rel, tol = (1e-3, 3e-4, 1e-4), (3e-2, 1e-2, 3e-3), (1e-2, 3e-3, 1e-3), 2e-5
        else:
            h_od, h_t, h_rel, tol = (1e-7,), (1e-4,), (1e-4,), 1e-6

        def cd(fun, x, idx, hs, want, rel=False):
            best = None
            for h in hs:
                h = h * x[idx] if rel else h
                x1, x2 = x.copy(), x.copy()
                x1[idx] += h
                x2[idx] -= h
                d = (fun(x1) - fun(x2)) / (2 * h)
                best = d if best is None or abs(d - want) < abs(best - want) else best
            return best
        for k in list(cloudy[:5]) + [0, Ku - 1]:
            fd = cd(lambda o: fwd(o, temp0), od0, k, h_od, dg[k])
            assert abs(fd - dg[k]) <= tol * np.abs(dg).max(), (l, k, fd, dg[k])
            fd = cd(lambda t: fwd(od0, t), temp0, k, h_t, dT[k])
            assert abs(fd - dT[k]) <= tol * np.abs(dT).max(), (l, k, fd, dT[k])
            for c in range(ctype.size):
                if not wc[c, k] > 1e-6:
                    assert dwc[c, k] == 0.0 and dre[c, k] == 0.0
                    continue
                fd = cd(lambda w: fwd(od0, temp0, wc=w), wc, (c, k), h_rel, dwc[c, k], rel=True)
                assert abs(fd - dwc[c, k]) <= tol * np.abs(dwc * wc).max() / wc[c, k] + 1e-12, (l, k, c)
                fd = cd(lambda r: fwd(od0, temp0, re=r), re, (c, k), h_rel, dre[c, k], rel=True)
                assert abs(fd - dre[c, k]) <= tol * np.abs(dre * re).max() / re[c, k] + 1e-12, (l, k, c)
        he = 1e-3
        fd = cd(lambda x: fwd(od0, temp0, e=x[0]), np.array([e]), 0, (he, 3e-4) if soi else (he,), eb.value)
        assert abs(fd - eb.value) <= 1e-5 * abs(eb.value) + 1e-15 * abs(rad.value) / he
        # the radiance is linear in the surface Planck radiance: a large step is exact (SOI:
        # while the count of orders stays the same)
        fd = cd(lambda x: fwd(od0, temp0, bs=x[0]), np.array([bs]), 0, (0.1, 1e-2, 1e-3) if soi else (0.1,),
                bb.value, rel=True)
        assert abs(fd - bb.value) <= 1e-6 * abs(bb.value) + 1e-12
    print("SOI orders", orders)


@pytest.mark.parametrize("overlap", [1, 2, 3, 4, 5])
def test_total_cloud_cover_matches_overlap_schemes(sx, overlap):
    """total_cloud_cover (the GPU's per-profile cloud cover) against the
    overlap formulas of CRTM_CloudCover_Define.f90:522-638 restated in the
    oracle tests, on random fractions with tiny, zero and unit values mixed in."""
    from test_oracle_scatter import _tcc
    sx.sx_total_cloud_cover.restype = ct.c_double
    rng = np.random.Generator(np.random.PCG64(400 + overlap))
    for trial in range(200):
        K, NC = 60, 3
        wc = np.where(rng.uniform(size=(NC, K)) < 0.3, 10.0 ** rng.uniform(-7, -2, (NC, K)), 0.0)
        special = rng.choice([0.0, 1e-13, 1e-9, 1.0, -0.1], size=K)
        cf = np.where(rng.uniform(size=K) < (0.5 if trial % 2 else 0.05), special, rng.uniform(0.0, 1.0, K))
        wcz = np.where(cf[None, :] < 1e-12, 0.0, wc)
        lwc = np.where(wcz > 1e-6, wcz, 0.0).sum(axis=0)
        frac = ((np.where(cf < 1e-12, 0.0, cf) > 1e-6) & (lwc > 0)).any()
        got = sx.sx_total_cloud_cover(K, NC, _p(cf), _p(np.ascontiguousarray(wc)), K, overlap)
        if not frac:
            assert got == -1.0
        else:
            assert abs(got - _tcc(cf, lwc, overlap)) < 1e-14
    assert sx.sx_total_cloud_cover(3, 1, _p(np.ones(3)), _p(np.full(3, 1e-3)), 3, 7) == -2.0


@pytest.mark.parametrize("overlap", [1, 2, 3, 4, 5])
def test_cloud_cover_derivatives_match_differences(sx, overlap):
    """cloud_cover_derivatives against central differences of total_cloud_cover
    in each layer's cloud fraction and (average overlap) each cloud's water
    content."""
    sx.sx_total_cloud_cover.restype = ct.c_double
    rng = np.random.Generator(np.random.PCG64(500 + overlap))
    for trial in range(20):
        K, NC = 40, 2
        wc = np.where(rng.uniform(size=(NC, K)) < 0.4, 10.0 ** rng.uniform(-5, -2, (NC, K)), 0.0)
        cf = np.where((wc > 0).any(axis=0), rng.uniform(0.05, 0.95, K), 0.0)

        def tcc(cf_, wc_):
            return sx.sx_total_cloud_cover(K, NC, _p(np.ascontiguousarray(cf_)), _p(np.ascontiguousarray(wc_)),
                                           K, overlap)
        t0 = tcc(cf, wc)
        assert t0 >= 0.0
        dcf, dwc = np.zeros(K), np.zeros(K)
        sx.sx_cloud_cover_derivatives(K, NC, _p(cf), _p(wc), K, overlap, ct.c_double(t0), _p(dcf), _p(dwc))
        h = 1e-7
        for k in range(K):
            if cf[k] == 0.0:
                continue
            c1, c2 = cf.copy(), cf.copy()
            c1[k] += h
            c2[k] -= h
            fd = (tcc(c1, wc) - tcc(c2, wc)) / (2 * h)
            assert abs(fd - dcf[k]) < 1e-6, (k, fd, dcf[k])
            for c in range(NC):
                if wc[c, k] <= 1e-6:
                    continue
                hw = 1e-4 * wc[c, k]
                w1, w2 = wc.copy(), wc.copy()
                w1[c, k] += hw
                w2[c, k] -= hw
                fd = (tcc(cf, w1) - tcc(cf, w2)) / (2 * hw)
                assert abs(fd - dwc[k]) <= 1e-6 * (abs(fd) + 1.0), (k, c, fd, dwc[k])


def test_double_float_arithmetic(sx):
    """Double-float (two FP32 words) arithmetic against FP64: about 2^-46
    relative for products, quotients and roots; sums to 2^-46 of the larger
    operand (cancellation is exact).  Magnitudes 1e-12..1e12 (the layer
    solver's range): below ~1e-30 the low word leaves FP32's normal range."""
    sx.sx_dd_op.restype = ct.c_double
    rng = np.random.Generator(np.random.PCG64(700))
    a = rng.uniform(-1, 1, 2000) * 10.0 ** rng.uniform(-12, 12, 2000)
    b = rng.uniform(-1, 1, 2000) * 10.0 ** rng.uniform(-12, 12, 2000)
    tol = 2.0 ** -45
    for x, y in zip(a, b):
        s = sx.sx_dd_op(0, ct.c_double(x), ct.c_double(y))
        assert abs(s - (x + y)) <= tol * max(abs(x), abs(y))
        s = sx.sx_dd_op(1, ct.c_double(x), ct.c_double(x * (1 + 1e-9)))
        assert abs(s - (x - x * (1 + 1e-9))) <= tol * abs(x)
        assert abs(sx.sx_dd_op(2, ct.c_double(x), ct.c_double(y)) - x * y) <= tol * abs(x * y)
        assert abs(sx.sx_dd_op(3, ct.c_double(x), ct.c_double(y)) - x / y) <= tol * abs(x / y)
        assert abs(sx.sx_dd_op(4, ct.c_double(abs(x)), ct.c_double(0)) - np.sqrt(abs(x))) <= tol * np.sqrt(abs(x))
    for x in rng.uniform(-60, 60, 200):   # the input's rounding, amplified by |x|
        assert abs(sx.sx_dd_op(5, ct.c_double(x), ct.c_double(0)) - np.exp(x)) <= tol * max(abs(x), 1) * np.exp(x)


@pytest.mark.parametrize("nleg,mu_s", [(2, 0.9), (4, 0.55), (6, 0.8), (16, 0.93)])
@pytest.mark.parametrize("w,tau", [(0.6, 0.5), (0.98, 6.0), (0.999999, 40.0), (0.3, 5e-9), (0.05, 0.02)])
def test_ada_layer_in_double_float_matches_fp64(sx, nleg, mu_s, w, tau):
    """The mixed form's layer solver (MOM in double-float on the FP32 pipe)
    against the FP64 solver, including near-conservative thick layers where
    plain FP32 fails."""
    from oracle.pyoracle import lib
    pc = 0.5 * 0.85 ** np.arange(nleg + 1)
    mu, wt = np.zeros(20), np.zeros(20)
    ff, bb = np.zeros(400), np.zeros(400)
    nz = ct.c_int(0)
    lib().or_phase_setup(nleg, mu_s, _p(pc), _p(mu), _p(wt), _p(ff), _p(bb), ct.byref(nz))
    nZ, nS = nz.value, (nleg + 2) // 2
    outs = [[np.zeros(nZ * nZ), np.zeros(nZ * nZ), np.zeros(nZ)] for _ in range(2)]
    args = (nS, nZ, ct.c_double(w), ct.c_double(tau), _p(mu), _p(wt), _p(ff), _p(bb), ct.c_double(1.7))
    assert sx.sx_ada_layer(*args, *[_p(x) for x in outs[0]]) == 0
    assert sx.sx_ada_layer_dd(*args, *[_p(x) for x in outs[1]]) == 0
    # T and R are at most 1; the source (1 - sum T - sum R) B cancels for
    # near-conservative layers, so it is held to 1e-10 of B
    assert np.abs(outs[0][0] - outs[1][0]).max() <= 1e-11
    assert np.abs(outs[0][1] - outs[1][1]).max() <= 1e-11
    assert np.abs(outs[0][2] - outs[1][2]).max() <= 1e-10 * 1.7


def test_nearly_defective_eigenbasis_derivatives(sx, coeff_dir):
    """A layer whose MOM quadrature eigenvalue nearly meets the sensor angle's
    (relative gap ~2e-6; an aerosol-only IR layer under the 'GOCART-GEOS5'
    table): the eigenbasis is nearly defective and derivatives through it lose
    ~eps/gap^2, while the layer's T, R and source stay smooth.  The K-matrix
    contraction's evaluation (derivatives at sensor angles mu (1 +- 1e-3))
    matches central differences of the record with a 1e-2 relative step
    (smaller steps drown in the ~1e-10 rounding of the record's values there)
    to 2e-5 of the largest derivative, for each aerosol's concentration."""
    from oracle.pyoracle import Oracle
    scheme = "GOCART-GEOS5"
    sensor = "irsynth_c616"
    sy.write_cloud_files(coeff_dir)
    apath = sy.write_aerosol_files(coeff_dir, scheme)
    ac = co.read_aerosolcoeff(apath, scheme)
    sc = co.read_spccoeff(f"{coeff_dir}/{sensor}.SpcCoeff.bin")
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, 4, 101, 97)
    sy.add_clouds(atm, (co.WATER_CLOUD, co.ICE_CLOUD), 98, wc_scale=30.0)
    sy.add_aerosols(atm, sy.AEROSOL_TYPES, 99, load_scale=20.0)
    sy.add_aerosol_scheme_inputs(atm, 100)
    _, _, lod = Oracle(coeff_dir, sensor).forward(atm, sfc, geo, opt, layer_od=True)
    p, l, k = 1, 107, 80
    f = lambda a: np.ascontiguousarray(np.ravel(a, order="F"))   # noqa: E731
    adims = np.array([ac.wavelength.size, ac.ke.shape[1], ac.ke.shape[2], ac.ke.shape[3], ac.ke.shape[4],
                      ac.pcoeff.shape[5] - 1, co.AEROSOL_SCHEMES.index(scheme), ac.rh.size], np.int32)
    aarrs = [f(x) for x in (1.0e4 / ac.wavelength, ac.reff, ac.rsig, ac.rh, ac.ke, ac.w, ac.pcoeff[..., 0])]
    atypes = np.ascontiguousarray(ac.type_id, np.int32)
    planck = np.array([sc.planck_c1[l], sc.planck_c2[l], sc.band_c1[l], sc.band_c2[l]])
    mu = float(np.cos(np.deg2rad(geo.sensor_zenith_angle[p])))
    nleg = sx.sx_stream_rule(ct.c_double(atm.aerosol_effective_radius[p].max()), ct.c_double(sc.wavenumber[l]))
    at = np.ascontiguousarray(atm.aerosol_type[p], np.int32)
    reff = np.ascontiguousarray(atm.aerosol_effective_radius[p, :, k])
    var = np.ascontiguousarray(atm.aerosol_effective_variance[p, :, k])
    rh, gas, tk = float(atm.relative_humidity[p, k]), float(lod[p, l, k]), float(atm.temperature[p, k])

    def rec(conc, a):
        outs = [np.zeros(2 * 100 + 20) for _ in range(3)]
        nz, gap = ct.c_int(), ct.c_double()
        kind = sx.sx_aerosol_layer_record(_p(adims, _ip), _p(atypes, _ip), *[_p(x) for x in aarrs], 3, _p(at, _ip),
                                          _p(conc), _p(reff), _p(var), ct.c_double(rh), nleg, ct.c_double(mu),
                                          _p(planck), ct.c_double(sc.wavenumber[l]), ct.c_double(gas),
                                          ct.c_double(tk), a, *[_p(o) for o in outs], ct.byref(nz), ct.byref(gap))
        assert kind == 1
        ne = 1 + 2 * nz.value ** 2 + nz.value
        return gap.value, [o[:ne] for o in outs]
    conc0 = np.ascontiguousarray(atm.aerosol_concentration[p, :, k])
    gap, _ = rec(conc0, 0)
    assert gap < 1e-5   # the configuration is the nearly defective one
    for a in range(3):
        _, (v, dc, _) = rec(conc0, a)
        h = 1e-2 * conc0[a]
        c1, c2 = conc0.copy(), conc0.copy()
        c1[a] += h
        c2[a] -= h
        fd = (rec(c1, a)[1][0] - rec(c2, a)[1][0]) / (2 * h)
        assert np.abs(fd - dc).max() <= 2e-5 * np.abs(fd).max(), a


@pytest.mark.parametrize("classification", ["Nalli", "Nalli2"])
def test_irssem_matches_oracle(sx, tmp_path, classification):
    """The GPU header's IR sea-surface emissivity (CRTM_IRSSEM) against the
    oracle's on random angles, frequencies, wind speeds and temperatures,
    inside and outside the table's axes, and its wind-speed / temperature
    derivatives against central differences."""
    from oracle.pyoracle import lib
    path = sy.write_irwater_file(str(tmp_path), classification, "irw.bin")
    w = co.read_irwatercoeff(path)
    L = lib()
    h = L.or_irwater_init(path.encode())
    assert h
    f = lambda a: np.ascontiguousarray(np.ravel(a, order="F"))   # noqa: E731
    dims = np.array([w.angle.size, w.frequency.size, w.wind_speed.size, w.temperature.size], np.int32)
    arrs = [f(x) for x in (w.angle, w.frequency, w.wind_speed, w.temperature, w.emissivity)]
    sx.sx_irssem.restype = ct.c_double
    rng = np.random.Generator(np.random.PCG64(11))
    nalli2 = int(classification == "Nalli2")

    def gpu(t, v, fr, a):
        dv, dt = ct.c_double(), ct.c_double()
        e = sx.sx_irssem(_p(dims, _ip), nalli2, *[_p(x) for x in arrs], ct.c_double(t), ct.c_double(v),
                         ct.c_double(fr), ct.c_double(a), ct.byref(dv), ct.byref(dt))
        return e, dv.value, dt.value
    try:
        for _ in range(300):
            t, v = rng.uniform(265.0, 315.0), rng.uniform(-1.0, 18.0)
            fr, a = rng.uniform(550.0, 3100.0), rng.uniform(-80.0, 88.0)
            e, dv, dt = gpu(t, v, fr, a)
            assert abs(e - L.or_irssem(h, t, v, fr, a)) <= 1e-14
            hv = 1e-5
            fd = (gpu(t, v + hv, fr, a)[0] - gpu(t, v - hv, fr, a)[0]) / (2 * hv)
            assert abs(fd - dv) <= 1e-7, (v, fd, dv)
            fd = (gpu(t + hv, v, fr, a)[0] - gpu(t - hv, v, fr, a)[0]) / (2 * hv)
            assert abs(fd - dt) <= 1e-7
            if not nalli2:
                assert dt == 0.0
        # at the table's nodes the interpolation returns the table
        i, j, k = 3, 10, 5
        assert abs(gpu(w.temperature[0], w.wind_speed[k], w.frequency[j], w.angle[i])[0] -
                   w.emissivity[i, j, k, 0]) <= 1e-14
    finally:
        L.or_irwater_destroy(h)


def _lut_args(coeff_dir, scheme):
    """CloudCoeff and AerosolCoeff arguments of the harness entry points."""
    cc = co.read_cloudcoeff(sy.write_cloud_files(coeff_dir))
    f = lambda a: np.ascontiguousarray(np.ravel(a, order="F"))   # noqa: E731
    arrs = [f(x) for x in (cc.frequency_mw, cc.reff_mw, cc.temperature, cc.frequency_ir, cc.reff_ir,
                           cc.ke_l_mw, cc.w_l_mw, cc.pcoeff_l_mw, cc.ke_s_mw, cc.w_s_mw, cc.pcoeff_s_mw,
                           cc.ke_ir, cc.w_ir, cc.pcoeff_ir)]
    dims = np.array([cc.frequency_mw.size, cc.reff_mw.size, cc.temperature.size, cc.density_mw.size,
                     cc.frequency_ir.size, cc.reff_ir.size, cc.n_legendre_terms], np.int32)
    ac = co.read_aerosolcoeff(sy.write_aerosol_files(coeff_dir, scheme), scheme)
    adims = np.array([ac.wavelength.size, ac.ke.shape[1], ac.ke.shape[2], ac.ke.shape[3], ac.ke.shape[4],
                      ac.pcoeff.shape[5] - 1, co.AEROSOL_SCHEMES.index(scheme), ac.rh.size], np.int32)
    aarrs = [f(x) for x in (1.0e4 / ac.wavelength, ac.reff, ac.rsig, ac.rh, ac.ke, ac.w, ac.pcoeff[..., 0])]
    atypes = np.ascontiguousarray(ac.type_id, np.int32)
    return dims, arrs, adims, atypes, aarrs


@pytest.mark.parametrize("sensor,n_streams,aer,scheme", [("mwsynth_c16", None, False, "CRTM"),
                                                         ("mwsynth_c16", 16, False, "CRTM"),
                                                         ("irsynth_c616", None, True, "CRTM"),
                                                         ("irsynth_c616", 8, True, "CMAQ"),
                                                         ("irsynth_c616", 16, True, "GOCART-GEOS5")])
def test_layer_adjoint_matches_derivative_numbers(sx, coeff_dir, sensor, n_streams, aer, scheme):
    """The reverse sweep through a layer's optics (MOM, phase normalisation,
    combine, LUT) gives the same contraction of the record adjoints as the
    forward-mode derivative numbers, for every input of the layer: gas
    optical depth, temperature, and each cloud's and aerosol's amount and
    LUT coordinates.  Agreement to 1e-9 of each group's largest value
    (both are exact derivatives; the difference is rounding)."""
    dims, arrs, adims, atypes, aarrs = _lut_args(coeff_dir, scheme)
    sc = co.read_spccoeff(f"{coeff_dir}/{sensor}.SpcCoeff.bin")
    mw = sc.sensor_type == co.MICROWAVE_SENSOR
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 2, 100, 61, wc_scale=30.0, n_streams=n_streams,
                                            cloud_types=(co.WATER_CLOUD, co.ICE_CLOUD, co.RAIN_CLOUD)
                                            if mw else (co.WATER_CLOUD, co.ICE_CLOUD))
    NA = 0
    if aer:
        sy.add_aerosols(atm, sy.AEROSOL_TYPES, 62, load_scale=20.0)
        sy.add_aerosol_scheme_inputs(atm, 63)
        NA = 3
    rng = np.random.default_rng(64)
    n_checked = 0
    for m in range(2):
        Ku = int(atm.n_layers[m])
        temp = np.ascontiguousarray(atm.temperature[m, :Ku])
        wc = np.ascontiguousarray(atm.cloud_water_content[m])
        re = np.ascontiguousarray(atm.cloud_effective_radius[m])
        ctype = np.ascontiguousarray(atm.cloud_type[m], np.int32)
        if aer:
            conc = np.ascontiguousarray(atm.aerosol_concentration[m])
            areff = np.ascontiguousarray(atm.aerosol_effective_radius[m])
            avar = np.ascontiguousarray(atm.aerosol_effective_variance[m])
            rh = np.ascontiguousarray(atm.relative_humidity[m])
            at = np.ascontiguousarray(atm.aerosol_type[m], np.int32)
            aptr = [_p(at, _ip), _p(conc), _p(areff), _p(avar), _p(rh), _p(adims, _ip), _p(atypes, _ip),
                    *[_p(x) for x in aarrs]]
        else:
            aptr = [None] * 14
        mu = float(np.cos(np.deg2rad(geo.sensor_zenith_angle[m])))
        for l in (0, sc.n_channels // 2, sc.n_channels - 1):
            planck = np.array([sc.planck_c1[l], sc.planck_c2[l], sc.band_c1[l], sc.band_c2[l]])
            rmax = max(re[:, :Ku].max(), atm.aerosol_effective_radius[m].max() if aer else 0.0)
            nleg = n_streams or sx.sx_stream_rule(ct.c_double(rmax), ct.c_double(sc.wavenumber[l]))
            if aer and nleg == 2:
                continue
            fr = sc.frequency[l] if mw else sc.wavenumber[l]
            cloudy = np.where((wc[:, :Ku] > 1e-6).any(axis=0))[0]
            for k in list(cloudy[:4]) + [Ku - 1]:
                nz = 10
                tb, rb, sb = rng.normal(size=nz * nz), rng.normal(size=nz * nz), rng.normal(size=nz)
                ns = 2 + 3 * (ctype.size + NA)
                gr, gd = np.zeros(ns), np.zeros(ns)
                kd, nzo = ct.c_int(), ct.c_int()
                kind = sx.sx_layer_adjoint_compare(
                    _p(dims, _ip), *[_p(a) for a in arrs], Ku, ctype.size, nleg, int(mw), ct.c_double(fr),
                    ct.c_double(mu), _p(planck), _p(temp), _p(ctype, _ip), _p(wc), _p(re), atm.max_layers,
                    NA, *aptr, ct.c_double(sc.wavenumber[l]), int(k), ct.c_double(0.01 + 0.02 * (k % 3)),
                    _p(tb), _p(rb), _p(sb), ct.c_double(0.7), ct.c_double(-0.3), _p(gr), _p(gd),
                    ct.byref(kd), ct.byref(nzo))
                assert kind >= 0, kind
                assert kind == kd.value
                groups = [slice(0, 1), slice(1, 2)] + [slice(2 + q, ns, 3) for q in range(3)]
                for gsl in groups:
                    scale = max(np.abs(gd[gsl]).max(), 1e-300)
                    assert np.abs(gr[gsl] - gd[gsl]).max() <= 1e-9 * scale, (m, l, k, gsl, gr[gsl], gd[gsl])
                n_checked += kind
    assert n_checked > 5


@pytest.mark.parametrize("sensor,n_streams,wc_scale", [("irsynth_c616", None, 100.0), ("irsynth_c616", 16, 3.0),
                                                       ("mwsynth_c22", None, 3.0), ("mwsynth_c16", 8, 100.0)])
def test_mixed_column_kmatrix_matches_fp64(sx, coeff_dir, sensor, n_streams, wc_scale):
    """The column K-matrix as the mixed form computes it (FP32 layer solver
    in loss form, FP64 for layers near a nearly defective MOM eigenbasis;
    FP32 adding with the (I - Rup R)^-1 inversions in FP64; FP32 reverse
    sweep) against the FP64 form on the same column: brightness temperature
    within 0.01 K, every Jacobian within 1e-3 of its largest value, on all
    five cloud types and stream counts from the rule to 16."""
    cc = co.read_cloudcoeff(sy.write_cloud_files(coeff_dir))
    sc = co.read_spccoeff(f"{coeff_dir}/{sensor}.SpcCoeff.bin")
    f = lambda a: np.ascontiguousarray(np.ravel(a, order="F"))   # noqa: E731
    arrs = [f(x) for x in (cc.frequency_mw, cc.reff_mw, cc.temperature, cc.frequency_ir, cc.reff_ir,
                           cc.ke_l_mw, cc.w_l_mw, cc.pcoeff_l_mw, cc.ke_s_mw, cc.w_s_mw, cc.pcoeff_s_mw,
                           cc.ke_ir, cc.w_ir, cc.pcoeff_ir)]
    dims = np.array([cc.frequency_mw.size, cc.reff_mw.size, cc.temperature.size, cc.density_mw.size,
                     cc.frequency_ir.size, cc.reff_ir.size, cc.n_legendre_terms], np.int32)
    mw = sc.sensor_type == co.MICROWAVE_SENSOR
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, 3, 101, 61, wc_scale=wc_scale, n_streams=n_streams)
    rng = np.random.default_rng(3)
    n_cols = 0
    for m in range(3):
        Ku = int(atm.n_layers[m])
        temp = np.ascontiguousarray(atm.temperature[m, :Ku])
        wc = np.ascontiguousarray(atm.cloud_water_content[m])
        re = np.ascontiguousarray(atm.cloud_effective_radius[m])
        ctype = np.ascontiguousarray(atm.cloud_type[m], np.int32)
        od = np.ascontiguousarray(0.02 * (1.0 + rng.uniform(size=Ku)))
        mu = float(np.cos(np.deg2rad(geo.sensor_zenith_angle[m])))
        for l in np.linspace(0, sc.n_channels - 1, 12).astype(int):
            planck = np.array([sc.planck_c1[l], sc.planck_c2[l], sc.band_c1[l], sc.band_c2[l]])
            nleg = n_streams or sx.sx_stream_rule(ct.c_double(re[:, :Ku].max()), ct.c_double(sc.wavenumber[l]))
            fr = sc.frequency[l] if mw else sc.wavenumber[l]
            e, bs = float(opt.emissivity[m, l]), 1.2 * planck[0] / (np.exp(planck[1] / 290.0) - 1.0)
            outs = []
            for mixed in (0, 1):
                o = [ct.c_double(), np.zeros(Ku), np.zeros(Ku), ct.c_double(), ct.c_double(), np.zeros_like(wc),
                     np.zeros_like(re)]
                assert sx.sx_cloudy_kmatrix_form(
                    _p(dims, _ip), *[_p(a) for a in arrs], Ku, ctype.size, nleg, int(mw), ct.c_double(fr),
                    ct.c_double(mu), ct.c_double(e), ct.c_double(bs), ct.c_double(float(sc.cosmic_background_radiance[l])),
                    _p(planck), _p(temp), _p(ctype, _ip), _p(wc), _p(re), atm.max_layers, _p(od), ct.byref(o[0]),
                    _p(o[1]), _p(o[2]), ct.byref(o[3]), ct.byref(o[4]), _p(o[5]), _p(o[6]), mixed) == 0
                outs.append(o)
            (r0, g0, t0, e0, b0, w0, q0), (r1, g1, t1, e1, b1, w1, q1) = outs
            bt = lambda R: (planck[1] / np.log(planck[0] / R + 1.0) - planck[2]) / planck[3]   # noqa: E731
            assert abs(bt(r1.value) - bt(r0.value)) <= 0.01
            for a, b in ((g1, g0), (t1, t0), (w1 * wc, w0 * wc), (q1 * re, q0 * re)):
                assert np.abs(a - b).max() <= 1e-3 * max(np.abs(b).max(), 1e-30)
            assert abs(e1.value - e0.value) <= 1e-3 * abs(e0.value) and abs(b1.value - b0.value) <= 1e-3 * abs(b0.value)
            n_cols += 1
    assert n_cols == 36


@pytest.mark.parametrize("sensor", ["mwsynth_c16", "irsynth_c616"])
def test_channel_cloud_tables_match_direct_lookups(sx, coeff_dir, sensor):
    """The cloud lookups through the sensor's channel-interpolated tables (the
    frequency step done once per channel at init, as the GPU library does) and
    the axes' precomputed Lagrange reciprocals equal the direct lookups: every cloud type, radii and temperatures on and
    between the grid nodes and beyond both ends, every stream set's Legendre
    terms, values and radius / temperature derivatives."""
    cc = co.read_cloudcoeff(sy.write_cloud_files(coeff_dir))
    sc = co.read_spccoeff(f"{coeff_dir}/{sensor}.SpcCoeff.bin")
    f = lambda a: np.ascontiguousarray(np.ravel(a, order="F"))   # noqa: E731
    arrs = [f(x) for x in (cc.frequency_mw, cc.reff_mw, cc.temperature, cc.frequency_ir, cc.reff_ir,
                           cc.ke_l_mw, cc.w_l_mw, cc.pcoeff_l_mw, cc.ke_s_mw, cc.w_s_mw, cc.pcoeff_s_mw,
                           cc.ke_ir, cc.w_ir, cc.pcoeff_ir)]
    dims = np.array([cc.frequency_mw.size, cc.reff_mw.size, cc.temperature.size, cc.density_mw.size,
                     cc.frequency_ir.size, cc.reff_ir.size, cc.n_legendre_terms], np.int32)
    mw = sc.sensor_type == co.MICROWAVE_SENSOR
    freq = np.ascontiguousarray((sc.frequency if mw else sc.wavenumber)[::7] if not mw else sc.frequency)
    rax = cc.reff_mw if mw else cc.reff_ir
    re = np.ascontiguousarray(np.concatenate([[rax[0] * 0.5], rax[::4], 0.5 * (rax[1:] + rax[:-1])[::3],
                                              [rax[-1] * 2.0]]))
    tg = np.ascontiguousarray(np.concatenate([[cc.temperature[0] - 10.0], cc.temperature,
                                              0.5 * (cc.temperature[1:] + cc.temperature[:-1]),
                                              [cc.temperature[-1] + 10.0]]))
    sx.sx_cloud_chan_compare.restype = ct.c_double
    worst = sx.sx_cloud_chan_compare(_p(dims, _ip), *[_p(a) for a in arrs], int(mw), freq.size, _p(freq),
                                     re.size, _p(re), tg.size, _p(tg))
    assert worst == 0.0

