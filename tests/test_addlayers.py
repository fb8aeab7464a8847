"""CRTM_Atmosphere_AddLayers (host code, crtmv3_gb300/addlayers.py) against the
oracle's C restatement, its layout and error rules, and the reference-named
entry points wired through it (a stand-in handle that computes with the
oracle, so that the wiring runs without a GPU).

Tolerances: the added layers agree with the oracle to 1e-12 relative; the
mapped K-matrix equals the oracle's K-matrix of the extended profiles at the
user's layers exactly; central differences of the forward model through
CRTM_Forward match the K-matrix to 1e-5 of the largest Jacobian.
"""
import dataclasses

import numpy as np
import pytest

from crtmv3_gb300 import addlayers as al, api, synthetic as sy
from crtmv3_gb300.structures import KMatrixBatch, RTSolutionBatch

SENSOR = "irsynth_c616"


def _cut(atm, cut):
    """The batch without its top `cut` layers: tops below 0.005 hPa."""
    cut = np.broadcast_to(np.asarray(cut), (atm.n_profiles,))
    K = atm.max_layers - int(cut.min())
    lp = np.zeros((atm.n_profiles, K + 1))
    pr, tt = np.zeros((atm.n_profiles, K)), np.zeros((atm.n_profiles, K))
    ab = np.zeros((atm.n_profiles, atm.n_absorbers, K))
    nl = np.zeros(atm.n_profiles, np.int32)
    for p in range(atm.n_profiles):
        c = int(cut[p])
        m = int(atm.n_layers[p]) - c
        nl[p] = m
        lp[p, :m + 1] = atm.level_pressure[p, c:c + m + 1]
        lp[p, m + 1:] = lp[p, m]
        pr[p, :m] = atm.pressure[p, c:c + m]
        tt[p, :m] = atm.temperature[p, c:c + m]
        ab[p, :, :m] = atm.absorber[p, :, c:c + m]
        pr[p, m:], tt[p, m:] = pr[p, m - 1], tt[p, m - 1]
        ab[p, :, m:] = ab[p, :, m - 1:m]
    return dataclasses.replace(atm, n_layers=nl, level_pressure=lp, pressure=pr, temperature=tt, absorber=ab)


def _workload(P=6, cut=(3, 10, 1, 25, 40, 7), seed=31):
    atm, sfc, geo, opt = sy.clear_sky_workload(SENSOR, P, 101, seed)
    return _cut(atm, cut[:P]), sfc, geo, opt


def test_model_table():
    p, t, a = al.model_profiles()
    assert p.shape == (101,) and t.shape == (6, 101) and a.shape == (6, 6, 101)
    assert p[0] == 0.005 and p[63] == 300.0 and p[100] == 1100.0
    assert (np.diff(p) > 0).all()
    assert (t > 150).all() and (t < 320).all()
    assert (a > 0).all()


def test_no_layers_at_the_top_of_the_atmosphere():
    atm, *_ = sy.clear_sky_workload(SENSOR, 3, 101, 4)
    assert (atm.level_pressure[:, 0] <= al.TOA_PRESSURE).all()
    ext, info = al.add_layers(atm)
    assert ext is atm and not info.any
    # Add_Extra_Layers off: profiles are used as given whatever their top
    cut = _cut(atm, 12)
    cut.add_extra_layers = np.zeros(3, bool)
    ext, info = al.add_layers(cut)
    assert ext is cut and not info.any


def test_layer_count_follows_the_model_grid():
    p = al.model_profiles()[0]
    for top in (0.0051, 0.016065, 0.0161, 0.3, 1.0, 299.9, 300.0, 1099.0):
        n = al.extra_layers(top)
        assert p[n - 1] < top <= p[n], (top, n)
    assert al.extra_layers(1100.5) == 0


@pytest.mark.parametrize("climatology", [None, 1, 2, 3, 4, 5, 6, 0, 9])
def test_added_layers_match_the_oracle(climatology):
    from oracle.pyoracle import add_layers_profile
    atm, *_ = _workload()
    if climatology is not None:
        atm.climatology = np.full(atm.n_profiles, climatology)
    ext, info = al.add_layers(atm)
    mp, mt, ma = al.model_profiles()
    model = 6 if climatology is None or not 1 <= climatology <= 6 else climatology
    rows = [{1: 0, 2: 2, 3: 1, 4: 3, 5: 4, 6: 5}[int(j)] for j in atm.absorber_id]
    for p in range(atm.n_profiles):
        pl, lp, t, a = add_layers_profile(mp, mt[model - 1], ma[model - 1][rows], atm.level_pressure[p, 0],
                                          atm.pressure[p], atm.temperature[p], atm.absorber[p])
        n = int(info.n_added[p])
        assert n == lp.shape[0] > 0
        np.testing.assert_allclose(ext.level_pressure[p, :n + 1], pl, rtol=1e-12, atol=0)
        np.testing.assert_allclose(ext.pressure[p, :n], lp, rtol=1e-12, atol=0)
        np.testing.assert_allclose(ext.temperature[p, :n], t, rtol=1e-12, atol=0)
        np.testing.assert_allclose(ext.absorber[p, :, :n], a, rtol=1e-12, atol=0)


def test_extended_layout():
    atm, *_ = _workload()
    atm.cloud_fraction = np.full((atm.n_profiles, atm.max_layers), 0.5)
    ext, info = al.add_layers(atm)
    assert (ext.n_layers == atm.n_layers + info.n_added).all()
    assert ext.max_layers == int(ext.n_layers.max())
    for p in range(atm.n_profiles):
        n, m = int(info.n_added[p]), int(atm.n_layers[p])
        assert ext.level_pressure[p, 0] == al.TOA_PRESSURE
        np.testing.assert_array_equal(ext.level_pressure[p, n:n + m + 1], atm.level_pressure[p, :m + 1])
        np.testing.assert_array_equal(ext.pressure[p, n:n + m], atm.pressure[p, :m])
        np.testing.assert_array_equal(ext.temperature[p, n:n + m], atm.temperature[p, :m])
        np.testing.assert_array_equal(ext.absorber[p, :, n:n + m], atm.absorber[p, :, :m])
        assert (np.diff(ext.level_pressure[p, :n + m + 1]) > 0).all()
        # layer pressures lie inside their levels
        assert (ext.pressure[p, :n] > ext.level_pressure[p, :n]).all()
        assert (ext.pressure[p, :n] < ext.level_pressure[p, 1:n + 1]).all()
        assert (ext.cloud_fraction[p, :n] == 0).all() and (ext.cloud_fraction[p, n:n + m] == 0.5).all()
        # the round trip of a layer field
        np.testing.assert_array_equal(al.user_layers(info, ext.temperature)[p, :m], atm.temperature[p, :m])


def test_shift_joins_the_user_profile():
    """The lowest added layer sits on the user's top two layers, extrapolated
    linearly in ln p (Shift_Profile)."""
    atm, *_ = _workload()
    ext, info = al.add_layers(atm)
    for p in range(atm.n_profiles):
        n = int(info.n_added[p])
        x = np.log(ext.pressure[p, n - 1])
        x1, x2 = np.log(atm.pressure[p, :2])
        e = (x - x1) / (x2 - x1)
        t = atm.temperature[p, 0] + (atm.temperature[p, 1] - atm.temperature[p, 0]) * e
        assert abs(ext.temperature[p, n - 1] - t) < 1e-9
        a = atm.absorber[p, :, 0] + (atm.absorber[p, :, 1] - atm.absorber[p, :, 0]) * e
        ok = a > 0
        np.testing.assert_allclose(ext.absorber[p, ok, n - 1], a[ok], rtol=1e-12)
        assert (ext.absorber[p, ~ok, :n] >= 0).all()


def test_negative_amounts_are_clamped():
    atm, *_ = _workload(P=1, cut=(10,))
    atm.absorber[0, 0, 1] = atm.absorber[0, 0, 0] * 50   # steep water vapour: the extrapolation goes negative
    ext, info = al.add_layers(atm)
    n = int(info.n_added[0])
    assert (ext.absorber[0, 0, :n] == al.MINIMUM_ABSORBER_AMOUNT).any()
    assert (ext.absorber[0, :, :n] > 0).all()


def test_errors_fail_the_call():
    atm, sfc, geo, opt = _workload(P=2, cut=(5, 5))
    bad = dataclasses.replace(atm, absorber_id=np.array([1, 3, 2, 4, 5, 7]))
    with pytest.raises(ValueError, match="id 7"):
        al.add_layers(bad)
    one = dataclasses.replace(atm, n_layers=np.array([1, 90], np.int32))
    with pytest.raises(ValueError, match="at least 2 layers"):
        al.add_layers(one)
    low = dataclasses.replace(atm, level_pressure=atm.level_pressure + 1200.0)
    with pytest.raises(ValueError, match="below the model profiles"):
        al.add_layers(low)
    # the reference-named entry points report FAILURE before any device work
    assert api.CRTM_Forward(bad, sfc, geo, [], []) == api.FAILURE
    assert api.CRTM_K_Matrix(bad, sfc, None, geo, [], [], []) == api.FAILURE
    assert api.CRTM_Adjoint(bad, sfc, [], geo, [], {}, []) == api.FAILURE


class OracleHandle:
    """Stands in for api.CRTM in the reference-named entry points: the same
    host calls, computed by the oracle."""

    def __init__(self, coeff_dir):
        from oracle.pyoracle import Oracle
        self.o = Oracle(coeff_dir, SENSOR)
        self.seen = []

    def forward(self, atm, sfc, geo, opt, sensor=0, components=False):
        self.seen.append(atm)
        if not components:
            rad, bt = self.o.forward(atm, sfc, geo, opt)
            return RTSolutionBatch(rad, bt, status=np.zeros(atm.n_profiles, np.int32))
        x = self.o.forward_components(atm, sfc, geo, opt)
        r = RTSolutionBatch(x.pop("radiance"), x.pop("bt"), status=np.zeros(atm.n_profiles, np.int32))
        for f, v in x.items():
            setattr(r, f, v)
        return r

    def k_matrix(self, atm, sfc, geo, opt, bt_k=None, sensor=0, components=False):
        self.seen.append(atm)
        r = self.o.k_matrix(atm, sfc, geo, opt, bt_k)
        km = KMatrixBatch(r["temperature_k"], r["absorber_k"], r["water_temperature_k"], r["surface_emissivity_k"])
        return km, RTSolutionBatch(r["radiance"], r["bt"], status=np.zeros(atm.n_profiles, np.int32))

    def tangent_linear(self, atm, sfc, geo, opt, atm_tl=None, sfc_tl=None, sensor=0, components=False):
        self.seen.append((atm, atm_tl))
        P, K = atm.n_profiles, atm.max_layers
        t_tl = np.ascontiguousarray(getattr(atm_tl, "temperature", None) if atm_tl is not None else None)
        t_tl = np.zeros((P, K)) if t_tl.ndim == 0 else t_tl
        a_tl = getattr(atm_tl, "absorber", None) if atm_tl is not None else None
        a_tl = np.zeros((P, atm.n_absorbers, K)) if a_tl is None else np.ascontiguousarray(a_tl)
        bt_tl = self.o.tangent_fd(atm, sfc, geo, opt, t_tl, a_tl, np.zeros(P), step=1e-4)
        rad, bt = self.o.forward(atm, sfc, geo, opt)
        return bt_tl, RTSolutionBatch(rad, bt, status=np.zeros(P, np.int32))

    def adjoint(self, atm, sfc, geo, opt, bt_ad, sensor=0, components=False):
        self.seen.append(atm)
        r = self.o.adjoint(atm, sfc, geo, opt, bt_ad)
        out = dict(temperature=r["temperature_ad"], absorber=r["absorber_ad"],
                   water_temperature=r["water_temperature_ad"])
        return out, RTSolutionBatch(r["radiance"], r["bt"], status=np.zeros(atm.n_profiles, np.int32))


def test_entry_points_run_on_the_extended_profiles(coeff_dir):
    atm, sfc, geo, opt = _workload(P=3, cut=(4, 12, 30))
    h = OracleHandle(coeff_dir)
    L = h.o.n_channels
    ci = [api.ChannelInfo(SENSOR, 0, L, h)]
    ext, info = al.add_layers(atm)

    rts = []
    assert api.CRTM_Forward(atm, sfc, geo, ci, rts, opt) == api.SUCCESS
    assert h.seen[-1].max_layers == ext.max_layers
    np.testing.assert_array_equal(rts[0].brightness_temperature, h.o.forward(ext, sfc, geo, opt)[1])
    # the layer components come back on the user's layers
    lod = h.o.forward(ext, sfc, geo, opt, layer_od=True)[2]
    assert rts[0].layer_optical_depth.shape == (3, L, atm.max_layers)
    for p in range(3):
        n, m = int(info.n_added[p]), int(atm.n_layers[p])
        np.testing.assert_array_equal(rts[0].layer_optical_depth[p, :, :m], lod[p, :, n:n + m])
        assert not rts[0].layer_optical_depth[p, :, m:].any()

    seed = np.random.default_rng(2).uniform(0.5, 1.5, (3, L))
    ks, rts = [], []
    assert api.CRTM_K_Matrix(atm, sfc, [seed], geo, ci, ks, rts, opt) == api.SUCCESS
    km = ks[0]
    assert km.temperature.shape == (3, L, atm.max_layers)
    assert km.absorber.shape == (3, L, atm.n_absorbers, atm.max_layers)
    ref = h.o.k_matrix(ext, sfc, geo, opt, seed)
    for p in range(3):
        n, m = int(info.n_added[p]), int(atm.n_layers[p])
        np.testing.assert_array_equal(km.temperature[p, :, :m], ref["temperature_k"][p, :, n:n + m])
        np.testing.assert_array_equal(km.absorber[p, :, :, :m], ref["absorber_k"][p, :, :, n:n + m])
        assert (km.temperature[p, :, m:] == 0).all()
    np.testing.assert_array_equal(km.water_temperature, ref["water_temperature_k"])

    ad, rts = {}, []
    assert api.CRTM_Adjoint(atm, sfc, [seed], geo, ci, ad, rts, opt) == api.SUCCESS
    assert ad["temperature"].shape == (3, atm.max_layers)
    np.testing.assert_allclose(ad["temperature"], km.temperature.sum(axis=1), rtol=1e-10,
                               atol=1e-12 * np.abs(km.temperature).max())


def test_k_matrix_matches_differences_below_the_top_two_layers(coeff_dir):
    """Below the user's top two layers (which enter the shift of the added
    layers, a dependence the reference does not differentiate) the mapped
    K-matrix is the derivative of CRTM_Forward."""
    atm, sfc, geo, opt = _workload(P=2, cut=(6, 20))
    h = OracleHandle(coeff_dir)
    L = h.o.n_channels
    ci = [api.ChannelInfo(SENSOR, 0, L, h)]
    ks, rts = [], []
    assert api.CRTM_K_Matrix(atm, sfc, None, geo, ci, ks, rts, opt) == api.SUCCESS
    kt = ks[0].temperature
    scale = np.abs(kt).max()
    step = 0.01
    for k in (2, 5, 40):
        bts = []
        for sgn in (1, -1):
            a = dataclasses.replace(atm, temperature=atm.temperature.copy())
            a.temperature[:, k] += sgn * step
            r = []
            assert api.CRTM_Forward(a, sfc, geo, ci, r, opt) == api.SUCCESS
            bts.append(r[0].brightness_temperature)
        fd = (bts[0] - bts[1]) / (2 * step)
        assert np.abs(fd - kt[:, :, k]).max() < 1e-5 * scale, k


def test_tangent_linear_gives_the_added_layers_no_perturbation(coeff_dir):
    import types
    atm, sfc, geo, opt = _workload(P=2, cut=(8, 15))
    h = OracleHandle(coeff_dir)
    L = h.o.n_channels
    ci = [api.ChannelInfo(SENSOR, 0, L, h)]
    ext, info = al.add_layers(atm)
    dT = np.random.default_rng(4).normal(0, 0.5, (2, atm.max_layers))
    for p in range(2):
        dT[p, atm.n_layers[p]:] = 0.0
    rts, tl = [], []
    assert api.CRTM_Tangent_Linear(atm, sfc, types.SimpleNamespace(temperature=dT), None, geo, ci, rts, tl,
                                   opt) == api.SUCCESS
    seen_atm, seen_tl = h.seen[-1]
    assert seen_atm.max_layers == ext.max_layers
    for p in range(2):
        n, m = int(info.n_added[p]), int(atm.n_layers[p])
        assert (seen_tl.temperature[p, :n] == 0).all()
        np.testing.assert_array_equal(seen_tl.temperature[p, n:n + m], dT[p, :m])
    ks, r2 = [], []
    assert api.CRTM_K_Matrix(atm, sfc, None, geo, ci, ks, r2, opt) == api.SUCCESS
    lin = np.einsum("plk,pk->pl", ks[0].temperature, dT)
    assert np.abs(tl[0] - lin).max() < 1e-5 * np.abs(lin).max()


def test_k_matrix_and_adjoint_accumulate_into_given_structures(coeff_dir):
    """CRTM_K_Matrix / CRTM_Adjoint add into the structures the caller passes
    (the reference's INTENT(IN OUT) Atmosphere_K and Atmosphere_AD), and fill
    an empty list / dict."""
    atm, sfc, geo, opt = _workload(P=2, cut=(5, 9))
    h = OracleHandle(coeff_dir)
    L = h.o.n_channels
    ci = [api.ChannelInfo(SENSOR, 0, L, h)]
    ks, rts = [], []
    assert api.CRTM_K_Matrix(atm, sfc, None, geo, ci, ks, rts, opt) == api.SUCCESS
    once = ks[0].temperature.copy()
    assert api.CRTM_K_Matrix(atm, sfc, None, geo, ci, ks, rts, opt) == api.SUCCESS
    np.testing.assert_allclose(ks[0].temperature, 2 * once, rtol=1e-15)
    zero = [dataclasses.replace(ks[0], **{f: np.zeros_like(getattr(ks[0], f)) for f in
                                          ("temperature", "absorber", "water_temperature", "surface_emissivity")})]
    assert api.CRTM_K_Matrix(atm, sfc, None, geo, ci, zero, rts, opt) == api.SUCCESS
    np.testing.assert_array_equal(zero[0].temperature, once)
    assert api.CRTM_K_Matrix(atm, sfc, None, geo, ci, [ks[0], ks[0]], rts, opt) == api.FAILURE
    seed = np.ones((2, L))
    ad, rts = {}, []
    assert api.CRTM_Adjoint(atm, sfc, [seed], geo, ci, ad, rts, opt) == api.SUCCESS
    first = ad["temperature"].copy()
    assert api.CRTM_Adjoint(atm, sfc, [seed], geo, ci, ad, rts, opt) == api.SUCCESS
    np.testing.assert_allclose(ad["temperature"], 2 * first, rtol=1e-15)


def test_channel_info_subset_host_logic(coeff_dir):
    """CRTM_ChannelInfo_Subset's checks and bookkeeping (the handle records
    the processed file positions): a subset in any order, too many channels,
    numbers out of range (which turn every channel off), reset."""
    class Handle:
        def __init__(self):
            self.calls = []

        def set_channel_subset(self, sensor, positions):
            self.calls.append(None if positions is None else list(positions))

    h = Handle()
    chans = np.array([3, 5, 9, 12, 40], np.int32)
    ci = api.ChannelInfo("s", 0, 5, h, chans, np.ones(5, bool))
    assert api.CRTM_ChannelInfo_Subset(ci, [40, 5]) == api.SUCCESS
    assert h.calls[-1] == [1, 4] and api.CRTM_ChannelInfo_n_Channels(ci) == 2
    assert list(api.CRTM_ChannelInfo_Channels(ci)) == [5, 40]
    assert api.CRTM_ChannelInfo_Subset(ci, list(range(6))) == api.FAILURE
    assert api.CRTM_ChannelInfo_n_Channels(ci) == 0 and h.calls[-1] == []
    assert api.CRTM_ChannelInfo_Subset(ci, [2]) == api.FAILURE
    assert api.CRTM_ChannelInfo_n_Channels(ci) == 0
    assert api.CRTM_ChannelInfo_Subset(ci, [9], reset=True) == api.SUCCESS
    assert api.CRTM_ChannelInfo_n_Channels(ci) == 5 and h.calls[-1] is None
    assert api.CRTM_ChannelInfo_Subset(ci, []) == api.SUCCESS
    assert api.CRTM_ChannelInfo_n_Channels(ci) == 0
