"""Profiles whose top lies below 0.005 hPa through the reference-named entry
points on the GPU: CRTM_Forward / CRTM_K_Matrix add the climatology layers
(CRTM_Atmosphere_AddLayers, host code) and run the library on the extended
profiles.  Checked against the oracle on the same extended profiles, with the
K-matrix mapped back to the user's layers.

Tolerances as the other parity tests: FP64 form 1e-4 K and 1e-6 relative to
the largest Jacobian; mixed form 0.01 K and 1e-3.
"""
import dataclasses

import numpy as np
import pytest

from crtmv3_gb300 import addlayers as al, synthetic as sy

pytestmark = pytest.mark.gpu

BT_TOL = {0: 1e-4, 1: 1e-2}
JAC_TOL = {0: 1e-6, 1: 1e-3}


def _cut_top(atm, cut):
    """The batch without its top cut[p] layers (tops below 0.005 hPa)."""
    P = atm.n_profiles
    K = atm.max_layers - int(min(cut))
    lp, pr, tt = np.zeros((P, K + 1)), np.zeros((P, K)), np.zeros((P, K))
    ab = np.zeros((P, atm.n_absorbers, K))
    nl = np.zeros(P, np.int32)
    for p in range(P):
        c, m = int(cut[p]), int(atm.n_layers[p]) - int(cut[p])
        nl[p] = m
        lp[p, :m + 1] = atm.level_pressure[p, c:c + m + 1]
        lp[p, m + 1:] = lp[p, m]
        pr[p, :m], tt[p, :m] = atm.pressure[p, c:c + m], atm.temperature[p, c:c + m]
        pr[p, m:], tt[p, m:] = pr[p, m - 1], tt[p, m - 1]
        ab[p, :, :m] = atm.absorber[p, :, c:c + m]
        ab[p, :, m:] = ab[p, :, m - 1:m]
    return dataclasses.replace(atm, n_layers=nl, level_pressure=lp, pressure=pr, temperature=tt, absorber=ab)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("sensor,nl", [("irsynth_c616", 101), ("mwsynth_c22", 100)])
def test_cut_top_profiles_match_the_oracle(gpu_lib, coeff_dir, sensor, nl, precision):
    from oracle.pyoracle import Oracle
    api = gpu_lib
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, 4, nl, 515)
    atm = _cut_top(atm, (3, 9, 17, 30))
    ext, info = al.add_layers(atm)
    assert (info.n_added > 0).all()
    ci = []
    assert api.CRTM_Init([sensor], ci, coeff_dir, precision) == api.SUCCESS
    L = ci[0].n_channels
    seed = np.random.default_rng(6).uniform(0.5, 1.5, (4, L))
    ks, rts = [], []
    assert api.CRTM_K_Matrix(atm, sfc, [seed], geo, ci, ks, rts, opt) == api.SUCCESS
    fw = []
    assert api.CRTM_Forward(atm, sfc, geo, ci, fw, opt) == api.SUCCESS
    ref = Oracle(coeff_dir, sensor).k_matrix(ext, sfc, geo, opt, seed)
    assert np.abs(rts[0].brightness_temperature - ref["bt"]).max() < BT_TOL[precision]
    assert np.abs(fw[0].brightness_temperature - ref["bt"]).max() < BT_TOL[precision]
    km = ks[0]
    assert km.temperature.shape == (4, L, atm.max_layers)
    tk = al.user_layers(info, ref["temperature_k"])
    ak = al.user_layers(info, ref["absorber_k"])
    scale = np.abs(tk).max()
    assert np.abs(km.temperature - tk).max() < JAC_TOL[precision] * scale
    for j in range(atm.n_absorbers):
        s = max(np.abs(ak[:, :, j]).max(), 1e-300)
        assert np.abs(km.absorber[:, :, j] - ak[:, :, j]).max() < JAC_TOL[precision] * 10 * s
    s = np.abs(ref["water_temperature_k"]).max()
    assert np.abs(km.water_temperature - ref["water_temperature_k"]).max() < JAC_TOL[precision] * s
    api.CRTM_Destroy(ci)
