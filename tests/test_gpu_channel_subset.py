"""Channel subsets (CRTM_ChannelInfo_Subset) on the GPU: a subset's outputs
are the full call's outputs at those channels, bit for bit (channels are
independent on this path), for clear-sky and cloudy batches, the forward,
K-matrix and adjoint; the reference-named entry points follow a ChannelInfo
subset and its reset."""
import numpy as np
import pytest

from crtmv3_gb300 import api, synthetic as sy

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cloud_dir(coeff_dir):
    sy.write_cloud_files(coeff_dir)
    return coeff_dir


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("sensor,cloudy", [("irsynth_c616", False), ("irsynth_c616", True), ("mwsynth_c22", True)])
def test_subset_outputs_are_the_full_outputs_at_those_channels(gpu_lib, cloud_dir, sensor, cloudy, precision):
    if cloudy:
        atm, sfc, geo, opt = sy.cloudy_workload(sensor, 4, 90, 91, wc_scale=30.0)
        atm.n_clouds[1] = 0
    else:
        atm, sfc, geo, opt = sy.clear_sky_workload(sensor, 4, 90, 91)
    h = gpu_lib.CRTM([sensor], cloud_dir, precision)
    L = h.n_channels[0]
    full_f = h.forward(atm, sfc, geo, opt, components=True)
    full_k, full_r = h.k_matrix(atm, sfc, geo, opt)
    seed = np.random.default_rng(3).uniform(0.5, 1.5, (4, L))
    pos = np.array(sorted(np.random.default_rng(4).choice(L, size=min(37, L - 3), replace=False)), np.int32)
    h.set_channel_subset(0, pos[::-1])   # any order: processed in file order
    assert h.n_channels[0] == pos.size and np.array_equal(h.channel_subset(0), pos)
    o2 = dict(vars(opt))
    o2["emissivity"] = opt.emissivity[:, pos]
    opt_s = type(opt)(**o2)
    sub_f = h.forward(atm, sfc, geo, opt_s, components=True)
    for f in ("radiance", "brightness_temperature", "tb_clear", "layer_optical_depth", "upwelling_radiance",
              "n_full_streams"):
        assert np.array_equal(getattr(sub_f, f), getattr(full_f, f)[:, pos]), f
    # SOD is accumulated over the layers with atomic additions: equal to rounding
    assert np.allclose(sub_f.sod, full_f.sod[:, pos], rtol=1e-13, atol=0)
    sub_k, sub_r = h.k_matrix(atm, sfc, geo, opt_s)
    for f in ("temperature", "absorber", "water_temperature", "surface_emissivity", "cloud_water_content"):
        a, b = getattr(sub_k, f, None), getattr(full_k, f, None)
        if a is None and b is None:
            continue
        assert np.array_equal(a, b[:, pos]), f
    ad_s, _ = h.adjoint(atm, sfc, geo, opt_s, seed[:, pos])
    h.set_channel_subset(0, None)
    assert h.n_channels[0] == L
    seed_full = np.zeros((4, L))
    seed_full[:, pos] = seed[:, pos]
    ad_f, _ = h.adjoint(atm, sfc, geo, opt, seed_full)
    assert np.abs(ad_s["temperature"] - ad_f["temperature"]).max() <= 1e-12 * np.abs(ad_f["temperature"]).max()
    # no channels: calls succeed and compute nothing
    h.set_channel_subset(0, [])
    assert h.n_channels[0] == 0
    o3 = dict(vars(opt))
    o3["emissivity"] = opt.emissivity[:, :0]
    r0 = h.forward(atm, sfc, geo, type(opt)(**o3))
    assert r0.radiance.shape == (4, 0)
    with pytest.raises(RuntimeError):
        h.set_channel_subset(0, [0, 0])
    with pytest.raises(RuntimeError):
        h.set_channel_subset(0, [L])


def test_reference_named_subset(gpu_lib, cloud_dir):
    sensor = "mwsynth_c22"
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, 3, 90, 93)
    ci: list = []
    assert api.CRTM_Init([sensor], ci, cloud_dir) == api.SUCCESS
    full: list = []
    assert api.CRTM_Forward(atm, sfc, geo, ci, full, opt) == api.SUCCESS
    chans = ci[0].sensor_channel
    pick = [chans[20], chans[3], chans[7]]
    assert api.CRTM_ChannelInfo_Subset(ci[0], pick) == api.SUCCESS
    assert api.CRTM_ChannelInfo_n_Channels(ci[0]) == 3
    assert list(api.CRTM_ChannelInfo_Channels(ci[0])) == [chans[3], chans[7], chans[20]]
    o2 = dict(vars(opt))
    o2["emissivity"] = opt.emissivity[:, [3, 7, 20]]
    sub: list = []
    assert api.CRTM_Forward(atm, sfc, geo, ci, sub, type(opt)(**o2)) == api.SUCCESS
    assert np.array_equal(sub[0].brightness_temperature, full[0].brightness_temperature[:, [3, 7, 20]])
    ks, rts = [], []
    assert api.CRTM_K_Matrix(atm, sfc, None, geo, ci, ks, rts, type(opt)(**o2)) == api.SUCCESS
    assert ks[0].temperature.shape[1] == 3
    assert api.CRTM_ChannelInfo_Subset(ci[0], [chans.max() + 1]) == api.FAILURE
    assert api.CRTM_ChannelInfo_n_Channels(ci[0]) == 0
    assert api.CRTM_ChannelInfo_Subset(ci[0], reset=True) == api.SUCCESS
    assert api.CRTM_ChannelInfo_n_Channels(ci[0]) == chans.size
    api.CRTM_Destroy(ci)
