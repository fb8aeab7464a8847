"""The further RTSolution components (Tb_clear, R_clear, Total_Cloud_Cover,
SOD, Surface_Emissivity, Up/Down_Radiance, Surface_Planck_Radiance,
n_Full_Streams, Layer_Optical_Depth, Upwelling_Radiance,
Upwelling_Overcast_Radiance) on the GPU against the oracle's CRTM_Forward
restatement, for clear-sky batches, and for batches mixing clear, cloudy,
fractionally cloudy, aerosol-only, n_Streams 8/16 and SOI profiles (the
bucketed pipelines).

The forward fills R_clear / Tb_clear for fractional profiles and for
profiles without clouds (CRTM_Forward_Module.f90:1108-1119); the K-matrix,
adjoint and tangent linear for fractional profiles only
(CRTM_K_Matrix_Module.f90:1328-1336).

Tolerances: FP64 form 1e-9 relative in radiances and optical depths, 1e-4 K
in brightness temperatures (the SOI solver's own rounding floor is near
1e-6 K); mixed form 1e-4 relative and 0.01 K (the layer optical depths and
radiances of FP32 gas optics)."""
import numpy as np
import pytest

from crtmv3_gb300 import api, coefficients as co, synthetic as sy

pytestmark = pytest.mark.gpu

RAD = ("r_clear", "up_radiance", "down_radiance", "surface_planck_radiance", "upwelling_radiance",
       "upwelling_overcast_radiance", "layer_optical_depth", "sod")
REL = {0: 1e-9, 1: 1e-4}
BT = {0: 1e-4, 1: 1e-2}


@pytest.fixture(scope="module")
def cloud_dir(coeff_dir):
    sy.write_cloud_files(coeff_dir)
    sy.write_aerosol_files(coeff_dir)
    return coeff_dir


def _compare(rts, ref, precision, k_semantics=False):
    exp = dict(ref)
    if k_semantics:   # R_clear / Tb_clear of fractional profiles only
        frac = ref["total_cloud_cover"] > 0.0
        exp["r_clear"] = np.where(frac, ref["r_clear"], 0.0)
        exp["tb_clear"] = np.where(frac, ref["tb_clear"], 0.0)
    assert np.abs(rts.brightness_temperature - exp["bt"]).max() <= BT[precision]
    assert np.array_equal(rts.n_full_streams, exp["n_full_streams"])
    assert np.abs(rts.tb_clear - exp["tb_clear"]).max() <= BT[precision]
    assert np.abs(rts.total_cloud_cover - exp["total_cloud_cover"]).max() <= 1e-12
    assert np.array_equal(rts.surface_emissivity, exp["surface_emissivity"])
    for f in RAD:
        got, want = getattr(rts, f), exp[f]
        scale = max(np.abs(want).max(), 1e-300)
        assert np.abs(got - want).max() <= REL[precision] * scale, f


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("sensor", ["mwsynth_c22", "irsynth_c616"])
def test_clear_sky_components_match_oracle(gpu_lib, cloud_dir, precision, sensor):
    from oracle.pyoracle import Oracle
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, 5, 100, 71)
    opt.n_streams = np.array([0, 8, 0, 16, 0], np.int32)   # n_Full_Streams = n_Streams + 2 without clouds too
    opt.use_n_streams = opt.n_streams > 0
    ref = Oracle(cloud_dir, sensor).forward_components(atm, sfc, geo, opt)
    h = gpu_lib.CRTM([sensor], cloud_dir, precision)
    rts = h.forward(atm, sfc, geo, opt, components=True)
    _compare(rts, ref, precision)
    assert (rts.up_radiance > 0).all() and (rts.upwelling_radiance[:, :, :90] > 0).all()
    km, rk = h.k_matrix(atm, sfc, geo, opt, components=True)
    _compare(rk, ref, precision, k_semantics=True)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("sensor", ["mwsynth_c16", "irsynth_c616"])
def test_cloudy_components_match_oracle(gpu_lib, cloud_dir, precision, sensor):
    """Profiles: 0 clear, 1 cloudy (fraction 1: fractional, cover 1), 2 fractional, 3 fractional
    with 16 streams, 4 aerosols only (IR), 5 fractional with 8 streams, 6 SOI
    (FP64 form), 7 cloudy with fractions of 1e-9 (kept, as above 1e-12, but
    not fractional, as below 1e-6)."""
    from oracle.pyoracle import Oracle
    P = 8
    atm, sfc, geo, opt = sy.cloudy_workload(sensor, P, 100, 73, wc_scale=30.0)
    ir = sensor.startswith("ir")
    cf = atm.cloud_fraction
    rng = np.random.default_rng(5)
    for p in (2, 3, 5):
        cf[p] = np.where(cf[p] > 0, rng.uniform(0.2, 0.9, cf.shape[1]), 0.0)
    cf[7] = np.where(cf[7] > 0, 1e-9, 0.0)
    opt.overlap_id = np.full(P, 2, np.int32)   # random overlap
    atm.n_clouds[0] = 0
    if ir:
        sy.add_aerosols(atm, sy.AEROSOL_TYPES, 74, load_scale=5.0)
        atm.n_aerosols[[0, 1, 2, 3, 5, 6, 7]] = 0
        atm.n_clouds[4] = 0
    ns = np.array([0, 0, 0, 16, 0, 8, 0, 0], np.int32)
    opt.use_n_streams, opt.n_streams = ns > 0, ns
    if precision == 0:
        opt.rt_algorithm_id = np.array([56, 56, 56, 56, 56, 56, 168, 56], np.int32)
    aer = f"{cloud_dir}/AerosolCoeff.bin" if ir else None
    ref = Oracle(cloud_dir, sensor).forward_components(atm, sfc, geo, opt, f"{cloud_dir}/CloudCoeff.bin", aer)
    # cloud fraction 1 is above 1e-6: a fractional profile with cover 1
    assert (ref["total_cloud_cover"][[2, 3, 5]] > 0).all() and (ref["total_cloud_cover"][1] == 1.0).all()
    assert (ref["sod"][1] > 0).any() and not ref["total_cloud_cover"][[0, 7]].any()
    h = gpu_lib.CRTM([sensor], cloud_dir, precision)
    rts = h.forward(atm, sfc, geo, opt, components=True)
    _compare(rts, ref, precision)
    # the K-matrix's and the tangent linear's RTSolution
    km, rk = h.k_matrix(atm, sfc, geo, opt, components=True)
    _compare(rk, ref, precision, k_semantics=True)
    bt_tl, rt = h.tangent_linear(atm, sfc, geo, opt, components=True)
    _compare(rt, ref, precision, k_semantics=True)


def test_reference_named_forward_returns_components_on_user_layers(gpu_lib, cloud_dir):
    """CRTM_Forward fills every component; profiles whose top is below
    0.005 hPa get AddLayers' added layers, and the layer components come back
    on the user's layers (Layer_Optical_Depth(1:no) = the extended profile's
    na+1:nt, Common_RTSolution.f90:239)."""
    from oracle.pyoracle import Oracle
    from test_gpu_upper_layers import _cut_top
    sensor = "mwsynth_c22"
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, 3, 100, 75)
    atm = _cut_top(atm, (4, 11, 20))
    ci: list = []
    assert api.CRTM_Init([sensor], ci, cloud_dir) == api.SUCCESS
    out: list = []
    assert api.CRTM_Forward(atm, sfc, geo, ci, out, opt) == api.SUCCESS
    r = out[0]
    assert r.layer_optical_depth.shape == (3, co.read_spccoeff(f"{cloud_dir}/{sensor}.SpcCoeff.bin").n_channels,
                                           atm.max_layers)
    from crtmv3_gb300 import addlayers
    ext, info = addlayers.add_layers(atm)
    assert (info.n_added > 0).all()
    ref = Oracle(cloud_dir, sensor).forward_components(ext, sfc, geo, opt)
    for f in ("layer_optical_depth", "upwelling_radiance", "upwelling_overcast_radiance"):
        want = addlayers.user_layers(info, ref[f])
        assert np.abs(getattr(r, f) - want).max() <= 1e-9 * np.abs(want).max(), f
    api.CRTM_Destroy(ci)
