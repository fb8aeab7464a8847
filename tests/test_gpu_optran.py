"""The compact-OPTRAN water-vapour-line term on the GPU against the oracle
(A9), on a 120-channel infrared sensor whose water vapour line component is
OPTRAN for 75 channels: forward, K-matrix (temperature and every absorber),
adjoint, a channel subset mixing OPTRAN and ODPS channels, and a cloudy batch.

Tolerances as the other parity tests: FP64 form 1e-4 K and 1e-6 of the
largest Jacobian; mixed form 0.01 K and 1e-3."""
import numpy as np
import pytest

from crtmv3_gb300 import coefficients as co, synthetic as sy

pytestmark = pytest.mark.gpu

SENSOR = "irsynth_o120"
BT_TOL = {0: 1e-4, 1: 1e-2}
JAC_TOL = {0: 1e-6, 1: 1e-3}


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("precision", [0, 1])
def test_optran_forward_and_k_matrix_match_oracle(gpu_lib, coeff_dir, precision):
    from oracle.pyoracle import Oracle
    atm, sfc, geo, opt = sy.clear_sky_workload(SENSOR, 6, 100, 41)
    o = Oracle(coeff_dir, SENSOR)
    h = gpu_lib.CRTM([SENSOR], coeff_dir, precision)
    seed = np.random.default_rng(2).uniform(0.5, 1.5, (6, h.n_channels[0]))
    ref = o.k_matrix(atm, sfc, geo, opt, seed)
    km, rts = h.k_matrix(atm, sfc, geo, opt, seed)
    assert np.abs(rts.brightness_temperature - ref["bt"]).max() < BT_TOL[precision]
    assert np.abs(h.forward(atm, sfc, geo, opt).brightness_temperature - ref["bt"]).max() < BT_TOL[precision]
    tol = JAC_TOL[precision]
    assert _rel(km.temperature, ref["temperature_k"]) < tol
    for j in range(atm.n_absorbers):
        assert _rel(km.absorber[:, :, j], ref["absorber_k"][:, :, j]) < tol * 10, j
    on = co.read_odps(f"{coeff_dir}/{SENSOR}.TauCoeff.bin").optran.significance == co.SIGNIFICANCE_OPTRAN
    h2o = list(atm.absorber_id).index(co.H2O_ID)
    assert _rel(km.absorber[:, on, h2o], ref["absorber_k"][:, on, h2o]) < tol
    ad, _ = h.adjoint(atm, sfc, geo, opt, seed)
    ra = o.adjoint(atm, sfc, geo, opt, seed)
    assert _rel(ad["temperature"], ra["temperature_ad"]) < tol
    assert _rel(ad["absorber"][:, h2o], ra["absorber_ad"][:, h2o]) < tol


def test_optran_channel_subset(gpu_lib, coeff_dir):
    atm, sfc, geo, opt = sy.clear_sky_workload(SENSOR, 3, 90, 43)
    h = gpu_lib.CRTM([SENSOR], coeff_dir, 0)
    full, fr = h.k_matrix(atm, sfc, geo, opt)
    pos = np.arange(5, 120, 7, dtype=np.int32)
    h.set_channel_subset(0, pos)
    o2 = dict(vars(opt))
    o2["emissivity"] = opt.emissivity[:, pos]
    sub, sr = h.k_matrix(atm, sfc, geo, type(opt)(**o2))
    assert np.array_equal(sr.brightness_temperature, fr.brightness_temperature[:, pos])
    assert np.array_equal(sub.absorber, full.absorber[:, pos])


def test_optran_cloudy_forward_matches_oracle(gpu_lib, coeff_dir):
    from oracle.pyoracle import Oracle
    cloud_dir = coeff_dir
    sy.write_cloud_files(cloud_dir)
    atm, sfc, geo, opt = sy.cloudy_workload(SENSOR, 4, 100, 45, cloud_types=(co.WATER_CLOUD, co.ICE_CLOUD),
                                            wc_scale=30.0)
    atm.n_clouds[1] = 0
    _, ref = Oracle(cloud_dir, SENSOR).forward_scatter(atm, sfc, geo, opt, f"{cloud_dir}/CloudCoeff.bin")
    rts = gpu_lib.CRTM([SENSOR], cloud_dir, 0).forward(atm, sfc, geo, opt)
    assert np.abs(rts.brightness_temperature - ref).max() < BT_TOL[0]
