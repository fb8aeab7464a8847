"""The compact-OPTRAN water-vapour-line term of an ODPS TauCoeff (A9): the
file's OPTRAN record round trip, and the oracle's restatement of
ODPS_Compute_Predictor_ODAS / Add_OPTRAN_wloOD and their adjoints checked
against central differences of its own forward (T and H2O Jacobians) and
against the same file with the OPTRAN record removed (the OPTRAN channels
change, the others do not)."""
import dataclasses
import os

import numpy as np
import pytest

from crtmv3_gb300 import coefficients as co, synthetic as sy

SENSOR = "irsynth_o120"


@pytest.fixture(scope="module")
def files(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("optran"))
    sy.write_sensor_files(d, SENSOR)
    # the same sensor without the OPTRAN record
    tc = co.read_odps(os.path.join(d, f"{SENSOR}.TauCoeff.bin"))
    plain = dataclasses.replace(tc, sensor_id="irsynth_p120", optran=None)
    co.write_odps(os.path.join(d, "irsynth_p120.TauCoeff.bin"), plain)
    os.link(os.path.join(d, f"{SENSOR}.SpcCoeff.bin"), os.path.join(d, "irsynth_p120.SpcCoeff.bin"))
    return d, tc


def test_optran_record_round_trip(files, tmp_path):
    d, tc = files
    o = tc.optran
    assert o is not None and o.significance.sum() > 20 and o.component_index == 2
    p = str(tmp_path / "x.TauCoeff.bin")
    co.write_odps(p, tc)
    back = co.read_odps(p)
    for f in dataclasses.fields(co.OPTRANCoeff):
        np.testing.assert_array_equal(getattr(back.optran, f.name), getattr(o, f.name))
    with open(p, "rb") as a, open(os.path.join(d, f"{SENSOR}.TauCoeff.bin"), "rb") as b:
        assert a.read() == b.read()


def test_optran_changes_only_its_channels(files):
    from oracle.pyoracle import Oracle
    d, tc = files
    atm, sfc, geo, opt = sy.clear_sky_workload(SENSOR, 4, 100, 31)
    _, bt = Oracle(d, SENSOR).forward(atm, sfc, geo, opt)
    _, bt0 = Oracle(d, "irsynth_p120").forward(atm, sfc, geo, opt)
    on = tc.optran.significance == co.SIGNIFICANCE_OPTRAN
    np.testing.assert_array_equal(bt[:, ~on], bt0[:, ~on])
    assert np.abs(bt[:, on] - bt0[:, on]).max() > 0.05


def test_optran_k_matrix_matches_central_differences(files):
    from oracle.pyoracle import Oracle
    d, tc = files
    atm, sfc, geo, opt = sy.clear_sky_workload(SENSOR, 2, 100, 33)
    o = Oracle(d, SENSOR)
    ref = o.k_matrix(atm, sfc, geo, opt)
    on = np.flatnonzero(tc.optran.significance == co.SIGNIFICANCE_OPTRAN)
    kt, ka = ref["temperature_k"], ref["absorber_k"]
    h2o = list(atm.absorber_id).index(co.H2O_ID)
    checked = 0
    for k in (3, 30, 60, 85, 97):
        for what in ("t", "q"):
            bts = []
            for sgn in (1, -1):
                a = dataclasses.replace(atm, temperature=atm.temperature.copy(), absorber=atm.absorber.copy())
                if what == "t":
                    a.temperature[:, k] += sgn * 0.01
                else:
                    a.absorber[:, h2o, k] *= 1.0 + sgn * 1e-4
                bts.append(o.forward(a, sfc, geo, opt)[1])
            if what == "t":
                fd, got, scale = (bts[0] - bts[1]) / 0.02, kt[:, :, k], np.abs(kt).max()
            else:
                step = 1e-4 * atm.absorber[:, h2o, k][:, None]
                fd, got = (bts[0] - bts[1]) / (2 * step), ka[:, :, h2o, k]
                scale = np.abs(ka[:, :, h2o] * atm.absorber[:, h2o][:, None]).max()
                fd, got = fd * atm.absorber[:, h2o, k][:, None], got * atm.absorber[:, h2o, k][:, None]
            assert np.abs(fd[:, on] - got[:, on]).max() <= 2e-5 * scale, (what, k)
            checked += 1
    assert checked == 10
    # adjoint = seeded K-matrix summed over channels
    seed = np.random.default_rng(4).uniform(0.5, 1.5, (2, tc.n_channels))
    kk = o.k_matrix(atm, sfc, geo, opt, seed)
    ad = o.adjoint(atm, sfc, geo, opt, seed)
    np.testing.assert_allclose(ad["temperature_ad"], kk["temperature_k"].sum(axis=1), rtol=1e-10,
                               atol=1e-12 * np.abs(kk["temperature_k"]).max())
