"""Coefficient file writers/readers (the repository's own) and the oracle's reader."""
import os

import numpy as np
import pytest

from crtmv3_gb300 import coefficients as co, synthetic as sy


def test_odps_round_trip(tmp_path):
    tc = sy.generate_odps(1, 40, 3, "t1", co.INFRARED_SENSOR)
    for bo in ("<", ">"):
        f = str(tmp_path / f"t{bo == '>'}.bin")
        co.write_odps(f, tc, byteorder=bo)
        back = co.read_odps(f)
        assert back.group_index == 1 and back.sensor_id == "t1"
        assert np.array_equal(back.c, tc.c)
        assert np.array_equal(back.n_predictors, tc.n_predictors)
        assert np.array_equal(back.pos_index, tc.pos_index)
        assert np.array_equal(back.ref_absorber, tc.ref_absorber)


def test_spccoeff_round_trip(tmp_path):
    sc = sy.generate_spccoeff("s", co.MICROWAVE_SENSOR, 12, 1)
    f = str(tmp_path / "s.bin")
    co.write_spccoeff(f, sc, byteorder=">")
    back = co.read_spccoeff(f)
    assert np.array_equal(back.planck_c1, sc.planck_c1)
    assert np.array_equal(back.cosmic_background_radiance, sc.cosmic_background_radiance)


def test_coefficient_layout_matches_pos_index():
    """C(Pos_Index(j,l) + (i-1)*K + k - 1) is predictor i, layer k (ODPS_AtmAbsorption.f90:198-204)."""
    tc = sy.generate_odps(2, 5, 9, "t2", co.MICROWAVE_SENSOR, max_predictors_per_channel=20)
    for l in range(5):
        assert tc.n_predictors[:, l].sum() <= 20
        for j in range(tc.n_components):
            blk = tc.coeff_block(j, l)
            assert blk.shape == (tc.n_predictors[j, l], tc.n_layers)


def test_oracle_reads_both_byte_orders(tmp_path):
    from oracle.pyoracle import Oracle
    for bo, d in (("<", tmp_path / "le"), (">", tmp_path / "be")):
        os.makedirs(d)
        tc = sy.generate_odps(3, 6, 5, "mw", co.MICROWAVE_SENSOR)
        sc = sy.generate_spccoeff("mw", co.MICROWAVE_SENSOR, 6, 6)
        co.write_odps(str(d / "mw.TauCoeff.bin"), tc, byteorder=bo)
        co.write_spccoeff(str(d / "mw.SpcCoeff.bin"), sc, byteorder=bo)
    atm, sfc, geo = sy.generate_profiles(2, 40, (co.H2O_ID,), 4)
    opt = sy.OptionsBatch(emissivity=sy.emissivity_for(1, 2, 6, 1))
    r1 = Oracle(str(tmp_path / "le"), "mw").forward(atm, sfc, geo, opt)[1]
    r2 = Oracle(str(tmp_path / "be"), "mw").forward(atm, sfc, geo, opt)[1]
    assert np.array_equal(r1, r2)


@pytest.mark.parametrize("damage", ["truncate", "magic", "pos_index"])
def test_oracle_rejects_corrupt_files(tmp_path, damage):
    from oracle.pyoracle import Oracle
    tc = sy.generate_odps(3, 4, 5, "mw", co.MICROWAVE_SENSOR)
    sc = sy.generate_spccoeff("mw", co.MICROWAVE_SENSOR, 4, 6)
    if damage == "pos_index":
        tc.pos_index = tc.pos_index.copy()
        tc.pos_index[0, 0] = tc.c.size + 10
    co.write_odps(str(tmp_path / "mw.TauCoeff.bin"), tc)
    co.write_spccoeff(str(tmp_path / "mw.SpcCoeff.bin"), sc)
    f = tmp_path / "mw.TauCoeff.bin"
    raw = f.read_bytes()
    if damage == "truncate":
        f.write_bytes(raw[: len(raw) // 2])
    elif damage == "magic":
        f.write_bytes(raw[:4] + b"\x00\x00\x00\x00" + raw[8:])
    with pytest.raises(IOError):
        Oracle(str(tmp_path), "mw")
