"""netCDF-classic SpcCoeff / ODPS TauCoeff files (crtmv3_gb300/netcdf_coeffs.py):
the reference's variable names, types and dimension order
(SpcCoeff_netCDF_IO.f90:68-183, ODPS_netCDF_IO.f90:63-240), lossless round
trips through the binary formats, the OPTRAN variables, and CRTM_Init's
SpcCoeff_Format / TauCoeff_Format options.  Exact comparisons throughout."""
import filecmp
import os

import numpy as np
import pytest
from scipy.io import netcdf_file

from crtmv3_gb300 import api, coefficients as co, netcdf_coeffs as nc, synthetic as sy


def _fields_equal(a, b):
    for f in a.__dataclass_fields__:
        x, y = getattr(a, f), getattr(b, f)
        if isinstance(x, np.ndarray) or isinstance(y, np.ndarray):
            np.testing.assert_array_equal(np.asarray(x), np.asarray(y), err_msg=f)
            assert np.asarray(x).dtype == np.asarray(y).dtype, f
        elif hasattr(x, "__dataclass_fields__") and hasattr(y, "__dataclass_fields__"):
            _fields_equal(x, y)
        else:
            assert x == y, f


@pytest.mark.parametrize("sensor", sy.SENSORS)
def test_round_trip_is_lossless(coeff_dir, tmp_path, sensor):
    tc = co.read_odps(os.path.join(coeff_dir, f"{sensor}.TauCoeff.bin"))
    sc = co.read_spccoeff(os.path.join(coeff_dir, f"{sensor}.SpcCoeff.bin"))
    nc.write_odps_nc(str(tmp_path / f"{sensor}.TauCoeff.nc"), tc)
    nc.write_spccoeff_nc(str(tmp_path / f"{sensor}.SpcCoeff.nc"), sc)
    _fields_equal(nc.read_odps_nc(str(tmp_path / f"{sensor}.TauCoeff.nc")), tc)
    _fields_equal(nc.read_spccoeff_nc(str(tmp_path / f"{sensor}.SpcCoeff.nc")), sc)
    out = tmp_path / "bin"
    out.mkdir()
    nc.convert_sensor(str(tmp_path), sensor, str(out), "netCDF", "netCDF")
    for kind in ("TauCoeff", "SpcCoeff"):
        assert filecmp.cmp(str(out / f"{sensor}.{kind}.bin"), os.path.join(coeff_dir, f"{sensor}.{kind}.bin"),
                           shallow=False), kind


def test_reference_layout(coeff_dir, tmp_path):
    sensor = "irsynth_c616"
    tc = co.read_odps(os.path.join(coeff_dir, f"{sensor}.TauCoeff.bin"))
    sc = co.read_spccoeff(os.path.join(coeff_dir, f"{sensor}.SpcCoeff.bin"))
    nc.write_odps_nc(str(tmp_path / "t.nc"), tc)
    nc.write_spccoeff_nc(str(tmp_path / "s.nc"), sc)
    with netcdf_file(str(tmp_path / "t.nc"), "r", mmap=False) as f:
        assert f.version_byte == 1   # netCDF classic
        dims = {k: f.variables[k].dimensions for k in f.variables}
        assert dims["Ref_Absorber"] == ("n_Absorbers", "n_Layers")
        assert dims["n_Predictors"] == ("n_Channels", "n_Components")
        assert dims["Pos_Index"] == ("n_Channels", "n_Components")
        assert dims["Ref_Level_Pressure"] == ("n_Levels",)
        assert dims["ODPS_Coefficients"] == ("n_Coeffs",)
        assert dims["Group_Index"] == () and dims["Sensor_Type"] == ()
        assert f.variables["ODPS_Coefficients"].data.dtype == np.dtype(">f4")
        assert f.variables["Ref_Absorber"].data.dtype == np.dtype(">f8")
        assert f.variables["Pos_Index"].data.dtype == np.dtype(">i4")
        assert f.Sensor_Id == sensor.encode()
        np.testing.assert_array_equal(f.variables["Absorber_ID"].data, tc.absorber_id)
        np.testing.assert_array_equal(f.variables["Ref_Absorber"].data, tc.ref_absorber.T)
    with netcdf_file(str(tmp_path / "s.nc"), "r", mmap=False) as f:
        for v in ("Sensor_Channel", "Polarization", "Polarization_Angle", "Channel_Flag", "Frequency",
                  "Wavenumber", "Planck_C1", "Planck_C2", "Band_C1", "Band_C2",
                  "Cosmic_Background_Radiance", "Solar_Irradiance"):
            assert f.variables[v].dimensions == ("n_Channels",), v
        assert f.variables["Sensor_Type"].dimensions == ()


def test_optran_variables_round_trip(coeff_dir, tmp_path):
    """A TauCoeff with the compact-OPTRAN term through netCDF and back to a
    byte-identical binary file; a file whose n_OCoeffs dimension lacks the
    OPTRAN variables is refused."""
    sensor = "irsynth_o120"
    src = os.path.join(coeff_dir, f"{sensor}.TauCoeff.bin")
    tc = co.read_odps(src)
    assert tc.optran is not None
    p = str(tmp_path / "o.nc")
    nc.write_odps_nc(p, tc)
    with netcdf_file(p, "r", mmap=False) as f:
        assert f.variables["OP_Index"].dimensions == ("n_Channels", "n_OPIndex")
        assert f.dimensions["n_OPIndex"] == 7 and f.dimensions["n_OCoeffs"] == tc.optran.oc.size
    back = str(tmp_path / "o.bin")
    co.write_odps(back, nc.read_odps_nc(p))
    with open(back, "rb") as a, open(src, "rb") as b:
        assert a.read() == b.read()
    bad = str(tmp_path / "b.nc")
    nc.write_odps_nc(bad, co.read_odps(os.path.join(coeff_dir, "mwsynth_c22.TauCoeff.bin")))
    with netcdf_file(bad, "a") as f:
        f.createDimension("n_OCoeffs", 4)
    with pytest.raises(ValueError, match="OPTRAN"):
        nc.read_odps_nc(bad)


def test_crtm_init_formats(coeff_dir, tmp_path, monkeypatch):
    sensor = "mwsynth_c22"
    src = tmp_path / "nc"
    src.mkdir()
    nc.write_odps_nc(str(src / f"{sensor}.TauCoeff.nc"),
                     co.read_odps(os.path.join(coeff_dir, f"{sensor}.TauCoeff.bin")))
    os.symlink(os.path.join(coeff_dir, f"{sensor}.SpcCoeff.bin"), str(src / f"{sensor}.SpcCoeff.bin"))
    seen = {}

    class FakeCRTM:   # stands in for the library handle: records the directory it is given
        def __init__(self, ids, path, *a):
            seen["path"] = path
            self.n_channels = [co.read_spccoeff(os.path.join(path, f"{i}.SpcCoeff.bin")).n_channels for i in ids]

    monkeypatch.setattr(api, "CRTM", FakeCRTM)
    ci = []
    assert api.CRTM_Init([sensor], ci, str(src), taucoeff_format="netCDF") == api.SUCCESS
    d = seen["path"]
    assert d != str(src)
    assert filecmp.cmp(os.path.join(d, f"{sensor}.TauCoeff.bin"),
                       os.path.join(coeff_dir, f"{sensor}.TauCoeff.bin"), shallow=False)
    assert ci[0].n_channels == 22
    # binary default: the directory is used as it is
    assert api.CRTM_Init([sensor], ci, coeff_dir) == api.SUCCESS and seen["path"] == coeff_dir
    # a missing file or an unknown format fails the call
    assert api.CRTM_Init([sensor], ci, str(src), spccoeff_format="netCDF") == api.FAILURE
    assert api.CRTM_Init([sensor], ci, str(src), taucoeff_format="HDF") == api.FAILURE


def test_irwater_round_trip_and_init(coeff_dir, tmp_path, monkeypatch):
    from crtmv3_gb300 import synthetic as sy2
    binp = sy2.write_irwater_file(str(tmp_path))
    wc = co.read_irwatercoeff(binp)
    src = tmp_path / "src"
    src.mkdir()
    nc.write_irwater_nc(str(src / (nc.IRWATER_FILE + ".nc")), wc)
    with netcdf_file(str(src / (nc.IRWATER_FILE + ".nc")), "r", mmap=False) as f:
        assert f.variables["Emissivity"].dimensions == ("n_Temperature", "n_Wind_Speeds", "n_Frequencies",
                                                         "n_Angles")
    _fields_equal(nc.read_irwater_nc(str(src / (nc.IRWATER_FILE + ".nc"))), wc)
    sensor = "irsynth_c616"
    for kind in ("TauCoeff", "SpcCoeff"):
        os.symlink(os.path.join(coeff_dir, f"{sensor}.{kind}.bin"), str(src / f"{sensor}.{kind}.bin"))
    seen = {}

    class FakeCRTM:
        def __init__(self, ids, path, *a):
            seen["path"] = path
            self.n_channels = [616]

    monkeypatch.setattr(api, "CRTM", FakeCRTM)
    assert api.CRTM_Init([sensor], [], str(src), irwatercoeff_format="netCDF") == api.SUCCESS
    assert filecmp.cmp(os.path.join(seen["path"], nc.IRWATER_FILE + ".bin"), binp, shallow=False)
