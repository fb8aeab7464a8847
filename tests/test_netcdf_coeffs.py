"""netCDF-classic coefficient files (crtmv3_gb300/netcdf_coeffs.py): SpcCoeff,
ODPS TauCoeff, IRwaterCoeff, CloudCoeff and AerosolCoeff in the reference's
variable names, types and dimension order (each *_netCDF_IO.f90), lossless
round trips through the binary formats, the OPTRAN variables, and CRTM_Init's
*_Format options.  Exact comparisons throughout."""
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


def test_cloudcoeff_round_trip_and_layout(tmp_path):
    """CloudCoeff through netCDF and back to a byte-identical binary file, in
    the layout of CloudCoeff_netCDF_IO.f90:2020-2545: the MW tables over
    (n_Temperatures | n_MW_Densities, n_MW_Radii, n_MW_Frequencies), the IR
    tables over the IR density axis, pcoeff_IR 4-D over n_Legendre_Terms."""
    src = tmp_path / "src"
    src.mkdir()
    binp = sy.write_cloud_files(str(src))
    cc = co.read_cloudcoeff(binp)
    nc.write_cloudcoeff_nc(str(src / "CloudCoeff.nc"), cc)
    _fields_equal(nc.read_cloudcoeff_nc(str(src / "CloudCoeff.nc")), cc)
    out = tmp_path / "out"
    out.mkdir()
    nc.convert_cloud(str(src), str(out))
    assert filecmp.cmp(str(out / "CloudCoeff.bin"), binp, shallow=False)
    nl, nd = cc.n_legendre_terms, cc.density_mw.size
    with netcdf_file(str(src / "CloudCoeff.nc"), "r", mmap=False) as f:
        assert f.version_byte == 1
        assert f.dimensions["n_Legendre_Terms"] == nl + 1
        assert f.dimensions["n_IR_Densities"] == nd + 1
        dims = {k: f.variables[k].dimensions for k in f.variables}
        assert dims["ke_L_MW"] == ("n_Temperatures", "n_MW_Radii", "n_MW_Frequencies")
        assert dims["kb_S_MW"] == ("n_MW_Densities", "n_MW_Radii", "n_MW_Frequencies")
        assert dims["pcoeff_L_MW"] == ("n_Phase_Elements", "n_Legendre_Terms", "n_Temperatures",
                                       "n_MW_Radii", "n_MW_Frequencies")
        assert dims["pcoeff_IR"] == ("n_Legendre_Terms", "n_IR_Densities", "n_IR_Radii", "n_IR_Frequencies")
        assert dims["Water_Density_MW"] == ("n_MW_Radii",) and dims["Density_IR"] == ("n_IR_Densities",)
        assert f.variables["ke_IR"].data.dtype == np.dtype(">f8")
        np.testing.assert_array_equal(f.variables["ke_L_MW"].data, cc.ke_l_mw.transpose(2, 1, 0))
        np.testing.assert_array_equal(f.variables["pcoeff_IR"].data[:nl], cc.pcoeff_ir[..., 0].transpose(3, 2, 1, 0))
        assert not f.variables["pcoeff_IR"].data[nl].any()
        assert not f.variables["kb_IR"].data.any()


@pytest.mark.parametrize("scheme", co.AEROSOL_SCHEMES)
def test_aerosolcoeff_round_trip_and_layout(tmp_path, scheme):
    """AerosolCoeff of each aerosol scheme through netCDF and back to a
    byte-identical binary file (AerosolCoeff_netCDF_IO.f90:1540-1830): the
    RH variable over n_RH_Radii for 'CRTM' / 'CMAQ', over n_RH otherwise;
    a file read for a scheme whose layout it lacks is refused."""
    src = tmp_path / "src"
    src.mkdir()
    binp = sy.write_aerosol_files(str(src), scheme)
    ac = co.read_aerosolcoeff(binp, scheme)
    ncp = str(src / "AerosolCoeff.nc")
    nc.write_aerosolcoeff_nc(ncp, ac, scheme)
    _fields_equal(nc.read_aerosolcoeff_nc(ncp, scheme), ac)
    out = tmp_path / "out"
    out.mkdir()
    name = nc.convert_aerosol(str(src), str(out), scheme)
    assert filecmp.cmp(str(out / name), binp, shallow=False)
    rh_radii = scheme in ("CRTM", "CMAQ")
    with netcdf_file(ncp, "r", mmap=False) as f:
        dims = {k: f.variables[k].dimensions for k in f.variables}
        assert dims["RH"] == (("n_RH_Radii",) if rh_radii else ("n_RH",))
        assert dims["ke"] == ("n_Types", "n_Sigma", "n_Radii", "n_RH", "n_Wavelengths")
        assert dims["pcoeff"] == ("n_Phase_Elements", "n_Legendre_Terms", "n_Types", "n_Sigma", "n_Radii",
                                  "n_RH", "n_Wavelengths")
        assert dims["Reff"] == ("n_Types", "n_Radii") and dims["Aerosol_Type_Name"] == ("n_Types", "tnsl")
        assert f.dimensions["tnsl"] == co.AEROSOL_SL
        np.testing.assert_array_equal(f.variables["Aerosol_Type"].data, ac.type_id)
        np.testing.assert_array_equal(f.variables["ke"].data, ac.ke.transpose(4, 3, 2, 1, 0))
    other = "NAAPS" if rh_radii else "CRTM"
    with pytest.raises(ValueError, match="n_RH_Radii"):
        nc.read_aerosolcoeff_nc(ncp, other)


def test_crtm_init_cloud_and_aerosol_formats(coeff_dir, tmp_path, monkeypatch):
    """CloudCoeff_Format / AerosolCoeff_Format = 'netCDF' and CloudCoeff_File
    (src/CRTM_LifeCycle.f90:679-800): the tables the library loads are the
    binary files the netCDF files came from."""
    sensor = "irsynth_c616"
    src = tmp_path / "src"
    src.mkdir()
    for kind in ("TauCoeff", "SpcCoeff"):
        os.symlink(os.path.join(coeff_dir, f"{sensor}.{kind}.bin"), str(src / f"{sensor}.{kind}.bin"))
    ref = tmp_path / "ref"
    ref.mkdir()
    cloud_bin = sy.write_cloud_files(str(ref))
    aer_bin = sy.write_aerosol_files(str(ref), "CMAQ")
    nc.write_cloudcoeff_nc(str(src / "MyClouds.nc"), co.read_cloudcoeff(cloud_bin))
    nc.write_aerosolcoeff_nc(str(src / "AerosolCoeff.nc"), co.read_aerosolcoeff(aer_bin, "CMAQ"), "CMAQ")
    seen = {}

    class FakeCRTM:
        def __init__(self, ids, path, *a):
            seen["path"], seen["args"] = path, a
            self.n_channels = [616]

    monkeypatch.setattr(api, "CRTM", FakeCRTM)
    assert api.CRTM_Init([sensor], [], str(src), aerosol_model="CMAQ", cloudcoeff_format="netCDF",
                         cloudcoeff_file="MyClouds.nc", aerosolcoeff_format="netCDF") == api.SUCCESS
    d = seen["path"]
    assert filecmp.cmp(os.path.join(d, "CloudCoeff.bin"), cloud_bin, shallow=False)
    assert seen["args"][1:] == ("CMAQ", "AerosolCoeff.bin")
    assert filecmp.cmp(os.path.join(d, "AerosolCoeff.bin"), aer_bin, shallow=False)
    # a binary cloud table under another name is loaded as CloudCoeff.bin
    os.symlink(cloud_bin, str(src / "Other.bin"))
    assert api.CRTM_Init([sensor], [], str(src), cloudcoeff_file="Other.bin") == api.SUCCESS
    assert filecmp.cmp(os.path.join(seen["path"], "CloudCoeff.bin"), cloud_bin, shallow=False)
    # the aerosol file read for a scheme whose layout it lacks fails the call
    assert api.CRTM_Init([sensor], [], str(src), aerosol_model="NAAPS",
                         aerosolcoeff_format="netCDF") == api.FAILURE


def test_crtm_init_table_options(coeff_dir, tmp_path, monkeypatch):
    """NC_File_Path (the netCDF tables' directory), IRwaterCoeff_File,
    Load_CloudCoeff and Load_AerosolCoeff (src/CRTM_LifeCycle.f90:653-656,
    :782-815, :865-867): the private directory holds exactly the tables the
    options ask for."""
    sensor = "irsynth_c616"
    src, ncdir, ref = tmp_path / "src", tmp_path / "ncdir", tmp_path / "ref"
    for d in (src, ncdir, ref):
        d.mkdir()
    for kind in ("TauCoeff", "SpcCoeff"):
        os.symlink(os.path.join(coeff_dir, f"{sensor}.{kind}.bin"), str(src / f"{sensor}.{kind}.bin"))
    cloud_bin = sy.write_cloud_files(str(ref))
    aer_bin = sy.write_aerosol_files(str(ref))
    os.symlink(cloud_bin, str(src / "CloudCoeff.bin"))
    os.symlink(aer_bin, str(src / "AerosolCoeff.bin"))
    wc = sy.generate_irwatercoeff()
    co.write_irwatercoeff(str(ref / "water.bin"), wc)
    nc.write_irwater_nc(str(ncdir / "MyWater.nc"), wc)
    nc.write_cloudcoeff_nc(str(ncdir / "CloudCoeff.nc"), co.read_cloudcoeff(cloud_bin))
    seen = {}

    class FakeCRTM:
        def __init__(self, ids, path, *a):
            seen["path"], seen["args"] = path, a
            self.n_channels = [616]

    monkeypatch.setattr(api, "CRTM", FakeCRTM)
    # netCDF tables from NC_File_Path; the sensors' files from File_Path
    assert api.CRTM_Init([sensor], [], str(src), nc_file_path=str(ncdir), cloudcoeff_format="netCDF",
                         irwatercoeff_format="netCDF", irwatercoeff_file="MyWater.nc",
                         cloud_model="CRTM") == api.SUCCESS
    d = seen["path"]
    assert filecmp.cmp(os.path.join(d, "CloudCoeff.bin"), cloud_bin, shallow=False)
    assert filecmp.cmp(os.path.join(d, nc.IRWATER_FILE + ".bin"), str(ref / "water.bin"), shallow=False)
    assert filecmp.cmp(os.path.join(d, "AerosolCoeff.bin"), aer_bin, shallow=False)
    # a binary IR water table under another name
    os.symlink(str(ref / "water.bin"), str(src / "water.bin"))
    assert api.CRTM_Init([sensor], [], str(src), irwatercoeff_file="water.bin") == api.SUCCESS
    assert filecmp.cmp(os.path.join(seen["path"], nc.IRWATER_FILE + ".bin"), str(ref / "water.bin"),
                       shallow=False)
    # Load_CloudCoeff / Load_AerosolCoeff = False: the tables are left out
    assert api.CRTM_Init([sensor], [], str(src), aerosol_model="CRTM", load_cloudcoeff=False,
                         load_aerosolcoeff=False) == api.SUCCESS
    d = seen["path"]
    assert d != str(src)
    assert not os.path.exists(os.path.join(d, "CloudCoeff.bin"))
    assert not os.path.exists(os.path.join(d, "AerosolCoeff.bin"))
    assert seen["args"][1:] == (None, None)
    assert os.path.exists(os.path.join(d, f"{sensor}.TauCoeff.bin"))


def test_cloudcoeff_nc_refuses_tables_it_cannot_hold(tmp_path):
    """pcoeff_IR has no phase dimension in the reference's layout, so a table
    with more than one phase element is refused rather than truncated; a file
    of another release is refused on reading."""
    cc = sy.generate_cloudcoeff()
    many = co.CloudCoeff(**{f: getattr(cc, f) for f in cc.__dataclass_fields__})
    many.pcoeff_l_mw = np.repeat(cc.pcoeff_l_mw, 2, axis=4)
    with pytest.raises(ValueError, match="n_Phase_Elements"):
        nc.write_cloudcoeff_nc(str(tmp_path / "x.nc"), many)
    nc.write_cloudcoeff_nc(str(tmp_path / "c.nc"), cc)
    with netcdf_file(str(tmp_path / "c.nc"), "a") as f:
        f.Release = np.int32(co.CLOUDCOEFF_RELEASE + 1)
    with pytest.raises(ValueError, match="release"):
        nc.read_cloudcoeff_nc(str(tmp_path / "c.nc"))

