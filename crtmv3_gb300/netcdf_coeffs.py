"""netCDF (classic format) coefficient files -- SpcCoeff, ODPS TauCoeff,
IRwaterCoeff, CloudCoeff and AerosolCoeff: readers, writers and the
conversion to the binary files that crtm_gpu_init loads.

The reference writes them with NF90_CREATE(..., NF90_CLOBBER), i.e. netCDF
classic (src/Coefficients/SpcCoeff/SpcCoeff_netCDF_IO.f90:1501,
src/Coefficients/TauCoeff/ODPS/ODPS_netCDF_IO.f90:1471).  Names, types and
dimensions follow each file's *_netCDF_IO.f90, cited at each writer.
A Fortran variable dimensioned (a, b) is stored in netCDF as (b, a), so the
arrays are transposed on the way in and out.

CRTM_Init's SpcCoeff_Format / TauCoeff_Format / CloudCoeff_Format /
AerosolCoeff_Format = 'netCDF' (src/CRTM_LifeCycle.f90:523-561, 783-800)
reads <Sensor_Id>.SpcCoeff.nc, <Sensor_Id>.TauCoeff.nc, CloudCoeff.nc and
AerosolCoeff.nc.  crtmv3_gb300.api.CRTM_Init does the same through the
``convert_*`` functions: the files become binary files in a private
directory, which the library then loads.
"""
from __future__ import annotations

import os
import shutil
import numpy as np
from scipy.io import netcdf_file

from . import coefficients as co

N_COMPONENTS_G = co.N_COMPONENTS_G
N_ABSORBERS_G = co.N_ABSORBERS_G


def _attr(f, name, default=None):
    v = getattr(f, name, default)
    if isinstance(v, bytes):
        return v.decode().strip()
    if isinstance(v, np.ndarray) and v.size == 1:
        return v.item()
    return v


def _var(f, name, dtype=None):
    if name not in f.variables:
        raise ValueError(f"netCDF coefficient file: variable {name} missing")
    a = np.array(f.variables[name].data)
    return a if dtype is None else a.astype(dtype)


# ---------------------------------------------------------------------------
# SpcCoeff
# ---------------------------------------------------------------------------

def write_spccoeff_nc(path: str, sc: co.SpcCoeff) -> None:
    """SpcCoeff_netCDF_IO's layout (:68-183): dimension n_Channels, scalar
    Sensor_Type, per-channel variables, Sensor_Id and WMO ids as global
    attributes."""
    L = sc.n_channels
    with netcdf_file(path, "w", version=1) as f:
        f.Release = np.int32(co.SPCCOEFF_RELEASE)
        f.Version = np.int32(1)
        f.Sensor_Id = sc.sensor_id
        f.WMO_Satellite_Id = np.int32(sc.wmo_satellite_id)
        f.WMO_Sensor_Id = np.int32(sc.wmo_sensor_id)
        f.createDimension("n_Channels", L)
        v = f.createVariable("Sensor_Type", "i4", ())
        v[...] = np.int32(sc.sensor_type)
        cols = [("Sensor_Channel", "i4", sc.sensor_channel),
                ("Polarization", "i4", sc.polarization if sc.polarization is not None else np.zeros(L)),
                ("Polarization_Angle", "f8", sc.pol_angle if sc.pol_angle is not None else np.zeros(L)),
                ("Channel_Flag", "i4", sc.channel_flag if sc.channel_flag is not None else np.zeros(L)),
                ("Frequency", "f8", sc.frequency), ("Wavenumber", "f8", sc.wavenumber),
                ("Planck_C1", "f8", sc.planck_c1), ("Planck_C2", "f8", sc.planck_c2),
                ("Band_C1", "f8", sc.band_c1), ("Band_C2", "f8", sc.band_c2),
                ("Cosmic_Background_Radiance", "f8", sc.cosmic_background_radiance),
                ("Solar_Irradiance", "f8", sc.solar_irradiance)]
        for name, t, data in cols:
            v = f.createVariable(name, t, ("n_Channels",))
            v[:] = np.asarray(data).astype(t)


def read_spccoeff_nc(path: str) -> co.SpcCoeff:
    with netcdf_file(path, "r", mmap=False) as f:
        return co.SpcCoeff(
            sensor_id=str(_attr(f, "Sensor_Id", "")),
            sensor_type=int(f.variables["Sensor_Type"].data[()]),
            sensor_channel=_var(f, "Sensor_Channel", np.int32),
            frequency=_var(f, "Frequency", np.float64), wavenumber=_var(f, "Wavenumber", np.float64),
            planck_c1=_var(f, "Planck_C1", np.float64), planck_c2=_var(f, "Planck_C2", np.float64),
            band_c1=_var(f, "Band_C1", np.float64), band_c2=_var(f, "Band_C2", np.float64),
            cosmic_background_radiance=_var(f, "Cosmic_Background_Radiance", np.float64),
            solar_irradiance=_var(f, "Solar_Irradiance", np.float64),
            polarization=_var(f, "Polarization", np.int32),
            pol_angle=_var(f, "Polarization_Angle", np.float64),
            channel_flag=_var(f, "Channel_Flag", np.int32),
            wmo_satellite_id=int(_attr(f, "WMO_Satellite_Id", 1023)),
            wmo_sensor_id=int(_attr(f, "WMO_Sensor_Id", 2047)))


# ---------------------------------------------------------------------------
# ODPS TauCoeff
# ---------------------------------------------------------------------------

def write_odps_nc(path: str, tc: co.ODPSCoeff) -> None:
    """ODPS_netCDF_IO's layout (:63-240), with the compact-OPTRAN variables
    (OSignificance, Order, OP_Index, OPos_Index, OC, Alpha, Alpha_C1,
    Alpha_C2, OComponent_Index; dimensions n_OPIndex and n_OCoeffs, :80-107,
    :232-240) when the file has them."""
    J, Jm, K, L = tc.n_components, tc.n_absorbers, tc.n_layers, int(tc.sensor_channel.shape[0])
    with netcdf_file(path, "w", version=1) as f:
        f.Release = np.int32(co.ODPS_RELEASE)
        f.Version = np.int32(1)
        f.Sensor_Id = tc.sensor_id
        f.Algorithm = np.int32(2)
        f.WMO_Satellite_Id = np.int32(tc.wmo_satellite_id)
        f.WMO_Sensor_Id = np.int32(tc.wmo_sensor_id)
        f.createDimension("n_Layers", K)
        f.createDimension("n_Levels", K + 1)
        f.createDimension("n_Components", J)
        f.createDimension("n_Absorbers", Jm)
        f.createDimension("n_Channels", L)
        f.createDimension("n_Coeffs", max(int(tc.c.shape[0]), 1))
        for name, val in (("Group_Index", tc.group_index), ("Sensor_Type", tc.sensor_type)):
            v = f.createVariable(name, "i4", ())
            v[...] = np.int32(val)
        spec = [("Ref_Level_Pressure", "f8", ("n_Levels",), tc.ref_level_pressure),
                ("Ref_Pressure", "f8", ("n_Layers",), tc.ref_pressure),
                ("Ref_Temperature", "f8", ("n_Layers",), tc.ref_temperature),
                ("Ref_Absorber", "f8", ("n_Absorbers", "n_Layers"), np.asarray(tc.ref_absorber).T),
                ("Min_Absorber", "f8", ("n_Absorbers", "n_Layers"), np.asarray(tc.min_absorber).T),
                ("Max_Absorber", "f8", ("n_Absorbers", "n_Layers"), np.asarray(tc.max_absorber).T),
                ("Sensor_Channel", "i4", ("n_Channels",), tc.sensor_channel),
                ("Component_ID", "i4", ("n_Components",), tc.component_id),
                ("Absorber_ID", "i4", ("n_Absorbers",), tc.absorber_id),
                ("n_Predictors", "i4", ("n_Channels", "n_Components"), np.asarray(tc.n_predictors).T),
                ("Pos_Index", "i4", ("n_Channels", "n_Components"), np.asarray(tc.pos_index).T),
                ("ODPS_Coefficients", "f4", ("n_Coeffs",),
                 tc.c if tc.c.shape[0] else np.zeros(1, np.float32))]
        o = tc.optran
        if o is not None and o.oc.size > 0:
            f.createDimension("n_OPIndex", co.N_PREDICTOR_USED_OPTRAN + 1)
            f.createDimension("n_OCoeffs", int(o.oc.size))
            for name, val, t in (("Alpha", o.alpha, "f8"), ("Alpha_C1", o.alpha_c1, "f8"),
                                 ("Alpha_C2", o.alpha_c2, "f8"), ("OComponent_Index", o.component_index, "i4")):
                v = f.createVariable(name, t, ())
                v[...] = np.asarray(val).astype(t)
            spec += [("OSignificance", "i4", ("n_Channels",), o.significance),
                     ("Order", "i4", ("n_Channels",), o.order),
                     ("OP_Index", "i4", ("n_Channels", "n_OPIndex"), np.asarray(o.op_index).T),
                     ("OPos_Index", "i4", ("n_Channels",), o.opos_index),
                     ("OC", "f8", ("n_OCoeffs",), o.oc)]
        for name, t, dims, data in spec:
            v = f.createVariable(name, t, dims)
            v[:] = np.asarray(data).astype(t)


def read_odps_nc(path: str) -> co.ODPSCoeff:
    with netcdf_file(path, "r", mmap=False) as f:
        optran = None
        if "n_OCoeffs" in f.dimensions and int(f.dimensions["n_OCoeffs"] or 0) > 0:
            for name in ("OSignificance", "Order", "OP_Index", "OPos_Index", "OC", "Alpha", "Alpha_C1",
                         "Alpha_C2", "OComponent_Index"):
                if name not in f.variables:
                    raise ValueError(f"{path}: OPTRAN variable {name} missing")
            optran = co.OPTRANCoeff(
                significance=_var(f, "OSignificance", np.int32), order=_var(f, "Order", np.int32),
                op_index=_var(f, "OP_Index", np.int32).T.copy(), opos_index=_var(f, "OPos_Index", np.int32),
                oc=_var(f, "OC", np.float64), alpha=float(f.variables["Alpha"].data[()]),
                alpha_c1=float(f.variables["Alpha_C1"].data[()]), alpha_c2=float(f.variables["Alpha_C2"].data[()]),
                component_index=int(f.variables["OComponent_Index"].data[()]))
        group = int(f.variables["Group_Index"].data[()])
        if group not in N_COMPONENTS_G:
            raise ValueError(f"{path}: unknown ODPS group index {group}")
        n_pred = _var(f, "n_Predictors", np.int32).T.copy()
        pos = _var(f, "Pos_Index", np.int32).T.copy()
        # a file without coefficients still has a one-element placeholder
        c = _var(f, "ODPS_Coefficients", np.float32) if n_pred.sum() > 0 else np.zeros(0, np.float32)
        if n_pred.shape[0] != N_COMPONENTS_G[group]:
            raise ValueError(f"{path}: {n_pred.shape[0]} components for group {group}")
        return co.ODPSCoeff(
            group_index=group, sensor_id=str(_attr(f, "Sensor_Id", "")),
            sensor_type=int(f.variables["Sensor_Type"].data[()]),
            sensor_channel=_var(f, "Sensor_Channel", np.int32),
            ref_level_pressure=_var(f, "Ref_Level_Pressure", np.float64),
            ref_pressure=_var(f, "Ref_Pressure", np.float64),
            ref_temperature=_var(f, "Ref_Temperature", np.float64),
            ref_absorber=_var(f, "Ref_Absorber", np.float64).T.copy(),
            min_absorber=_var(f, "Min_Absorber", np.float64).T.copy(),
            max_absorber=_var(f, "Max_Absorber", np.float64).T.copy(),
            n_predictors=n_pred, pos_index=pos, c=c,
            wmo_satellite_id=int(_attr(f, "WMO_Satellite_Id", 1023)),
            wmo_sensor_id=int(_attr(f, "WMO_Sensor_Id", 2047)), optran=optran)


# ---------------------------------------------------------------------------
# IRwaterCoeff (IR sea-surface emissivity table)
# ---------------------------------------------------------------------------

IRWATER_FILE = "Nalli.IRwater.EmisCoeff"


def write_irwater_nc(path: str, wc: co.IRwaterCoeff) -> None:
    """IRwaterCoeff_netCDF_IO's layout (src/Coefficients/EmisCoeff/IR_Water/
    IRwaterCoeff_netCDF_IO.f90:62-121, :1262-1338): the four axes and
    Emissivity(n_Angles, n_Frequencies, n_Wind_Speeds, n_Temperature),
    stored as (n_Temperature, n_Wind_Speeds, n_Frequencies, n_Angles)."""
    with netcdf_file(path, "w", version=1) as f:
        f.Release = np.int32(1)
        f.Version = np.int32(wc.version)
        f.Classification_Name = wc.classification
        for dim, name, data in (("n_Angles", "Angle", wc.angle), ("n_Frequencies", "Frequency", wc.frequency),
                                ("n_Wind_Speeds", "Wind_Speed", wc.wind_speed),
                                ("n_Temperature", "Temperature", wc.temperature)):
            f.createDimension(dim, int(np.asarray(data).shape[0]))
            v = f.createVariable(name, "f8", (dim,))
            v[:] = np.asarray(data, np.float64)
        v = f.createVariable("Emissivity", "f8", ("n_Temperature", "n_Wind_Speeds", "n_Frequencies", "n_Angles"))
        v[:] = np.asarray(wc.emissivity, np.float64).transpose(3, 2, 1, 0)


def read_irwater_nc(path: str) -> co.IRwaterCoeff:
    with netcdf_file(path, "r", mmap=False) as f:
        return co.IRwaterCoeff(
            classification=str(_attr(f, "Classification_Name", "")),
            angle=_var(f, "Angle", np.float64), frequency=_var(f, "Frequency", np.float64),
            wind_speed=_var(f, "Wind_Speed", np.float64), temperature=_var(f, "Temperature", np.float64),
            emissivity=np.ascontiguousarray(_var(f, "Emissivity", np.float64).transpose(3, 2, 1, 0)),
            version=int(_attr(f, "Version", 2)))


# ---------------------------------------------------------------------------
# CloudCoeff (cloud optical property table)
# ---------------------------------------------------------------------------

CLOUDCOEFF_FILE = "CloudCoeff"


def _nc_order(a):
    """A Fortran-ordered array as netCDF stores it: the dimensions reversed."""
    a = np.asarray(a, np.float64)
    return a.transpose(tuple(range(a.ndim))[::-1])


def write_cloudcoeff_nc(path: str, cc: co.CloudCoeff) -> None:
    """CloudCoeff_netCDF_IO's layout (src/Coefficients/CloudCoeff/
    CloudCoeff_netCDF_IO.f90:60-103 names, :229-253 types, :2020-2545
    definitions).  Its dimensions for a table read from the binary file:
    n_IR_Densities is the IR density axis (the MW densities and the liquid
    entry), n_Legendre_Terms counts the terms 0..n_Legendre_Terms of the MW
    phase coefficients.  pcoeff_IR is 4-D (no phase dimension, :2533-2537)
    and holds the IR terms 1..n_Legendre_Terms in its first
    n_Legendre_Terms slabs, the last slab zero, which is how the reference's
    writer fills that variable from its array.  The kb variables are written
    as zero and Water_Density_MW as zero (a table indexed by effective
    radius, :1362-1372); Density_IR is 100 followed by the MW densities (the
    reader's fallback, :1578-1586).  None of these three enters the binary
    file."""
    nfm, nrm, nt = cc.ke_l_mw.shape
    nfi, nri, ndi = cc.ke_ir.shape
    nd, nl, nph = cc.density_mw.size, cc.n_legendre_terms, cc.n_phase_elements
    if nph != 1:
        raise ValueError("CloudCoeff netCDF: pcoeff_IR has no phase dimension; n_Phase_Elements must be 1")
    if ndi != nd + 1 or cc.pcoeff_ir.shape[3] != nl:
        raise ValueError("CloudCoeff: IR tables do not match the density and Legendre axes")
    with netcdf_file(path, "w", version=1) as f:
        f.Release = np.int32(co.CLOUDCOEFF_RELEASE)
        f.Version = np.int32(cc.version)
        for dim, n in (("n_MW_Frequencies", nfm), ("n_MW_Radii", nrm), ("n_IR_Frequencies", nfi),
                       ("n_IR_Radii", nri), ("n_Temperatures", nt), ("n_MW_Densities", nd),
                       ("n_IR_Densities", nd + 1), ("n_Legendre_Terms", nl + 1), ("n_Phase_Elements", nph)):
            f.createDimension(dim, int(n))
        axes = (("Frequency_MW", "n_MW_Frequencies", cc.frequency_mw),
                ("Frequency_IR", "n_IR_Frequencies", cc.frequency_ir),
                ("Water_Density_MW", "n_MW_Radii", np.zeros(nrm)),
                ("Reff_MW", "n_MW_Radii", cc.reff_mw), ("Reff_IR", "n_IR_Radii", cc.reff_ir),
                ("Temperature", "n_Temperatures", cc.temperature),
                ("Density_MW", "n_MW_Densities", cc.density_mw),
                ("Density_IR", "n_IR_Densities", np.concatenate([[100.0], cc.density_mw])))
        for name, dim, data in axes:
            v = f.createVariable(name, "f8", (dim,))
            v[:] = np.asarray(data, np.float64)
        blocks = (("L_MW", ("n_Temperatures", "n_MW_Radii", "n_MW_Frequencies"),
                   (cc.ke_l_mw, cc.w_l_mw, cc.g_l_mw, cc.pcoeff_l_mw)),
                  ("S_MW", ("n_MW_Densities", "n_MW_Radii", "n_MW_Frequencies"),
                   (cc.ke_s_mw, cc.w_s_mw, cc.g_s_mw, cc.pcoeff_s_mw)),
                  ("IR", ("n_IR_Densities", "n_IR_Radii", "n_IR_Frequencies"),
                   (cc.ke_ir, cc.w_ir, cc.g_ir, None)))
        for suffix, dims, (ke, w, g, pc) in blocks:
            for name, data in (("ke", ke), ("w", w), ("g", g), ("kb", np.zeros_like(ke))):
                v = f.createVariable(f"{name}_{suffix}", "f8", dims)
                v[:] = _nc_order(data)
            if pc is not None:
                v = f.createVariable(f"pcoeff_{suffix}", "f8", ("n_Phase_Elements", "n_Legendre_Terms") + dims)
                v[:] = _nc_order(pc)
        pir = np.zeros((nfi, nri, ndi, nl + 1))
        pir[..., :nl] = cc.pcoeff_ir[..., 0]
        v = f.createVariable("pcoeff_IR", "f8", ("n_Legendre_Terms",) + blocks[2][1])
        v[:] = _nc_order(pir)


def read_cloudcoeff_nc(path: str) -> co.CloudCoeff:
    with netcdf_file(path, "r", mmap=False) as f:
        rel = int(_attr(f, "Release", co.CLOUDCOEFF_RELEASE))
        if rel != co.CLOUDCOEFF_RELEASE:
            raise ValueError(f"CloudCoeff netCDF: release {rel} not supported")
        nl = int(f.dimensions["n_Legendre_Terms"]) - 1

        def fortran(name):
            a = _var(f, name, np.float64)
            return np.ascontiguousarray(a.transpose(tuple(range(a.ndim))[::-1]))
        axes = [_var(f, n, np.float64) for n in ("Frequency_MW", "Frequency_IR", "Reff_MW", "Reff_IR",
                                                 "Temperature", "Density_MW")]
        tables = []
        for suffix in ("L_MW", "S_MW"):
            tables += [fortran(f"{n}_{suffix}") for n in ("ke", "w", "g", "pcoeff")]
        pir = fortran("pcoeff_IR")
        if pir.ndim != 4:
            raise ValueError("CloudCoeff netCDF: pcoeff_IR must have four dimensions")
        tables += [fortran(f"{n}_IR") for n in ("ke", "w", "g")]
        tables.append(np.ascontiguousarray(pir[..., :nl, None]))
        return co.CloudCoeff(*axes, *tables, version=int(_attr(f, "Version", co.MIE_TAMU_CLOUDCOEFF)))


# ---------------------------------------------------------------------------
# AerosolCoeff (aerosol optical property table)
# ---------------------------------------------------------------------------

AEROSOLCOEFF_FILE = "AerosolCoeff"


def write_aerosolcoeff_nc(path: str, ac: co.AerosolCoeff, scheme: str = "CRTM") -> None:
    """AerosolCoeff_netCDF_IO's layout (src/Coefficients/AerosolCoeff/
    AerosolCoeff_netCDF_IO.f90:67-95 names, :152-162 types, :1540-1830
    definitions): dimension n_RH for the tables' humidity axis and, for the
    'CRTM' and 'CMAQ' tables, n_RH_Radii for the RH variable (:1728-1736);
    n_Legendre_Terms counts the terms 0..n_Legendre_Terms; the type names are
    characters over the tnsl dimension."""
    nw, nrh, nr, ns, nt = ac.ke.shape
    nl, nph = ac.pcoeff.shape[5] - 1, ac.pcoeff.shape[6]
    rh_radii = co._rh_radii_record(scheme)
    if not rh_radii and ac.rh.size != nrh:
        raise ValueError("the RH axis of a GOCART-GEOS5 / NAAPS table has n_RH entries")
    with netcdf_file(path, "w", version=1) as f:
        f.Release = np.int32(co.AEROSOLCOEFF_RELEASE)
        f.Version = np.int32(ac.version)
        f.Data_Source = ac.data_source
        for dim, n in (("n_Wavelengths", nw), ("n_Radii", nr), ("n_Sigma", ns), ("n_Types", nt), ("n_RH", nrh)):
            f.createDimension(dim, int(n))
        if rh_radii:
            f.createDimension("n_RH_Radii", int(ac.rh.size))
        f.createDimension("n_Legendre_Terms", nl + 1)
        f.createDimension("n_Phase_Elements", nph)
        f.createDimension("tnsl", co.AEROSOL_SL)
        v = f.createVariable("Aerosol_Type", "i4", ("n_Types",))
        v[:] = np.asarray(ac.type_id, np.int32)
        v = f.createVariable("Aerosol_Type_Name", "c", ("n_Types", "tnsl"))
        v[:] = np.array([list(n.ljust(co.AEROSOL_SL)[:co.AEROSOL_SL]) for n in ac.type_name], "S1")
        for name, dims, data in (("Wavelength", ("n_Wavelengths",), ac.wavelength),
                                 ("Reff", ("n_Types", "n_Radii"), ac.reff),
                                 ("Rsig", ("n_Types", "n_Sigma"), ac.rsig),
                                 ("RH", ("n_RH_Radii" if rh_radii else "n_RH",), ac.rh)):
            v = f.createVariable(name, "f8", dims)
            v[:] = _nc_order(data)
        dims5 = ("n_Types", "n_Sigma", "n_Radii", "n_RH", "n_Wavelengths")
        for name, data in (("ke", ac.ke), ("w", ac.w), ("g", ac.g)):
            v = f.createVariable(name, "f8", dims5)
            v[:] = _nc_order(data)
        v = f.createVariable("pcoeff", "f8", ("n_Phase_Elements", "n_Legendre_Terms") + dims5)
        v[:] = _nc_order(ac.pcoeff)


def read_aerosolcoeff_nc(path: str, scheme: str = "CRTM") -> co.AerosolCoeff:
    rh_radii = co._rh_radii_record(scheme)
    with netcdf_file(path, "r", mmap=False) as f:
        rel = int(_attr(f, "Release", co.AEROSOLCOEFF_RELEASE))
        if rel != co.AEROSOLCOEFF_RELEASE:
            raise ValueError(f"AerosolCoeff netCDF: release {rel} not supported")
        if rh_radii != ("n_RH_Radii" in f.dimensions):
            raise ValueError(f"AerosolCoeff netCDF: the n_RH_Radii dimension does not fit the {scheme!r} scheme")

        def fortran(name, dtype=np.float64):
            a = _var(f, name, dtype)
            return np.ascontiguousarray(a.transpose(tuple(range(a.ndim))[::-1]))
        names = [b"".join(row).decode("ascii", "replace").rstrip()
                 for row in np.asarray(f.variables["Aerosol_Type_Name"].data)]
        return co.AerosolCoeff(
            type_id=_var(f, "Aerosol_Type", np.int32), type_name=names,
            wavelength=_var(f, "Wavelength", np.float64), reff=fortran("Reff"), rsig=fortran("Rsig"),
            rh=_var(f, "RH", np.float64), ke=fortran("ke"), w=fortran("w"), g=fortran("g"),
            pcoeff=fortran("pcoeff"), data_source=str(_attr(f, "Data_Source", "")),
            version=int(_attr(f, "Version", 1)))


# ---------------------------------------------------------------------------
# conversion for CRTM_Init
# ---------------------------------------------------------------------------

def convert_sensor(src_dir: str, sensor_id: str, out_dir: str, spc_format: str = "Binary",
                   tau_format: str = "Binary") -> None:
    """Put <sensor_id>.SpcCoeff.bin and .TauCoeff.bin into out_dir: converted
    from the .nc files of src_dir for the formats given as 'netCDF', linked
    to src_dir's binary files otherwise."""
    for kind, fmt, read, write in (("SpcCoeff", spc_format, read_spccoeff_nc, co.write_spccoeff),
                                   ("TauCoeff", tau_format, read_odps_nc, co.write_odps)):
        dst = os.path.join(out_dir, f"{sensor_id}.{kind}.bin")
        if fmt.lower() == "netcdf":
            write(dst, read(os.path.join(src_dir, f"{sensor_id}.{kind}.nc")))
        elif fmt.lower() == "binary":
            _link(os.path.join(src_dir, f"{sensor_id}.{kind}.bin"), dst)
        else:
            raise ValueError(f"{kind}_Format must be 'Binary' or 'netCDF' (got {fmt!r})")


def convert_irwater(src_dir: str, out_dir: str, nc_file: str = IRWATER_FILE + ".nc") -> None:
    """The netCDF IRwaterCoeff file of src_dir (Nalli.IRwater.EmisCoeff.nc by
    default) as Nalli.IRwater.EmisCoeff.bin in out_dir."""
    co.write_irwatercoeff(os.path.join(out_dir, IRWATER_FILE + ".bin"),
                          read_irwater_nc(os.path.join(src_dir, nc_file)))


def convert_cloud(src_dir: str, out_dir: str, nc_file: str = CLOUDCOEFF_FILE + ".nc") -> None:
    """The netCDF CloudCoeff file of src_dir as CloudCoeff.bin in out_dir."""
    co.write_cloudcoeff(os.path.join(out_dir, CLOUDCOEFF_FILE + ".bin"),
                        read_cloudcoeff_nc(os.path.join(src_dir, nc_file)))


def convert_aerosol(src_dir: str, out_dir: str, scheme: str = "CRTM",
                    nc_file: str = AEROSOLCOEFF_FILE + ".nc") -> str:
    """The netCDF AerosolCoeff file of src_dir, for the aerosol scheme, as
    AerosolCoeff.bin in out_dir; returns that file's name."""
    name = AEROSOLCOEFF_FILE + ".bin"
    co.write_aerosolcoeff(os.path.join(out_dir, name),
                          read_aerosolcoeff_nc(os.path.join(src_dir, nc_file), scheme), scheme=scheme)
    return name


SHARED_FILES = ("CloudCoeff.bin", "AerosolCoeff.bin", "AerosolCoeff.CMAQ.bin", "AerosolCoeff.GOCART-GEOS5.bin",
                "AerosolCoeff.NAAPS.bin", IRWATER_FILE + ".bin")


def link_shared_files(src_dir: str, out_dir: str, names=SHARED_FILES, extra=()) -> None:
    """The coefficient files shared by all sensors, as src_dir has them."""
    for n in tuple(names) + tuple(extra):
        p = os.path.join(src_dir, n)
        if os.path.exists(p) and not os.path.exists(os.path.join(out_dir, n)):
            _link(p, os.path.join(out_dir, n))


def _link(src: str, dst: str) -> None:
    if not os.path.exists(src):
        raise FileNotFoundError(src)
    try:
        os.symlink(os.path.abspath(src), dst)
    except OSError:
        shutil.copyfile(src, dst)
