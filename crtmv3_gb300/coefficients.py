"""ODPS TauCoeff and SpcCoeff tables: in-memory form and binary file I/O.

The record order follows the reference writers so that files made here have
the reference's on-disk layout:

* ODPS TauCoeff: ``src/Coefficients/TauCoeff/ODPS/ODPS_Binary_IO.f90:1042-1180``
  (Release/Version, Algorithm, dimensions, Group_Index, sensor ids, channel
  list, component ids, absorber ids, reference profile, n_Predictors/Pos_Index,
  C as REAL(Single)).  The coefficient index of channel ``l``, component ``j``,
  predictor ``i`` and layer ``k`` is ``Pos_Index(j,l) + (i-1)*n_Layers + k - 1``
  (1-based; ``ODPS_AtmAbsorption.f90:198-204``).
* SpcCoeff (Release 8, Version 3 with PolAngle):
  ``src/Coefficients/SpcCoeff/SpcCoeff_Binary_IO.f90:660-711``.
"""
from __future__ import annotations

import dataclasses
from typing import Optional

import numpy as np

from .fortran_io import RecordReader, RecordWriter

# Sensor types (``ODPS_Define.f90:90-95``)
MICROWAVE_SENSOR = 1
INFRARED_SENSOR = 2
VISIBLE_SENSOR = 3
ULTRAVIOLET_SENSOR = 4

ODPS_ALGORITHM = 2          # ``src/CRTM_Parameters.f90:128``
ODPS_RELEASE = 2            # ``ODPS_Define.f90:79``
ODPS_VERSION = 1
SPCCOEFF_RELEASE = 8        # ``SpcCoeff_Define.f90:152``
SPCCOEFF_VERSION = 3
SL = 20                     # sensor id length

# Predictor groups (``ODPS_Predictor.f90:85-116``)
N_COMPONENTS_G = {1: 8, 2: 5, 3: 2}
N_ABSORBERS_G = {1: 6, 2: 3, 3: 1}
N_PREDICTORS_G = {
    1: (7, 18, 7, 11, 11, 14, 10, 11),
    2: (7, 15, 7, 11, 10),
    3: (7, 14),
}
COMPONENT_ID_G = {
    1: (7, 101, 15, 114, 121, 120, 119, 118),
    2: (20, 101, 15, 114, 121),
    3: (113, 12),
}
# HITRAN absorber ids per group, in the order the predictor code indexes them
ABSORBER_ID_G = {1: (1, 3, 2, 4, 5, 6), 2: (1, 3, 2), 3: (1,)}

H2O_ID, CO2_ID, O3_ID, N2O_ID, CO_ID, CH4_ID = 1, 2, 3, 4, 5, 6
MASS_MIXING_RATIO_UNITS = 3     # g/kg
VOLUME_MIXING_RATIO_UNITS = 1   # ppmv


# Compact-OPTRAN water-vapour-line term of an ODPS file (ODPS_Define.f90:103,
# 186-203): predictors used per channel, polynomial order, channel flag value
N_PREDICTOR_USED_OPTRAN = 6
MAX_OPTRAN_ORDER = 10
MAX_OPTRAN_PREDICTORS = 14
SIGNIFICANCE_OPTRAN = 1


@dataclasses.dataclass
class OPTRANCoeff:
    """The compact-OPTRAN part of an ODPS TauCoeff (``ODPS_Define.f90:186-203``):
    per channel the flag OSignificance (1: the OComponent_Index component of
    that channel is computed by OPTRAN), the polynomial Order, OP_Index
    (OP_Index[0, l] the predictor count, then the predictor numbers 1-14;
    Fortran index order, as the file's OP_Index(0:6, L)) and OPos_Index
    (1-based start in OC); the coefficients OC and the absorber transform
    Alpha, Alpha_C1, Alpha_C2."""
    significance: np.ndarray        # (L,) int32
    order: np.ndarray               # (L,) int32
    op_index: np.ndarray            # (N_PREDICTOR_USED_OPTRAN + 1, L) int32
    opos_index: np.ndarray          # (L,) int32, 1-based
    oc: np.ndarray                  # (n_OCoeffs,) float64
    alpha: float
    alpha_c1: float
    alpha_c2: float
    component_index: int            # 1-based component the term replaces


@dataclasses.dataclass
class ODPSCoeff:
    """The ODPS TauCoeff structure (``ODPS_Define.f90:110-203``)."""
    group_index: int
    sensor_id: str
    sensor_type: int
    sensor_channel: np.ndarray          # (L,) int32
    ref_level_pressure: np.ndarray      # (K+1,) hPa
    ref_pressure: np.ndarray            # (K,)
    ref_temperature: np.ndarray         # (K,)
    ref_absorber: np.ndarray            # (K, Jm)
    min_absorber: np.ndarray            # (K, Jm)
    max_absorber: np.ndarray            # (K, Jm)
    n_predictors: np.ndarray            # (J, L) int32
    pos_index: np.ndarray               # (J, L) int32, 1-based
    c: np.ndarray                       # (n_Coeffs,) float32
    wmo_satellite_id: int = 1023
    wmo_sensor_id: int = 2047
    optran: Optional[OPTRANCoeff] = None

    @property
    def n_layers(self) -> int:
        return int(self.ref_pressure.shape[0])

    @property
    def n_components(self) -> int:
        return N_COMPONENTS_G[self.group_index]

    @property
    def n_absorbers(self) -> int:
        return N_ABSORBERS_G[self.group_index]

    @property
    def n_channels(self) -> int:
        return int(self.sensor_channel.shape[0])

    @property
    def component_id(self) -> np.ndarray:
        return np.asarray(COMPONENT_ID_G[self.group_index], dtype=np.int32)

    @property
    def absorber_id(self) -> np.ndarray:
        return np.asarray(ABSORBER_ID_G[self.group_index], dtype=np.int32)

    def coeff_block(self, j: int, l: int) -> np.ndarray:
        """Coefficients of component ``j`` and channel ``l`` (0-based) as (np, K)."""
        npred = int(self.n_predictors[j, l])
        if npred <= 0:
            return np.zeros((0, self.n_layers), np.float32)
        p0 = int(self.pos_index[j, l]) - 1
        return self.c[p0:p0 + npred * self.n_layers].reshape(npred, self.n_layers)


def write_odps(path: str, tc: ODPSCoeff, byteorder: str = "<") -> None:
    K, J, Jm, L = tc.n_layers, tc.n_components, tc.n_absorbers, tc.n_channels
    with open(path, "wb") as f:
        w = RecordWriter(f, byteorder)
        w.record(np.array([ODPS_RELEASE, ODPS_VERSION], np.int32))
        w.record(np.array([ODPS_ALGORITHM], np.int32))
        n_oc = 0 if tc.optran is None else int(tc.optran.oc.size)
        w.record(np.array([K, J, Jm, L, tc.c.size, N_PREDICTOR_USED_OPTRAN, n_oc], np.int32))
        w.record(np.array([tc.group_index], np.int32))
        w.record(tc.sensor_id.ljust(SL)[:SL].encode("ascii"),
                 np.array([tc.wmo_satellite_id, tc.wmo_sensor_id, tc.sensor_type], np.int32))
        w.record(tc.sensor_channel.astype(np.int32))
        w.record(tc.component_id)
        w.record(tc.absorber_id)
        w.record(tc.ref_level_pressure.astype(np.float64), tc.ref_pressure.astype(np.float64),
                 tc.ref_temperature.astype(np.float64), tc.ref_absorber.astype(np.float64),
                 tc.min_absorber.astype(np.float64), tc.max_absorber.astype(np.float64))
        w.record(tc.n_predictors.astype(np.int32), tc.pos_index.astype(np.int32))
        if tc.c.size > 0:
            w.record(tc.c.astype(np.float32))
        if n_oc > 0:   # ODPS_Binary_IO.f90:1173-1180
            o = tc.optran
            w.record(o.significance.astype(np.int32), o.order.astype(np.int32),
                     o.op_index.astype(np.int32), o.opos_index.astype(np.int32),
                     o.oc.astype(np.float64), np.array([o.alpha, o.alpha_c1, o.alpha_c2], np.float64),
                     np.array([o.component_index], np.int32))


def read_odps(path: str) -> ODPSCoeff:
    with open(path, "rb") as f:
        r = RecordReader(f)
        release, version = r.split(r.record(), [("i4", (2,))])[0]
        if release != ODPS_RELEASE:
            raise IOError(f"ODPS release {release} not supported")
        (alg,) = r.split(r.record(), [("i4", ())])
        if alg != ODPS_ALGORITHM:
            raise IOError(f"TauCoeff algorithm {alg} is not ODPS")
        dims = r.split(r.record(), [("i4", (7,))])[0]
        K, J, Jm, L, n_coeffs, _n_opindex, n_ocoeffs = (int(x) for x in dims)
        (group,) = r.split(r.record(), [("i4", ())])
        sid, ids = r.split(r.record(), [("S", SL), ("i4", (3,))])
        chans = r.split(r.record(), [("i4", (L,))])[0]
        r.record()  # component ids (fixed by group)
        r.record()  # absorber ids (fixed by group)
        lev, lay, temp, ra, mn, mx = r.split(r.record(), [
            ("f8", (K + 1,)), ("f8", (K,)), ("f8", (K,)),
            ("f8", (K, Jm)), ("f8", (K, Jm)), ("f8", (K, Jm))])
        npred, pos = r.split(r.record(), [("i4", (J, L)), ("i4", (J, L))])
        c = np.zeros(0, np.float32)
        if n_coeffs > 0:
            c = r.split(r.record(), [("f4", (n_coeffs,))])[0]
        optran = None
        if n_ocoeffs > 0:   # ODPS_Binary_IO.f90:778-800
            nu = N_PREDICTOR_USED_OPTRAN + 1
            sig, order, opi, opos, oc, alph, ocomp = r.split(r.record(), [
                ("i4", (L,)), ("i4", (L,)), ("i4", (nu, L)), ("i4", (L,)), ("f8", (n_ocoeffs,)),
                ("f8", (3,)), ("i4", ())])
            optran = OPTRANCoeff(sig, order, opi, opos, oc, float(alph[0]), float(alph[1]), float(alph[2]),
                                 int(ocomp))
    return ODPSCoeff(int(group), sid, int(ids[2]), chans, lev, lay, temp, ra, mn, mx,
                     npred, pos, c, int(ids[0]), int(ids[1]), optran)


@dataclasses.dataclass
class SpcCoeff:
    """Spectral coefficients (``SpcCoeff_Define.f90:160-200``)."""
    sensor_id: str
    sensor_type: int
    sensor_channel: np.ndarray
    frequency: np.ndarray
    wavenumber: np.ndarray
    planck_c1: np.ndarray
    planck_c2: np.ndarray
    band_c1: np.ndarray
    band_c2: np.ndarray
    cosmic_background_radiance: np.ndarray
    solar_irradiance: np.ndarray
    polarization: Optional[np.ndarray] = None
    pol_angle: Optional[np.ndarray] = None
    channel_flag: Optional[np.ndarray] = None
    wmo_satellite_id: int = 1023
    wmo_sensor_id: int = 2047

    @property
    def n_channels(self) -> int:
        return int(self.sensor_channel.shape[0])


def write_spccoeff(path: str, sc: SpcCoeff, byteorder: str = "<") -> None:
    L = sc.n_channels
    pol = sc.polarization if sc.polarization is not None else np.zeros(L, np.int32)
    pang = sc.pol_angle if sc.pol_angle is not None else np.zeros(L)
    flag = sc.channel_flag if sc.channel_flag is not None else np.zeros(L, np.int32)
    with open(path, "wb") as f:
        w = RecordWriter(f, byteorder)
        w.record(np.array([SPCCOEFF_RELEASE, SPCCOEFF_VERSION], np.int32))
        w.record(np.array([L], np.int32))
        w.record(sc.sensor_id.ljust(SL)[:SL].encode("ascii"),
                 np.array([sc.sensor_type, sc.wmo_satellite_id, sc.wmo_sensor_id], np.int32))
        w.record(sc.sensor_channel.astype(np.int32), pol.astype(np.int32), pang.astype(np.float64),
                 flag.astype(np.int32), sc.frequency, sc.wavenumber, sc.planck_c1, sc.planck_c2,
                 sc.band_c1, sc.band_c2, sc.cosmic_background_radiance, sc.solar_irradiance)
        w.record(np.array([0], np.int32))  # antenna correction data absent
        w.record(np.array([0], np.int32))  # NLTE correction data absent


def read_spccoeff(path: str) -> SpcCoeff:
    with open(path, "rb") as f:
        r = RecordReader(f)
        release, version = r.split(r.record(), [("i4", (2,))])[0]
        if release != SPCCOEFF_RELEASE or version < 3:
            raise IOError(f"SpcCoeff release/version {release}/{version} not supported")
        (L,) = r.split(r.record(), [("i4", ())])
        L = int(L)
        sid, ids = r.split(r.record(), [("S", SL), ("i4", (3,))])
        fields = r.split(r.record(), [("i4", (L,)), ("i4", (L,)), ("f8", (L,)), ("i4", (L,))]
                         + [("f8", (L,))] * 8)
    ch, pol, pang, flag, freq, wn, c1, c2, b1, b2, cb, si = fields
    return SpcCoeff(sid, int(ids[0]), ch, freq, wn, c1, c2, b1, b2, cb, si, pol, pang, flag,
                    int(ids[1]), int(ids[2]))


# ---------------------------------------------------------------------------
# CloudCoeff (cloud optical property LUT)
# ---------------------------------------------------------------------------

CLOUDCOEFF_RELEASE = 3          # ``CloudCoeff_Define.f90:72``
MIE_TAMU_CLOUDCOEFF = 1         # Version of a LUT indexed by effective radius

# Cloud types (``src/Atmosphere/Cloud/CRTM_Cloud_Define.f90:150-155``)
WATER_CLOUD, ICE_CLOUD, RAIN_CLOUD, SNOW_CLOUD, GRAUPEL_CLOUD, HAIL_CLOUD = 1, 2, 3, 4, 5, 6


@dataclasses.dataclass
class CloudCoeff:
    """Cloud optical property LUT (``CloudCoeff_Define.f90:87-131``).

    Arrays are shaped in the reference's Fortran index order (first index
    fastest on disk): ``ke_l_mw[f, r, t]``, ``pcoeff_l_mw[f, r, t, l, m]`` with
    l = 0..n_legendre_terms, ``ke_s_mw[f, r, d]``, ``ke_ir[f, r, d]`` with
    d = 1..n_mw_densities+1 and ``pcoeff_ir[f, r, d, l, m]`` with
    l = 1..n_legendre_terms.
    """
    frequency_mw: np.ndarray      # GHz
    frequency_ir: np.ndarray      # cm^-1
    reff_mw: np.ndarray           # microns
    reff_ir: np.ndarray
    temperature: np.ndarray       # K
    density_mw: np.ndarray
    ke_l_mw: np.ndarray
    w_l_mw: np.ndarray
    g_l_mw: np.ndarray
    pcoeff_l_mw: np.ndarray
    ke_s_mw: np.ndarray
    w_s_mw: np.ndarray
    g_s_mw: np.ndarray
    pcoeff_s_mw: np.ndarray
    ke_ir: np.ndarray
    w_ir: np.ndarray
    g_ir: np.ndarray
    pcoeff_ir: np.ndarray
    version: int = MIE_TAMU_CLOUDCOEFF

    @property
    def n_legendre_terms(self) -> int:
        return int(self.pcoeff_l_mw.shape[3]) - 1

    @property
    def n_phase_elements(self) -> int:
        return int(self.pcoeff_l_mw.shape[4])


def write_cloudcoeff(path: str, cc: CloudCoeff, byteorder: str = "<") -> None:
    """Record order of ``CloudCoeff_Binary_IO.f90:597-660`` (the kb arrays are
    not part of the binary file)."""
    with open(path, "wb") as f:
        w = RecordWriter(f, byteorder)
        w.record(np.array([CLOUDCOEFF_RELEASE, cc.version], np.int32))
        w.record(np.array([cc.frequency_mw.size, cc.reff_mw.size, cc.frequency_ir.size,
                           cc.reff_ir.size, cc.temperature.size, cc.density_mw.size,
                           cc.n_legendre_terms, cc.n_phase_elements], np.int32))
        w.record(cc.frequency_mw, cc.frequency_ir, cc.reff_mw, cc.reff_ir, cc.temperature,
                 cc.density_mw)
        w.record(cc.ke_l_mw, cc.w_l_mw, cc.g_l_mw, cc.pcoeff_l_mw)
        w.record(cc.ke_s_mw, cc.w_s_mw, cc.g_s_mw, cc.pcoeff_s_mw)
        w.record(cc.ke_ir, cc.w_ir, cc.g_ir, cc.pcoeff_ir)


def read_cloudcoeff(path: str) -> CloudCoeff:
    with open(path, "rb") as f:
        r = RecordReader(f)
        rel, ver = r.split(r.record(), [("i4", (2,))])[0]
        if rel != CLOUDCOEFF_RELEASE:
            raise IOError(f"CloudCoeff release {rel} not supported")
        dims = r.split(r.record(), [("i4", (8,))])[0]
        nfm, nrm, nfi, nri, nt, nd, nl, nph = (int(x) for x in dims)
        axes = r.split(r.record(), [("f8", (nfm,)), ("f8", (nfi,)), ("f8", (nrm,)),
                                    ("f8", (nri,)), ("f8", (nt,)), ("f8", (nd,))])

        def block(shape3, pshape):
            n3 = int(np.prod(shape3))
            parts = r.split(r.record(), [("f8", (n3,))] * 3 + [("f8", (int(np.prod(pshape)),))])
            return [p.reshape(shape3, order="F") for p in parts[:3]] + [parts[3].reshape(pshape, order="F")]
        lmw = block((nfm, nrm, nt), (nfm, nrm, nt, nl + 1, nph))
        smw = block((nfm, nrm, nd), (nfm, nrm, nd, nl + 1, nph))
        ir = block((nfi, nri, nd + 1), (nfi, nri, nd + 1, nl, nph))
    return CloudCoeff(*axes, *lmw, *smw, *ir, version=int(ver))


# ---------------------------------------------------------------------------
# AerosolCoeff (aerosol optical property LUT), schemes 'CRTM', 'CMAQ',
# 'GOCART-GEOS5', 'NAAPS'
# ---------------------------------------------------------------------------

AEROSOLCOEFF_RELEASE = 4        # ``AerosolCoeff_Define.f90:75``
AEROSOL_SL = 80                 # character length of the names (``AerosolCoeff_Define.f90:82``)


@dataclasses.dataclass
class AerosolCoeff:
    """Aerosol LUT (``AerosolCoeff_Define.f90:94-125``).  Arrays in the
    reference's Fortran index order: ``ke[w, rh, r, sigma, type]``,
    ``pcoeff[w, rh, r, sigma, type, l, m]`` with l = 0..n_legendre_terms;
    ``reff[r, type]``, ``rsig[sigma, type]``, ``rh[n_rh_radii]``.
    Wavelengths in microns; the reference converts them to frequencies
    10^4/wavelength (cm^-1), which must increase along the axis."""
    type_id: np.ndarray
    type_name: list
    wavelength: np.ndarray
    reff: np.ndarray
    rsig: np.ndarray
    rh: np.ndarray
    ke: np.ndarray
    w: np.ndarray
    g: np.ndarray
    pcoeff: np.ndarray
    data_source: str = "synthetic"
    version: int = 1


AEROSOL_SCHEMES = ("CRTM", "CMAQ", "GOCART-GEOS5", "NAAPS")


def _rh_radii_record(scheme: str) -> bool:
    """'CRTM' and 'CMAQ' files carry the n_RH_Radii record and an RH axis of
    that length; 'GOCART-GEOS5' / 'NAAPS' an RH axis of n_RH entries
    (``AerosolCoeff_Binary_IO.f90:421-424``, ``AerosolCoeff_Define.f90:342-354``)."""
    if scheme not in AEROSOL_SCHEMES:
        raise ValueError(f"unknown aerosol scheme {scheme!r}")
    return scheme in ("CRTM", "CMAQ")


def write_aerosolcoeff(path: str, ac: AerosolCoeff, byteorder: str = "<", scheme: str = "CRTM") -> None:
    """Record order of ``AerosolCoeff_Binary_IO.f90:396-530`` for a Version
    <= 300 file (no kb); the scheme decides the n_RH_Radii record."""
    nw, nrh, nr, ns, nt = ac.ke.shape
    nl = ac.pcoeff.shape[5] - 1
    if not _rh_radii_record(scheme) and ac.rh.size != nrh:
        raise ValueError("the RH axis of a GOCART-GEOS5 / NAAPS table has n_RH entries")
    with open(path, "wb") as f:
        wr = RecordWriter(f, byteorder)
        wr.record(np.array([AEROSOLCOEFF_RELEASE, ac.version], np.int32))
        wr.record(np.array([nw, nr, ns, nt, nrh, nl, ac.pcoeff.shape[6]], np.int32))
        if _rh_radii_record(scheme):
            wr.record(np.array([ac.rh.size], np.int32))
        wr.record(np.array([AEROSOL_SL], np.int32))
        wr.record(ac.data_source.ljust(AEROSOL_SL)[:AEROSOL_SL].encode("ascii"))
        wr.record(np.asarray(ac.type_id, np.int32))
        wr.record(np.array([AEROSOL_SL], np.int32))
        wr.record(b"".join(n.ljust(AEROSOL_SL)[:AEROSOL_SL].encode("ascii") for n in ac.type_name))
        wr.record(ac.wavelength, ac.reff, ac.rsig, ac.rh)
        wr.record(ac.ke, ac.w, ac.g, ac.pcoeff)


def read_aerosolcoeff(path: str, scheme: str = "CRTM") -> AerosolCoeff:
    with open(path, "rb") as f:
        r = RecordReader(f)
        rel, ver = r.split(r.record(), [("i4", (2,))])[0]
        if rel != AEROSOLCOEFF_RELEASE:
            raise IOError(f"AerosolCoeff release {rel} not supported")
        nw, nr, ns, nt, nrh, nl, nph = (int(x) for x in r.split(r.record(), [("i4", (7,))])[0])
        if _rh_radii_record(scheme):
            (nrr,) = r.split(r.record(), [("i4", ())])
        else:
            nrr = nrh
        r.record()
        src = r.split(r.record(), [("S", AEROSOL_SL)])[0]
        tid = r.split(r.record(), [("i4", (nt,))])[0]
        r.record()
        names = r.split(r.record(), [("S", AEROSOL_SL)] * nt)
        wl, reff, rsig, rh = r.split(r.record(), [("f8", (nw,)), ("f8", (nr, nt)), ("f8", (ns, nt)),
                                                  ("f8", (int(nrr),))])
        shp = (nw, nrh, nr, ns, nt)
        n5 = int(np.prod(shp))
        parts = r.split(r.record(), [("f8", (n5,))] * 3 + [("f8", (n5 * (nl + 1) * nph,))])
    return AerosolCoeff(tid, names, wl, reff, rsig, rh, *[p.reshape(shp, order="F") for p in parts[:3]],
                        parts[3].reshape(shp + (nl + 1, nph), order="F"), src, int(ver))


# ---------------------------------------------------------------------------
# IRwaterCoeff (IR sea-surface emissivity LUT, CRTM_IRSSEM)
# ---------------------------------------------------------------------------

IRWATERCOEFF_RELEASE = 4        # ``IRwaterCoeff_Define.f90:65``
IRWATER_SL = 80                 # Classification_Name length (``IRwaterCoeff_Define.f90:77``)


@dataclasses.dataclass
class IRwaterCoeff:
    """IR water emissivity table (``IRwaterCoeff_Define.f90:86-106``):
    ``emissivity[angle, frequency, wind speed, temperature]`` (Fortran order),
    angles in degrees, frequencies in cm^-1, wind speeds in m/s, temperatures
    in K.  A 'Nalli2' classification interpolates in temperature as well
    (``CRTM_IRSSEM.f90:252-301``); other tables use the first temperature."""
    classification: str
    angle: np.ndarray
    frequency: np.ndarray
    wind_speed: np.ndarray
    temperature: np.ndarray
    emissivity: np.ndarray
    version: int = 2


def write_irwatercoeff(path: str, wc: IRwaterCoeff, byteorder: str = "<") -> None:
    """Record order of ``IRwaterCoeff_Define.f90:1147-1210`` (IRwaterCoeff_WriteFile):
    Release/Version, the 4 dimensions, 5 global attributes (length, then the
    text when the length is not 0), the classification name, the 4 axes, the
    emissivity."""
    with open(path, "wb") as f:
        wr = RecordWriter(f, byteorder)
        wr.record(np.array([IRWATERCOEFF_RELEASE, wc.version], np.int32))
        wr.record(np.array([wc.angle.size, wc.frequency.size, wc.wind_speed.size, wc.temperature.size], np.int32))
        for text in ("write_module: crtmv3_gb300.coefficients", "", "title: synthetic IR water emissivity",
                     "", ""):
            wr.record(np.array([len(text)], np.int32))
            if text:
                wr.record(text.encode("ascii"))
        wr.record(wc.classification.ljust(IRWATER_SL)[:IRWATER_SL].encode("ascii"))
        wr.record(wc.angle, wc.frequency, wc.wind_speed, wc.temperature)
        wr.record(np.asfortranarray(wc.emissivity))


def read_irwatercoeff(path: str) -> IRwaterCoeff:
    with open(path, "rb") as f:
        r = RecordReader(f)
        rel, ver = r.split(r.record(), [("i4", (2,))])[0]
        if rel != IRWATERCOEFF_RELEASE:
            raise IOError(f"IRwaterCoeff release {rel} not supported")
        na, nf, nv, nt = (int(x) for x in r.split(r.record(), [("i4", (4,))])[0])
        for _ in range(5):
            (n,) = r.split(r.record(), [("i4", ())])
            if n:
                r.record()
        name = r.split(r.record(), [("S", IRWATER_SL)])[0].strip()
        a, fr, v, t = r.split(r.record(), [("f8", (na,)), ("f8", (nf,)), ("f8", (nv,)), ("f8", (nt,))])
        (e,) = r.split(r.record(), [("f8", (na * nf * nv * nt,))])
    return IRwaterCoeff(name, a, fr, v, t, e.reshape((na, nf, nv, nt), order="F"), int(ver))
