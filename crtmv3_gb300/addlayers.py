"""CRTM_Atmosphere_AddLayers and its K-matrix / adjoint / tangent-linear
counterparts (src/Atmosphere/CRTM_Atmosphere.f90:248-400, :454-514, :569-659).

A profile whose top level lies below the top of the atmosphere
(Level_Pressure(0) > TOA_PRESSURE = 0.005 hPa, src/CRTM_Parameters.f90:157)
gets layers from a climatological model profile
(src/Atmosphere/CRTM_Model_Profiles.f90:1120-1141) between 0.005 hPa and its
top, shifted to join its top two layers without a step.  The forward model
then runs on the extended profile.

As in the reference, the added layers are constants for the derivatives.  The
tangent-linear model gives them zero perturbations (:504).  The K-matrix and
the adjoint return the extended profile's derivatives at the user's layers
only (:620-652).  The user's top two layers enter the shift, but that
dependence is not differentiated.

This is host code.  It builds the extended batch before the call and maps the
outputs back to the user's layers afterwards; the GPU kernels see an ordinary
batch.
"""
from __future__ import annotations

import dataclasses
import functools
import json
import os
from typing import Optional, Tuple

import numpy as np

from .structures import AtmosphereBatch

TOA_PRESSURE = 0.005                 # hPa, CRTM_Parameters.f90:157
MINIMUM_ABSORBER_AMOUNT = 1.0e-76    # CRTM_Parameters.f90:140
US_STANDARD_ATMOSPHERE = 6           # CRTM_Atmosphere_Define.f90:411, Climatology default :448
N_MODELS = 6
# HITRAN absorber id -> index of the model table's absorber axis
# (H2O, O3, CO2, N2O, CO, CH4; CRTM_Model_Profiles.f90:56-78)
_TABLE_INDEX = {1: 0, 2: 2, 3: 1, 4: 3, 5: 4, 6: 5}

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "model_profiles.json")


@functools.lru_cache(maxsize=1)
def model_profiles() -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(level pressure (101,) hPa, level temperature (6, 101) K, level absorber
    (6, 6, 101) in g/kg for H2O and ppmv for the others)."""
    with open(_DATA) as f:
        d = json.load(f)
    return (np.asarray(d["level_pressure_hpa"], np.float64),
            np.asarray(d["level_temperature_k"], np.float64),
            np.asarray(d["level_absorber"], np.float64))


def extra_layers(top_pressure: float) -> int:
    """Number of added layers: the first model level at or below the profile
    top (Extra_Layers, CRTM_Atmosphere.f90:1043-1050); 0 when there is none."""
    pl = model_profiles()[0]
    hits = np.nonzero(pl[1:] >= top_pressure)[0]
    return int(hits[0]) + 1 if hits.size else 0


def needs_layers(atm: AtmosphereBatch, p: int) -> bool:
    if atm.add_extra_layers is not None and not bool(atm.add_extra_layers[p]):
        return False
    return float(atm.level_pressure[p, 0]) > TOA_PRESSURE


def _table_rows(absorber_id: np.ndarray) -> list:
    rows = []
    for j in absorber_id:
        if int(j) not in _TABLE_INDEX:
            raise ValueError(f"AddLayers: the model profiles have no absorber with id {int(j)} "
                             f"(ids 1-6 only)")
        rows.append(_TABLE_INDEX[int(j)])
    return rows


def profile_layers(atm: AtmosphereBatch, p: int):
    """The added layers of profile p: (level pressures (n+1,), layer pressures,
    temperatures (n,), absorbers (J, n)).  The steps follow
    CRTM_Atmosphere.f90:308-353."""
    top = float(atm.level_pressure[p, 0])
    n = extra_layers(top)
    if n < 1:
        raise ValueError(f"AddLayers: profile {p} top pressure {top} hPa is below the model profiles")
    if int(atm.n_layers[p]) < 2:
        raise ValueError(f"AddLayers: profile {p} needs at least 2 layers to extrapolate its top")
    plev, tlev, alev = model_profiles()
    model = US_STANDARD_ATMOSPHERE
    if atm.climatology is not None:
        model = int(atm.climatology[p])
        if model < 1 or model > N_MODELS:
            model = US_STANDARD_ATMOSPHERE   # CRTM_Model_Profiles.f90:1127-1131
    rows = _table_rows(atm.absorber_id)
    pl = plev[:n + 1].copy()
    tl = tlev[model - 1, :n + 1].copy()
    al = alev[model - 1][rows][:, :n + 1].copy()
    # the model's level n moved to the profile top, linear in ln p (:316-327)
    w = (np.log(top) - np.log(pl[n - 1])) / (np.log(pl[n]) - np.log(pl[n - 1]))
    pl[n] = top
    tl[n] = (tl[n] - tl[n - 1]) * w + tl[n - 1]
    al[:, n] = (al[:, n] - al[:, n - 1]) * w + al[:, n - 1]
    # layer means (Layer_P, Layer_X; :330-338, :1054-1066)
    lp = (pl[1:] - pl[:-1]) / np.log(pl[1:] / pl[:-1])
    t = 0.5 * (tl[:-1] + tl[1:])
    a = 0.5 * (al[:, :-1] + al[:, 1:])
    # shift onto the user's top two layers, extrapolated to the lowest added
    # layer's pressure (Shift_Profile, :343-347, :1088-1098)
    P1, P2 = float(atm.pressure[p, 0]), float(atm.pressure[p, 1])
    e = (np.log(lp[n - 1]) - np.log(P1)) / (np.log(P2) - np.log(P1))
    T1, T2 = float(atm.temperature[p, 0]), float(atm.temperature[p, 1])
    t = t + ((T2 - T1) * e + T1 - t[n - 1])
    A1, A2 = atm.absorber[p, :, 0].astype(np.float64), atm.absorber[p, :, 1].astype(np.float64)
    a = a + ((A2 - A1) * e + A1 - a[:, n - 1])[:, None]
    a = np.where(a < 0.0, MINIMUM_ABSORBER_AMOUNT, a)   # :352-353
    return pl, lp, t, a


@dataclasses.dataclass
class AddedLayers:
    """The extension of a batch: layers added on top of each profile and the
    user batch's shape, to map outputs back."""
    n_added: np.ndarray      # (P,) layers added to each profile
    n_layers: np.ndarray     # (P,) the user's layer counts
    max_layers: int          # the user batch's max_layers

    @property
    def any(self) -> bool:
        return bool(self.n_added.any())


def _shift(user: np.ndarray, n_added: np.ndarray, n_layers: np.ndarray, K_ext: int, levels: bool = False,
           fill=None) -> np.ndarray:
    """User arrays (P, ..., K) into the extended layout (P, ..., K_ext): the
    user's layers (or levels) start at n_added[p]; the added part is `fill`
    (per profile, shaped (..., n)) or zero; padding repeats the last value."""
    P = user.shape[0]
    lead = user.shape[1:-1]
    out = np.zeros((P,) + lead + (K_ext + (1 if levels else 0),), np.float64)
    for p in range(P):
        n = int(n_added[p])
        m = int(n_layers[p]) + (1 if levels else 0)
        out[p, ..., n:n + m] = user[p, ..., :m]
        if fill is not None and n:
            out[p, ..., :n] = fill[p]
        if n + m < out.shape[-1]:
            out[p, ..., n + m:] = out[p, ..., n + m - 1:n + m]
    return out


def add_layers(atm: AtmosphereBatch) -> Tuple[AtmosphereBatch, AddedLayers]:
    """CRTM_Atmosphere_AddLayers over a batch.  Returns the batch unchanged when
    no profile needs layers (every top at or above 0.005 hPa, or
    Add_Extra_Layers off)."""
    P = atm.n_profiles
    n_added = np.zeros(P, np.int32)
    parts = {}
    for p in range(P):
        if needs_layers(atm, p):
            parts[p] = profile_layers(atm, p)
            n_added[p] = parts[p][1].shape[0]
    info = AddedLayers(n_added, atm.n_layers.astype(np.int32).copy(), atm.max_layers)
    if not info.any:
        return atm, info
    n_ext = info.n_layers + n_added
    K = int(n_ext.max())

    def fill(i, empty):
        return [parts[p][i] if p in parts else empty for p in range(P)]

    # the added levels are the model levels above the user's top level, which
    # stays the first user level (Atm_Out%Level_Pressure(0:n) = iAtm%pl, :368)
    level_pressure = _shift(atm.level_pressure, n_added, info.n_layers, K, True,
                            [parts[p][0][:-1] if p in parts else np.zeros(0) for p in range(P)])
    pressure = _shift(atm.pressure, n_added, info.n_layers, K, False, fill(1, np.zeros(0)))
    temperature = _shift(atm.temperature, n_added, info.n_layers, K, False, fill(2, np.zeros(0)))
    absorber = _shift(atm.absorber, n_added, info.n_layers, K, False,
                      fill(3, np.zeros((atm.n_absorbers, 0))))

    def zeros_on_top(a):
        return None if a is None else _shift(a, n_added, info.n_layers, K)

    ext = dataclasses.replace(
        atm, n_layers=n_ext.astype(np.int32), level_pressure=level_pressure, pressure=pressure,
        temperature=temperature, absorber=absorber,
        cloud_water_content=zeros_on_top(atm.cloud_water_content),
        cloud_effective_radius=zeros_on_top(atm.cloud_effective_radius),
        cloud_fraction=zeros_on_top(atm.cloud_fraction),
        aerosol_concentration=zeros_on_top(atm.aerosol_concentration),
        aerosol_effective_radius=zeros_on_top(atm.aerosol_effective_radius),
        aerosol_effective_variance=zeros_on_top(atm.aerosol_effective_variance),
        relative_humidity=zeros_on_top(atm.relative_humidity))
    # padding past a profile's last layer carries no cloud or aerosol
    for name in ("cloud_water_content", "cloud_effective_radius", "cloud_fraction", "aerosol_concentration",
                 "aerosol_effective_radius", "aerosol_effective_variance", "relative_humidity"):
        v = getattr(ext, name)
        if v is not None:
            for p in range(P):
                v[p, ..., int(n_ext[p]):] = 0.0
    return ext, info


def extend_perturbation(info: AddedLayers, user_tl: Optional[np.ndarray]) -> Optional[np.ndarray]:
    """A tangent-linear input (P, ..., K) in the extended layout: zero in the
    added layers (CRTM_Atmosphere_AddLayers_TL, CRTM_Atmosphere.f90:504)."""
    if user_tl is None or not info.any:
        return user_tl
    K = int((info.n_layers + info.n_added).max())
    out = np.zeros(user_tl.shape[:-1] + (K,), np.float64)
    for p in range(user_tl.shape[0]):
        n, m = int(info.n_added[p]), int(info.n_layers[p])
        out[p, ..., n:n + m] = user_tl[p, ..., :m]
    return out


def user_layers(info: AddedLayers, ext: Optional[np.ndarray]) -> Optional[np.ndarray]:
    """A layer-indexed output (P, ..., K_ext) back on the user's layers
    (P, ..., max_layers): the extended layers n_added[p] onwards
    (CRTM_Atmosphere_AddLayers_AD, CRTM_Atmosphere.f90:620-652); zero past
    each profile's last layer."""
    if ext is None or not info.any:
        return ext
    out = np.zeros(ext.shape[:-1] + (info.max_layers,), ext.dtype)
    for p in range(ext.shape[0]):
        n, m = int(info.n_added[p]), int(info.n_layers[p])
        out[p, ..., :m] = ext[p, ..., n:n + m]
    return out
