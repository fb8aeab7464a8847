"""Batched, structure-of-arrays forms of CRTM's public input and output structures.

The reference passes arrays of derived types (one object per profile, each
holding allocatable arrays):

* ``CRTM_Atmosphere_type`` (``src/Atmosphere/CRTM_Atmosphere_Define.f90:433-464``),
  with ``CRTM_Cloud_type`` (``Cloud/CRTM_Cloud_Define.f90:295-310``) and
  ``CRTM_Aerosol_type`` (``Aerosol/CRTM_Aerosol_Define.f90:119-133``);
* ``CRTM_Surface_type`` (``src/Surface/CRTM_Surface_Define.f90:204-244``);
* ``CRTM_Geometry_type`` (``src/GeometryInfo/CRTM_Geometry_Define.f90:99-121``);
* ``CRTM_Options_type`` (``src/Options/CRTM_Options_Define.f90:122-179``);
* ``CRTM_RTSolution_type`` (``src/RTSolution/CRTM_RTSolution_Define.f90:201-245``).

Here one object holds a whole batch, padded to the largest layer count, with a
per-profile layer count for ragged batches.  Layer index 0 is the top layer,
as in the reference (its index 1).  The same layout crosses the C-ABI
(``include/crtm_gpu.h``).
"""
from __future__ import annotations

import dataclasses
from typing import Optional

import numpy as np

# Cloud types (``src/Atmosphere/Cloud/CRTM_Cloud_Define.f90:150-154``)
INVALID_CLOUD, WATER_CLOUD, ICE_CLOUD, RAIN_CLOUD, SNOW_CLOUD, GRAUPEL_CLOUD, HAIL_CLOUD = range(7)
# Aerosol types (``src/CRTM_Parameters.f90:286-294``)
DUST_AEROSOL, SEASALT_SSAM_AEROSOL, SULFATE_AEROSOL = 1, 2, 8
# RT algorithm ids (``src/CRTM_Parameters.f90:247-248``)
RT_ADA = 56
RT_SOI = 168


@dataclasses.dataclass
class AtmosphereBatch:
    """P profiles padded to ``max_layers`` layers."""
    n_layers: np.ndarray            # (P,) int32
    level_pressure: np.ndarray      # (P, Kmax+1) hPa; [:,0] is the top level
    pressure: np.ndarray            # (P, Kmax) hPa
    temperature: np.ndarray         # (P, Kmax) K
    absorber: np.ndarray            # (P, Jabs, Kmax)
    absorber_id: np.ndarray         # (Jabs,) HITRAN ids
    absorber_units: np.ndarray      # (Jabs,)
    # clouds (optional): up to NC clouds per profile
    n_clouds: Optional[np.ndarray] = None         # (P,)
    cloud_type: Optional[np.ndarray] = None       # (P, NC)
    cloud_water_content: Optional[np.ndarray] = None   # (P, NC, Kmax) kg/m^2
    cloud_effective_radius: Optional[np.ndarray] = None  # (P, NC, Kmax) microns
    cloud_fraction: Optional[np.ndarray] = None   # (P, Kmax)
    # aerosols (optional)
    n_aerosols: Optional[np.ndarray] = None       # (P,)
    aerosol_type: Optional[np.ndarray] = None     # (P, NA)
    aerosol_concentration: Optional[np.ndarray] = None   # (P, NA, Kmax) kg/m^2
    aerosol_effective_radius: Optional[np.ndarray] = None  # (P, NA, Kmax) microns
    # aerosol scheme inputs: Effective_Variance ('CMAQ') and the layers'
    # Relative_Humidity ('GOCART-GEOS5', 'NAAPS'); None means zero, as the
    # reference's structures are initialised (the LUT lookup clamps them)
    aerosol_effective_variance: Optional[np.ndarray] = None  # (P, NA, Kmax)
    relative_humidity: Optional[np.ndarray] = None  # (P, Kmax), 0..1
    # Atmosphere%Climatology (1-6, default 6 = US Standard Atmosphere) and
    # %Add_Extra_Layers (default true): the model profile that supplies the
    # layers above a top level below 0.005 hPa (CRTM_Atmosphere_Define.f90:436-448)
    climatology: Optional[np.ndarray] = None        # (P,) int
    add_extra_layers: Optional[np.ndarray] = None   # (P,) bool

    @property
    def n_profiles(self) -> int:
        return int(self.n_layers.shape[0])

    @property
    def max_layers(self) -> int:
        return int(self.temperature.shape[1])

    @property
    def n_absorbers(self) -> int:
        return int(self.absorber_id.shape[0])

    def subset(self, idx) -> "AtmosphereBatch":
        def take(a):
            return None if a is None else np.ascontiguousarray(a[idx])
        return AtmosphereBatch(
            take(self.n_layers), take(self.level_pressure), take(self.pressure),
            take(self.temperature), take(self.absorber), self.absorber_id, self.absorber_units,
            take(self.n_clouds), take(self.cloud_type), take(self.cloud_water_content),
            take(self.cloud_effective_radius), take(self.cloud_fraction),
            take(self.n_aerosols), take(self.aerosol_type), take(self.aerosol_concentration),
            take(self.aerosol_effective_radius), take(self.aerosol_effective_variance),
            take(self.relative_humidity), take(self.climatology), take(self.add_extra_layers))


@dataclasses.dataclass
class SurfaceBatch:
    """Surface coverage and temperatures (only the temperatures enter this path)."""
    land_coverage: np.ndarray
    water_coverage: np.ndarray
    snow_coverage: np.ndarray
    ice_coverage: np.ndarray
    land_temperature: np.ndarray
    water_temperature: np.ndarray
    snow_temperature: np.ndarray
    ice_temperature: np.ndarray
    # Surface%Wind_Speed (m/s), read by the IR water emissivity model when the
    # emissivity is not supplied (CRTM_Surface_Define.f90:183 default 5 m/s)
    wind_speed: Optional[np.ndarray] = None

    @staticmethod
    def ocean(water_temperature: np.ndarray) -> "SurfaceBatch":
        P = water_temperature.shape[0]
        z = np.zeros(P)
        return SurfaceBatch(z.copy(), np.ones(P), z.copy(), z.copy(),
                            np.full(P, 280.0), np.asarray(water_temperature, np.float64),
                            np.full(P, 260.0), np.full(P, 260.0))

    def subset(self, idx) -> "SurfaceBatch":
        return SurfaceBatch(*[None if getattr(self, f.name) is None else
                              np.ascontiguousarray(getattr(self, f.name)[idx]) for f in dataclasses.fields(self)])


@dataclasses.dataclass
class GeometryBatch:
    sensor_zenith_angle: np.ndarray   # degrees
    sensor_scan_angle: np.ndarray
    sensor_azimuth_angle: np.ndarray
    source_zenith_angle: np.ndarray
    source_azimuth_angle: np.ndarray
    surface_altitude: np.ndarray      # metres? (reference uses the Atmosphere height; 0 here)

    @staticmethod
    def nadir_like(zenith: np.ndarray) -> "GeometryBatch":
        P = zenith.shape[0]
        return GeometryBatch(np.asarray(zenith, np.float64), np.asarray(zenith, np.float64),
                             np.zeros(P), np.full(P, 100.0), np.zeros(P), np.zeros(P))

    def subset(self, idx) -> "GeometryBatch":
        return GeometryBatch(*[np.ascontiguousarray(getattr(self, f.name)[idx])
                               for f in dataclasses.fields(self)])


@dataclasses.dataclass
class OptionsBatch:
    """Per-profile options (``CRTM_Options_Define.f90:122-179``)."""
    emissivity: Optional[np.ndarray] = None      # (P, L) when Use_Emissivity
    use_n_streams: Optional[np.ndarray] = None   # (P,) bool
    n_streams: Optional[np.ndarray] = None       # (P,) int
    rt_algorithm_id: Optional[np.ndarray] = None  # (P,) RT_ADA / RT_SOI
    include_scattering: bool = True
    overlap_id: Optional[np.ndarray] = None      # (P,) cloud-cover overlap 1-5 (None: 4, average)

    def subset(self, idx) -> "OptionsBatch":
        def take(a):
            return None if a is None else np.ascontiguousarray(a[idx])
        return OptionsBatch(take(self.emissivity), take(self.use_n_streams), take(self.n_streams),
                            take(self.rt_algorithm_id), self.include_scattering, take(self.overlap_id))


@dataclasses.dataclass
class RTSolutionBatch:
    """Outputs per (profile, channel): (P, L) arrays; the layer components
    (layer_optical_depth, upwelling_radiance, upwelling_overcast_radiance)
    are (P, L, max_layers).  The components after the brightness temperature
    are CRTM_RTSolution_type's (CRTM_RTSolution_Define.f90:201-245), filled
    when a call asks for them."""
    radiance: np.ndarray
    brightness_temperature: np.ndarray
    up_radiance: Optional[np.ndarray] = None
    down_radiance: Optional[np.ndarray] = None
    surface_emissivity: Optional[np.ndarray] = None
    n_full_streams: Optional[np.ndarray] = None
    status: Optional[np.ndarray] = None
    tb_clear: Optional[np.ndarray] = None
    r_clear: Optional[np.ndarray] = None
    total_cloud_cover: Optional[np.ndarray] = None
    sod: Optional[np.ndarray] = None
    surface_planck_radiance: Optional[np.ndarray] = None
    layer_optical_depth: Optional[np.ndarray] = None
    upwelling_radiance: Optional[np.ndarray] = None
    upwelling_overcast_radiance: Optional[np.ndarray] = None


@dataclasses.dataclass
class KMatrixBatch:
    """K-matrix outputs: d(BT)/d(input) per (profile, channel).

    ``temperature`` is (P, L, Kmax), ``absorber`` is (P, L, Jabs, Kmax) and the
    surface terms are (P, L).  The reference returns these in
    ``Atmosphere_K(L,M)`` and ``Surface_K(L,M)`` (``CRTM_K_Matrix_Module.f90:300-322``).
    """
    temperature: np.ndarray
    absorber: np.ndarray
    water_temperature: np.ndarray
    surface_emissivity: np.ndarray
    cloud_water_content: Optional[np.ndarray] = None     # (P, L, NC, Kmax)
    cloud_effective_radius: Optional[np.ndarray] = None  # (P, L, NC, Kmax)
    cloud_fraction: Optional[np.ndarray] = None          # (P, L, Kmax)
    aerosol_concentration: Optional[np.ndarray] = None   # (P, L, NA, Kmax)
    aerosol_effective_radius: Optional[np.ndarray] = None  # (P, L, NA, Kmax)
    aerosol_effective_variance: Optional[np.ndarray] = None  # (P, L, NA, Kmax) ('CMAQ')
    relative_humidity: Optional[np.ndarray] = None         # (P, L, Kmax) ('GOCART-GEOS5', 'NAAPS')
    wind_speed: Optional[np.ndarray] = None                # (P, L) through the IR water emissivity model
