"""Python host API over the C-ABI (include/crtm_gpu.h).

Mirrors the reference's public interface for this path:

* ``CRTM_Init`` / ``CRTM_Destroy`` / ``CRTM_IsInitialized``
                                            (src/CRTM_LifeCycle.f90:520, :1131, :1291)
* ``CRTM_Forward``                          (src/CRTM_Forward_Module.f90:229-245)
* ``CRTM_K_Matrix``                         (src/CRTM_K_Matrix_Module.f90:300-322)
* ``CRTM_Adjoint``                          (src/CRTM_Adjoint_Module.f90:299-309)

Each call returns the reference's integer status (SUCCESS=0, FAILURE=3) and
fills caller-provided output objects, as the Fortran routines do.  The
``CRTM`` class underneath offers the same calls on numpy arrays (host
buffers, copies inside the call) and on torch CUDA tensors (device-resident,
no copies).

The GPU library is required: importing succeeds without it, but every call
raises if ``libcrtm_gb300.so`` is missing or no CUDA device is present.
There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as ct
import dataclasses
import os
import types
from typing import List, Optional, Sequence

import numpy as np

from . import addlayers
from .structures import (AtmosphereBatch, GeometryBatch, KMatrixBatch, OptionsBatch,
                         RTSolutionBatch, SurfaceBatch)

SUCCESS, INFORMATION, WARNING, FAILURE = 0, 1, 2, 3
FP64, MIXED = 0, 1

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libcrtm_gb300.so")

_dp = ct.POINTER(ct.c_double)
_ip = ct.POINTER(ct.c_int)


class CBatch(ct.Structure):
    _fields_ = [("n_profiles", ct.c_int), ("max_layers", ct.c_int), ("n_layers", ct.c_void_p),
                ("n_absorbers", ct.c_int), ("absorber_id", ct.c_void_p),
                ("level_pressure", ct.c_void_p), ("pressure", ct.c_void_p),
                ("temperature", ct.c_void_p), ("absorber", ct.c_void_p),
                ("land_coverage", ct.c_void_p), ("water_coverage", ct.c_void_p),
                ("snow_coverage", ct.c_void_p), ("ice_coverage", ct.c_void_p),
                ("land_temperature", ct.c_void_p), ("water_temperature", ct.c_void_p),
                ("snow_temperature", ct.c_void_p), ("ice_temperature", ct.c_void_p),
                ("sensor_zenith_angle", ct.c_void_p), ("source_zenith_angle", ct.c_void_p),
                ("surface_altitude", ct.c_void_p), ("emissivity", ct.c_void_p),
                ("max_clouds", ct.c_int), ("n_clouds", ct.c_void_p), ("cloud_type", ct.c_void_p),
                ("cloud_water_content", ct.c_void_p), ("cloud_effective_radius", ct.c_void_p),
                ("n_streams", ct.c_void_p), ("rt_algorithm_id", ct.c_void_p),
                ("max_aerosols", ct.c_int), ("n_aerosols", ct.c_void_p), ("aerosol_type", ct.c_void_p),
                ("aerosol_concentration", ct.c_void_p), ("aerosol_effective_radius", ct.c_void_p),
                ("cloud_fraction", ct.c_void_p), ("overlap_id", ct.c_void_p),
                ("aerosol_effective_variance", ct.c_void_p), ("relative_humidity", ct.c_void_p),
                ("wind_speed", ct.c_void_p)]


# RTSolution components beyond radiance and brightness temperature, in the
# header's order (crtm_gpu_rtsolution); the last three are (P, L, max_layers)
RTS_COMPONENTS = ("tb_clear", "r_clear", "total_cloud_cover", "sod", "surface_emissivity", "up_radiance",
                  "down_radiance", "surface_planck_radiance", "n_full_streams", "layer_optical_depth",
                  "upwelling_radiance", "upwelling_overcast_radiance")
RTS_LAYER_COMPONENTS = ("layer_optical_depth", "upwelling_radiance", "upwelling_overcast_radiance")


class CRTSolution(ct.Structure):
    _fields_ = [("radiance", ct.c_void_p), ("brightness_temperature", ct.c_void_p),
                ("status", ct.c_void_p)] + [(f, ct.c_void_p) for f in RTS_COMPONENTS]


def _rts(P: int, L: int, K: int, components: bool) -> RTSolutionBatch:
    """Host RTSolution arrays of a call; with ``components`` every further
    RTSolution component too."""
    r = RTSolutionBatch(np.zeros((P, L)), np.zeros((P, L)), status=np.zeros(P, np.int32))
    if components:
        for f in RTS_COMPONENTS:
            shape = (P, L, K) if f in RTS_LAYER_COMPONENTS else (P, L)
            setattr(r, f, np.zeros(shape, np.int32 if f == "n_full_streams" else np.float64))
    return r


def _crts(r: RTSolutionBatch) -> CRTSolution:
    return CRTSolution(r.radiance.ctypes.data, r.brightness_temperature.ctypes.data, _addr(r.status),
                       *[_addr(getattr(r, f, None)) for f in RTS_COMPONENTS])


def _crts_device(out: dict) -> CRTSolution:
    """Device RTSolution of an output dict: radiance, bt, optional status and
    any of the further components under their RTS_COMPONENTS names."""
    return CRTSolution(out["radiance"].data_ptr(), out["bt"].data_ptr(), _addr(out.get("status")),
                       *[_addr(out.get(f)) for f in RTS_COMPONENTS])


SCATTER_JACOBIANS = ("cloud_water_content", "cloud_effective_radius", "cloud_fraction",
                     "aerosol_concentration", "aerosol_effective_radius")


SURFACE_COVERS = ("land_temperature", "snow_temperature", "ice_temperature")

# the aerosol schemes' second LUT coordinate: Effective_Variance ('CMAQ'),
# Relative_Humidity ('GOCART-GEOS5', 'NAAPS')
SCHEME_JACOBIANS = ("aerosol_effective_variance", "relative_humidity", "wind_speed")
AEROSOL_MODELS = ("CRTM", "CMAQ", "GOCART-GEOS5", "NAAPS")


class CKMatrix(ct.Structure):
    _fields_ = [("temperature", ct.c_void_p), ("absorber", ct.c_void_p),
                ("water_temperature", ct.c_void_p), ("surface_emissivity", ct.c_void_p),
                ("n_k_absorbers", ct.c_int), ("k_absorber_index", ct.c_void_p)] + \
               [(f, ct.c_void_p) for f in SCATTER_JACOBIANS + SURFACE_COVERS + SCHEME_JACOBIANS]


class CAdjoint(ct.Structure):
    _fields_ = [("temperature", ct.c_void_p), ("absorber", ct.c_void_p),
                ("water_temperature", ct.c_void_p)] + \
               [(f, ct.c_void_p) for f in SCATTER_JACOBIANS + SURFACE_COVERS + SCHEME_JACOBIANS]


TL_FIELDS = ("temperature", "absorber", "land_temperature", "water_temperature", "snow_temperature",
             "ice_temperature", "emissivity", "cloud_water_content", "cloud_effective_radius", "cloud_fraction",
             "aerosol_concentration", "aerosol_effective_radius", "aerosol_effective_variance",
             "relative_humidity", "wind_speed")


class CTLIn(ct.Structure):
    _fields_ = [(f, ct.c_void_p) for f in TL_FIELDS]


class CTuning(ct.Structure):
    """crtm_gpu_tuning: channels per map CTA, profile cap per pipeline pass,
    measured milliseconds per call."""
    _fields_ = [("map_channels", ct.c_int), ("chunk_profiles", ct.c_int), ("ms_per_call", ct.c_double)]


def _scatter_shapes(atm, aerosol_model: str = "CRTM") -> dict:
    """Per-profile shapes (after the profile axis) of the scattering Jacobians
    that a batch has: clouds (NC, Kmax) and the cloud fraction (Kmax,), aerosols
    (NA, Kmax), and the aerosol scheme's effective variance (NA, Kmax; 'CMAQ')
    or relative humidity (Kmax,; 'GOCART-GEOS5', 'NAAPS')."""
    K = atm.max_layers
    out = {}
    if atm.cloud_type is not None and atm.cloud_type.shape[1] > 0:
        NC = atm.cloud_type.shape[1]
        out.update(cloud_water_content=(NC, K), cloud_effective_radius=(NC, K), cloud_fraction=(K,))
    if atm.aerosol_type is not None and atm.aerosol_type.shape[1] > 0:
        NA = atm.aerosol_type.shape[1]
        out.update(aerosol_concentration=(NA, K), aerosol_effective_radius=(NA, K))
        if aerosol_model == "CMAQ":
            out["aerosol_effective_variance"] = (NA, K)
        if aerosol_model in ("GOCART-GEOS5", "NAAPS"):
            out["relative_humidity"] = (K,)
    return out


_lib = None


def library() -> ct.CDLL:
    """Load the GPU library; raises if it is missing (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"GPU library not built: {LIB_PATH} (run crtmv3_gb300.build.build())")
    L = ct.CDLL(LIB_PATH)
    L.crtm_gpu_init.argtypes = [ct.c_char_p, ct.c_int, ct.POINTER(ct.c_char_p), ct.POINTER(ct.c_void_p)]
    L.crtm_gpu_init_aerosol.argtypes = [ct.c_char_p, ct.c_int, ct.POINTER(ct.c_char_p), ct.c_char_p, ct.c_char_p,
                                        ct.POINTER(ct.c_void_p)]
    L.crtm_gpu_destroy.argtypes = [ct.c_void_p]
    L.crtm_gpu_n_channels.argtypes = [ct.c_void_p, ct.c_int]
    L.crtm_gpu_set_precision.argtypes = [ct.c_void_p, ct.c_int]
    L.crtm_gpu_set_channel_subset.argtypes = [ct.c_void_p, ct.c_int, ct.c_int, ct.c_void_p]
    L.crtm_gpu_get_channel_subset.argtypes = [ct.c_void_p, ct.c_int, ct.c_int, ct.c_void_p]
    L.crtm_gpu_forward.argtypes = [ct.c_void_p, ct.c_int, ct.POINTER(CBatch), ct.POINTER(CRTSolution)]
    L.crtm_gpu_k_matrix.argtypes = [ct.c_void_p, ct.c_int, ct.POINTER(CBatch), ct.c_void_p,
                                    ct.POINTER(CKMatrix), ct.POINTER(CRTSolution)]
    L.crtm_gpu_adjoint.argtypes = [ct.c_void_p, ct.c_int, ct.POINTER(CBatch), ct.c_void_p,
                                   ct.POINTER(CAdjoint), ct.POINTER(CRTSolution)]
    L.crtm_gpu_forward_device.argtypes = [ct.c_void_p, ct.c_int, ct.POINTER(CBatch),
                                          ct.POINTER(CRTSolution), ct.c_void_p]
    L.crtm_gpu_k_matrix_device.argtypes = [ct.c_void_p, ct.c_int, ct.POINTER(CBatch), ct.c_void_p,
                                           ct.POINTER(CKMatrix), ct.POINTER(CRTSolution), ct.c_void_p]
    L.crtm_gpu_adjoint_device.argtypes = [ct.c_void_p, ct.c_int, ct.POINTER(CBatch), ct.c_void_p,
                                          ct.POINTER(CAdjoint), ct.POINTER(CRTSolution), ct.c_void_p]
    L.crtm_gpu_k_matrix_device_static.argtypes = L.crtm_gpu_k_matrix_device.argtypes
    L.crtm_gpu_linearize.argtypes = [ct.c_void_p, ct.c_int, ct.POINTER(CBatch), ct.POINTER(CRTSolution),
                                     ct.c_void_p]
    L.crtm_gpu_tangent_linear_apply.argtypes = [ct.c_void_p, ct.POINTER(CTLIn), ct.c_void_p, ct.c_void_p]
    L.crtm_gpu_adjoint_apply.argtypes = [ct.c_void_p, ct.c_void_p, ct.POINTER(CAdjoint), ct.c_void_p]
    L.crtm_gpu_get_tuning.argtypes = [ct.c_void_p, ct.c_int, ct.c_int, ct.POINTER(CTuning)]
    L.crtm_gpu_set_tuning.argtypes = [ct.c_void_p, ct.c_int, ct.c_int, ct.POINTER(CTuning)]
    L.crtm_gpu_autotune_k_matrix_device.argtypes = L.crtm_gpu_k_matrix_device.argtypes + [
        ct.c_int, ct.POINTER(CTuning), ct.c_int, ct.POINTER(ct.c_int), ct.POINTER(CTuning)]
    L.crtm_gpu_last_error.argtypes = [ct.c_void_p, ct.c_char_p, ct.c_int]
    L.crtm_gpu_launch_count.argtypes = [ct.c_void_p]
    L.crtm_gpu_launch_count.restype = ct.c_longlong
    L.crtm_gpu_set_profiling.argtypes = [ct.c_void_p, ct.c_int]
    L.crtm_gpu_stage_times.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_int]
    _lib = L
    return L


def _addr(a) -> Optional[int]:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()   # torch tensor


class CRTM:
    """One library handle: the coefficient tables of a list of sensors."""

    def __init__(self, sensor_ids: Sequence[str], coeff_path: str, precision: int = FP64,
                 aerosol_model: Optional[str] = None, aerosol_coeff_file: Optional[str] = None):
        """``aerosol_model`` / ``aerosol_coeff_file``: CRTM_Init's Aerosol_Model
        ('CRTM' by default, 'CMAQ', 'GOCART-GEOS5', 'NAAPS') and the AerosolCoeff
        file name under ``coeff_path`` (default AerosolCoeff.bin)."""
        L = library()
        h = ct.c_void_p()
        ids = (ct.c_char_p * len(sensor_ids))(*[s.encode() for s in sensor_ids])
        if aerosol_model is None and aerosol_coeff_file is None:
            rc = L.crtm_gpu_init(coeff_path.encode(), len(sensor_ids), ids, ct.byref(h))
        else:
            rc = L.crtm_gpu_init_aerosol(coeff_path.encode(), len(sensor_ids), ids,
                                         None if aerosol_model is None else aerosol_model.encode(),
                                         None if aerosol_coeff_file is None else aerosol_coeff_file.encode(),
                                         ct.byref(h))
        if rc != SUCCESS:
            raise RuntimeError("crtm_gpu_init: " + self._err(None))
        self.h = h
        self.aerosol_model = aerosol_model or "CRTM"
        self.sensor_ids = list(sensor_ids)
        self.n_channels = [L.crtm_gpu_n_channels(h, i) for i in range(len(sensor_ids))]
        self.set_precision(precision)

    def set_channel_subset(self, sensor: int, positions=None) -> None:
        """Process only the channels at these 0-based file positions in later
        calls for ``sensor`` (crtm_gpu_set_channel_subset); None: all channels."""
        if positions is None:
            rc = library().crtm_gpu_set_channel_subset(self.h, sensor, -1, None)
        else:
            idx = np.ascontiguousarray(positions, np.int32)
            rc = library().crtm_gpu_set_channel_subset(self.h, sensor, int(idx.size), idx.ctypes.data)
        self._check(rc)
        self.n_channels[sensor] = library().crtm_gpu_n_channels(self.h, sensor)

    def channel_subset(self, sensor: int) -> np.ndarray:
        """0-based file positions of the channels calls for ``sensor`` process."""
        n = library().crtm_gpu_n_channels(self.h, sensor)
        out = np.zeros(max(n, 0), np.int32)
        library().crtm_gpu_get_channel_subset(self.h, sensor, int(out.size), out.ctypes.data if n > 0 else None)
        return out

    @staticmethod
    def _err(h) -> str:
        L = library()
        buf = ct.create_string_buffer(2048)
        L.crtm_gpu_last_error(h, buf, 2048)
        return buf.value.decode(errors="replace")

    def error(self) -> str:
        return self._err(self.h)

    def set_precision(self, precision: int) -> None:
        if library().crtm_gpu_set_precision(self.h, precision) != SUCCESS:
            raise ValueError(self.error())
        self.precision = precision

    def launch_count(self) -> int:
        return int(library().crtm_gpu_launch_count(self.h))

    STAGES = ("prep", "absorb_fwd", "column", "absorb_ad", "map_out", "adjoint_sum", "scatter_layers",
              "scatter_adding", "scatter_contract", "scatter_species")

    def set_profiling(self, enable: bool) -> None:
        library().crtm_gpu_set_profiling(self.h, int(enable))

    def stage_times(self, reset: bool = True) -> dict:
        """{stage: (milliseconds, launches)} accumulated while profiling was enabled."""
        ms = np.zeros(len(self.STAGES))
        n = np.zeros(len(self.STAGES), np.int64)
        k = library().crtm_gpu_stage_times(self.h, ms.ctypes.data, n.ctypes.data, len(self.STAGES), int(reset))
        return {self.STAGES[i]: (float(ms[i]), int(n[i])) for i in range(min(k, len(self.STAGES)))}

    def close(self) -> None:
        if getattr(self, "h", None):
            library().crtm_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------
    # host (numpy) calls
    # ------------------------------------------------------------------
    def _cbatch(self, atm: AtmosphereBatch, sfc: SurfaceBatch, geo: GeometryBatch,
                opt: OptionsBatch, keep: list) -> CBatch:
        def c(a, dt=np.float64):
            a = np.ascontiguousarray(a, dtype=dt)
            keep.append(a)
            return a.ctypes.data
        b = CBatch()
        b.n_profiles = atm.n_profiles
        b.max_layers = atm.max_layers
        b.n_layers = c(atm.n_layers, np.int32)
        b.n_absorbers = atm.n_absorbers
        b.absorber_id = c(atm.absorber_id, np.int32)
        b.level_pressure = c(atm.level_pressure)
        b.pressure = c(atm.pressure)
        b.temperature = c(atm.temperature)
        b.absorber = c(atm.absorber)
        for f in ("land_coverage", "water_coverage", "snow_coverage", "ice_coverage",
                  "land_temperature", "water_temperature", "snow_temperature", "ice_temperature"):
            setattr(b, f, c(getattr(sfc, f)))
        b.sensor_zenith_angle = c(geo.sensor_zenith_angle)
        b.source_zenith_angle = c(geo.source_zenith_angle)
        b.surface_altitude = c(geo.surface_altitude)
        # no emissivity: the IR sea-surface emissivity model (clear-sky IR batches over water)
        if opt is not None and opt.emissivity is not None:
            b.emissivity = c(opt.emissivity)
        if getattr(sfc, "wind_speed", None) is not None:
            b.wind_speed = c(sfc.wind_speed)
        if atm.n_clouds is not None and atm.cloud_type is not None and atm.cloud_type.shape[1] > 0:
            b.max_clouds = int(atm.cloud_type.shape[1])
            b.n_clouds = c(atm.n_clouds, np.int32)
            b.cloud_type = c(atm.cloud_type, np.int32)
            b.cloud_water_content = c(atm.cloud_water_content)
            b.cloud_effective_radius = c(atm.cloud_effective_radius)
            if atm.cloud_fraction is not None:
                b.cloud_fraction = c(atm.cloud_fraction)
        if getattr(opt, "overlap_id", None) is not None:
            b.overlap_id = c(opt.overlap_id, np.int32)
        if opt.n_streams is not None:
            use = opt.use_n_streams if opt.use_n_streams is not None else np.ones(atm.n_profiles, bool)
            b.n_streams = c(np.where(use, opt.n_streams, 0), np.int32)
        if opt.rt_algorithm_id is not None:
            b.rt_algorithm_id = c(opt.rt_algorithm_id, np.int32)
        if atm.n_aerosols is not None and atm.aerosol_type is not None and atm.aerosol_type.shape[1] > 0:
            b.max_aerosols = int(atm.aerosol_type.shape[1])
            b.n_aerosols = c(atm.n_aerosols, np.int32)
            b.aerosol_type = c(atm.aerosol_type, np.int32)
            b.aerosol_concentration = c(atm.aerosol_concentration)
            b.aerosol_effective_radius = c(atm.aerosol_effective_radius)
            if getattr(atm, "aerosol_effective_variance", None) is not None:
                b.aerosol_effective_variance = c(atm.aerosol_effective_variance)
            if getattr(atm, "relative_humidity", None) is not None:
                b.relative_humidity = c(atm.relative_humidity)
        return b

    def _check(self, rc: int) -> None:
        if rc != SUCCESS:
            raise RuntimeError(self.error())

    def forward(self, atm, sfc, geo, opt, sensor: int = 0, components: bool = False) -> RTSolutionBatch:
        """CRTM_Forward with host buffers.  ``components``: also return the
        further RTSolution components (RTS_COMPONENTS)."""
        P, L = atm.n_profiles, self.n_channels[sensor]
        keep: list = []
        b = self._cbatch(atm, sfc, geo, opt, keep)
        rts = _rts(P, L, atm.max_layers, components)
        cr = _crts(rts)
        self._check(library().crtm_gpu_forward(self.h, sensor, ct.byref(b), ct.byref(cr)))
        return rts

    def k_matrix(self, atm, sfc, geo, opt, bt_k=None, sensor: int = 0, k_absorbers=None, out=None,
                 scattering_jacobians: bool = True, components: bool = False, rts_out=None):
        """K-matrix with host buffers.  ``k_absorbers``: optional list of user absorber
        indices whose Jacobians are returned (default: all).  ``out`` / ``rts_out``:
        optional preallocated KMatrixBatch / RTSolutionBatch (e.g. in pinned memory).  ``scattering_jacobians``:
        also return the cloud water content / effective radius / fraction and
        aerosol concentration / effective radius Jacobians of a batch with clouds
        or aerosols.  ``components``: also return the further RTSolution
        components."""
        P, L, K, J = atm.n_profiles, self.n_channels[sensor], atm.max_layers, atm.n_absorbers
        keep: list = []
        b = self._cbatch(atm, sfc, geo, opt, keep)
        seed = None if bt_k is None else np.ascontiguousarray(bt_k, np.float64)
        sel = None if k_absorbers is None else np.ascontiguousarray(k_absorbers, np.int32)
        JK = J if sel is None else int(sel.shape[0])
        rts = rts_out if rts_out is not None else _rts(P, L, K, components)
        km = out if out is not None else KMatrixBatch(np.zeros((P, L, K)), np.zeros((P, L, JK, K)),
                                                      np.zeros((P, L)), np.zeros((P, L)))
        if out is None and scattering_jacobians:
            for f, shp in _scatter_shapes(atm, self.aerosol_model).items():
                setattr(km, f, np.zeros((P, L) + shp))
        if out is None:
            for f in SURFACE_COVERS:
                setattr(km, f, np.zeros((P, L)))
            if opt is None or opt.emissivity is None:
                km.wind_speed = np.zeros((P, L))
        cr = _crts(rts)
        ck = CKMatrix(km.temperature.ctypes.data, km.absorber.ctypes.data,
                      km.water_temperature.ctypes.data, km.surface_emissivity.ctypes.data,
                      0 if sel is None else JK, None if sel is None else sel.ctypes.data,
                      *[_addr(getattr(km, f, None)) for f in SCATTER_JACOBIANS + SURFACE_COVERS + SCHEME_JACOBIANS])
        self._check(library().crtm_gpu_k_matrix(self.h, sensor, ct.byref(b), _addr(seed),
                                                ct.byref(ck), ct.byref(cr)))
        return km, rts

    def adjoint(self, atm, sfc, geo, opt, bt_ad, sensor: int = 0, components: bool = False):
        P, L, K, J = atm.n_profiles, self.n_channels[sensor], atm.max_layers, atm.n_absorbers
        keep: list = []
        b = self._cbatch(atm, sfc, geo, opt, keep)
        seed = np.ascontiguousarray(bt_ad, np.float64)
        rts = _rts(P, L, K, components)
        out = dict(temperature=np.zeros((P, K)), absorber=np.zeros((P, J, K)), water_temperature=np.zeros(P))
        for f, shp in _scatter_shapes(atm, self.aerosol_model).items():
            out[f] = np.zeros((P,) + shp)
        for f in SURFACE_COVERS:
            out[f] = np.zeros(P)
        if opt is None or opt.emissivity is None:
            out["wind_speed"] = np.zeros(P)
        cr = _crts(rts)
        ca = CAdjoint(out["temperature"].ctypes.data, out["absorber"].ctypes.data,
                      out["water_temperature"].ctypes.data,
                      *[_addr(out.get(f)) for f in SCATTER_JACOBIANS + SURFACE_COVERS + SCHEME_JACOBIANS])
        self._check(library().crtm_gpu_adjoint(self.h, sensor, ct.byref(b), seed.ctypes.data,
                                               ct.byref(ca), ct.byref(cr)))
        return out, rts

    def tangent_linear(self, atm, sfc, geo, opt, atm_tl=None, sfc_tl=None, emissivity_tl=None,
                       sensor: int = 0, components: bool = False):
        """CRTM_Tangent_Linear: the brightness-temperature perturbation (P, L)
        from perturbations of the atmosphere (``atm_tl``: an object with any of
        temperature, absorber, cloud_water_content, cloud_effective_radius,
        cloud_fraction, aerosol_concentration, aerosol_effective_radius shaped
        like ``atm``'s), the surface (``sfc_tl``: cover temperatures) and the
        emissivity (P, L).  Returns (bt_tl, rts)."""
        P, L = atm.n_profiles, self.n_channels[sensor]
        keep: list = []
        b = self._cbatch(atm, sfc, geo, opt, keep)

        def arr(obj, name):
            v = getattr(obj, name, None) if obj is not None else None
            if v is None:
                return None
            a = np.ascontiguousarray(v, np.float64)
            keep.append(a)
            return a.ctypes.data
        vals = {f: arr(atm_tl, f) for f in ("temperature", "absorber", "cloud_water_content",
                                             "cloud_effective_radius", "cloud_fraction", "aerosol_concentration",
                                             "aerosol_effective_radius", "aerosol_effective_variance",
                                             "relative_humidity")}
        vals.update({f: arr(sfc_tl, f) for f in ("land_temperature", "water_temperature", "snow_temperature",
                                                  "ice_temperature", "wind_speed")})
        if emissivity_tl is not None:
            e = np.ascontiguousarray(emissivity_tl, np.float64)
            keep.append(e)
            vals["emissivity"] = e.ctypes.data
        tl = CTLIn(*[vals.get(f) for f in TL_FIELDS])
        rts = _rts(P, L, atm.max_layers, components)
        cr = _crts(rts)
        bt_tl = np.zeros((P, L))
        self._check(library().crtm_gpu_tangent_linear(self.h, sensor, ct.byref(b), ct.byref(tl), ct.byref(cr),
                                                      bt_tl.ctypes.data))
        return bt_tl, rts

    # ------------------------------------------------------------------
    # device-resident (torch CUDA tensors) calls
    # ------------------------------------------------------------------
    def device_batch(self, dev: dict, absorber_id: np.ndarray) -> tuple:
        """``dev``: dict of torch CUDA tensors with the batch fields (float64 /
        int32 n_layers).  absorber_id stays on the host."""
        keep = [np.ascontiguousarray(absorber_id, np.int32)]
        b = CBatch()
        P, K = dev["temperature"].shape
        b.n_profiles = P
        b.max_layers = K
        b.n_layers = dev["n_layers"].data_ptr()
        b.n_absorbers = int(keep[0].shape[0])
        b.absorber_id = keep[0].ctypes.data
        for f in ("level_pressure", "pressure", "temperature", "absorber", "land_coverage",
                  "water_coverage", "snow_coverage", "ice_coverage", "land_temperature",
                  "water_temperature", "snow_temperature", "ice_temperature",
                  "sensor_zenith_angle", "source_zenith_angle", "surface_altitude", "emissivity",
                  "n_clouds", "cloud_type", "cloud_water_content", "cloud_effective_radius",
                  "n_streams", "rt_algorithm_id", "n_aerosols", "aerosol_type", "aerosol_concentration",
                  "aerosol_effective_radius", "cloud_fraction", "overlap_id", "aerosol_effective_variance",
                  "relative_humidity", "wind_speed"):
            t = dev.get(f)
            setattr(b, f, None if t is None else t.data_ptr())
        if dev.get("cloud_type") is not None:
            b.max_clouds = int(dev["cloud_type"].shape[1])
        if dev.get("aerosol_type") is not None:
            b.max_aerosols = int(dev["aerosol_type"].shape[1])
        return b, keep

    def k_matrix_device(self, b: CBatch, out: dict, seed=None, sensor: int = 0, stream=None,
                        k_absorbers=None, static_scratch: bool = False) -> None:
        """K-matrix on device tensors.  ``static_scratch``: use the entry point that
        keeps its intermediates in the library's fixed per-device scratch and
        allocates no device memory (calls must not overlap in time)."""
        cr, ck, sel = self._kmatrix_structs(out, k_absorbers)
        fn = (library().crtm_gpu_k_matrix_device_static if static_scratch
              else library().crtm_gpu_k_matrix_device)
        self._check(fn(self.h, sensor, ct.byref(b), _addr(seed), ct.byref(ck), ct.byref(cr), stream))

    @staticmethod
    def _kmatrix_structs(out: dict, k_absorbers=None):
        cr = _crts_device(out)
        sel = None if k_absorbers is None else np.ascontiguousarray(k_absorbers, np.int32)
        ck = CKMatrix(out["temperature_k"].data_ptr(), out["absorber_k"].data_ptr(),
                      out["water_temperature_k"].data_ptr(), out["surface_emissivity_k"].data_ptr(),
                      0 if sel is None else int(sel.shape[0]), None if sel is None else sel.ctypes.data,
                      *[_addr(out.get(f + "_k")) for f in SCATTER_JACOBIANS])
        for f in SCHEME_JACOBIANS:
            setattr(ck, f, _addr(out.get(f + "_k")))
        return cr, ck, sel   # sel keeps the absorber selection alive during the call

    def tuning(self, sensor: int = 0, precision: Optional[int] = None) -> dict:
        """The tuning in effect for a sensor and arithmetic form (default: the
        handle's): map_channels, chunk_profiles, ms_per_call."""
        t = CTuning()
        pr = self.precision if precision is None else precision
        self._check(library().crtm_gpu_get_tuning(self.h, sensor, pr, ct.byref(t)))
        return dict(map_channels=t.map_channels, chunk_profiles=t.chunk_profiles, ms_per_call=t.ms_per_call)

    def set_tuning(self, map_channels: int = 0, chunk_profiles: int = 0, sensor: int = 0,
                   precision: Optional[int] = None) -> None:
        pr = self.precision if precision is None else precision
        t = CTuning(map_channels, chunk_profiles, 0.0)
        self._check(library().crtm_gpu_set_tuning(self.h, sensor, pr, ct.byref(t)))

    def autotune_k_matrix_device(self, b: CBatch, out: dict, seed=None, sensor: int = 0, stream=None,
                                 reps: int = 3, k_absorbers=None) -> dict:
        """Time the device K-matrix of this batch under each candidate tuning
        and keep the fastest for the sensor (crtm_gpu_autotune_k_matrix_device).
        Returns {"chosen": {...}, "trials": [{...}, ...]}; ``out`` holds the
        batch's K-matrix afterwards."""
        cr, ck, sel = self._kmatrix_structs(out, k_absorbers)
        trials = (CTuning * 16)()
        n = ct.c_int(0)
        best = CTuning()
        self._check(library().crtm_gpu_autotune_k_matrix_device(
            self.h, sensor, ct.byref(b), _addr(seed), ct.byref(ck), ct.byref(cr), stream, reps,
            trials, 16, ct.byref(n), ct.byref(best)))
        conv = lambda t: dict(map_channels=t.map_channels, chunk_profiles=t.chunk_profiles,
                              ms_per_call=t.ms_per_call)
        return dict(chosen=conv(best), trials=[conv(trials[i]) for i in range(min(n.value, 16))])

    def forward_device(self, b: CBatch, out: dict, sensor: int = 0, stream=None) -> None:
        cr = _crts_device(out)
        self._check(library().crtm_gpu_forward_device(self.h, sensor, ct.byref(b), ct.byref(cr), stream))

    def adjoint_device(self, b: CBatch, seed, out: dict, sensor: int = 0, stream=None) -> None:
        cr = _crts_device(out)
        ca = CAdjoint(out["temperature_ad"].data_ptr(), out["absorber_ad"].data_ptr(),
                      out["water_temperature_ad"].data_ptr(), *[_addr(out.get(f + "_ad")) for f in SCATTER_JACOBIANS])
        for f in SCHEME_JACOBIANS:
            setattr(ca, f, _addr(out.get(f + "_ad")))
        self._check(library().crtm_gpu_adjoint_device(self.h, sensor, ct.byref(b), seed.data_ptr(),
                                                      ct.byref(ca), ct.byref(cr), stream))


    # -- a trajectory for variational inner loops (no reference counterpart) --
    def linearize_device(self, b: CBatch, out: dict, sensor: int = 0, stream=None) -> None:
        """crtm_gpu_linearize: the trajectory's forward (out: radiance, bt,
        status) and its K-matrix, kept by the handle for the apply calls."""
        cr = _crts_device(out)
        self._check(library().crtm_gpu_linearize(self.h, sensor, ct.byref(b), ct.byref(cr), stream))

    def tangent_linear_apply_device(self, tl: dict, bt_tl, stream=None) -> None:
        """crtm_gpu_tangent_linear_apply: bt_tl (P, L) from the perturbations in
        ``tl`` (device tensors under TL_FIELDS names) about the trajectory."""
        ctl = CTLIn(*[_addr(tl.get(f)) for f in TL_FIELDS])
        self._check(library().crtm_gpu_tangent_linear_apply(self.h, ct.byref(ctl), bt_tl.data_ptr(), stream))

    def adjoint_apply_device(self, seed, out: dict, stream=None) -> None:
        """crtm_gpu_adjoint_apply: the adjoint outputs (``out`` as
        adjoint_device's: temperature_ad, absorber_ad, water_temperature_ad and
        any scattering / surface / scheme ``*_ad``) for the seed (P, L)."""
        ca = CAdjoint(out["temperature_ad"].data_ptr(), out["absorber_ad"].data_ptr(),
                      out["water_temperature_ad"].data_ptr(), *[_addr(out.get(f + "_ad")) for f in SCATTER_JACOBIANS])
        for f in SURFACE_COVERS + SCHEME_JACOBIANS:
            setattr(ca, f, _addr(out.get(f + "_ad")))
        self._check(library().crtm_gpu_adjoint_apply(self.h, seed.data_ptr(), ct.byref(ca), stream))


# ---------------------------------------------------------------------------
# Reference-named entry points
# ---------------------------------------------------------------------------

@dataclasses.dataclass
class ChannelInfo:
    """CRTM_ChannelInfo_type (src/ChannelInfo/CRTM_ChannelInfo_Define.f90:70-85), reduced to
    what this path needs: the sensor, its index in the handle, the count of
    channels calls process, the Sensor_Channel numbers of the coefficient
    files' channels and which of them are processed (Process_Channel)."""
    sensor_id: str
    sensor_index: int
    n_channels: int
    handle: CRTM
    sensor_channel: Optional[np.ndarray] = None
    process_channel: Optional[np.ndarray] = None


def CRTM_ChannelInfo_n_Channels(channel_info: ChannelInfo) -> int:
    """CRTM_ChannelInfo_n_Channels (CRTM_ChannelInfo_Define.f90:336-340)."""
    return int(channel_info.n_channels)


def CRTM_ChannelInfo_Channels(channel_info: ChannelInfo) -> np.ndarray:
    """CRTM_ChannelInfo_Channels (CRTM_ChannelInfo_Define.f90:373-377): the
    Sensor_Channel numbers of the processed channels."""
    return channel_info.sensor_channel[channel_info.process_channel]


def CRTM_ChannelInfo_Subset(channel_info: ChannelInfo, channel_subset=None, reset: bool = False) -> int:
    """CRTM_ChannelInfo_Subset (CRTM_ChannelInfo_Define.f90:444-517): later
    calls with this ChannelInfo process only the channels whose Sensor_Channel
    number is in ``channel_subset`` (in the files' order; their RTSolution,
    K-matrix and Options%Emissivity have that many channels).  ``reset``:
    all channels again (the subset is then ignored).  An empty subset turns
    every channel off.  A subset with more channels than the sensor's, or
    with numbers outside the sensor's range, fails and turns every channel
    off, as the reference does."""
    ci = channel_info
    if reset:
        ci.handle.set_channel_subset(ci.sensor_index, None)
        ci.process_channel = np.ones(ci.sensor_channel.size, bool)
        ci.n_channels = int(ci.process_channel.sum())
        return SUCCESS
    if channel_subset is None:
        return SUCCESS
    sub = np.asarray(channel_subset, np.int64).ravel()
    ci.process_channel = np.zeros(ci.sensor_channel.size, bool)
    err = None
    if sub.size > ci.sensor_channel.size:
        err = "Specified Channel_Subset contains too many channels!"
    elif sub.size and (sub.min() < ci.sensor_channel.min() or sub.max() > ci.sensor_channel.max()):
        err = "Specified Channel_Subset contains invalid channels!"
    else:
        ci.process_channel = np.isin(ci.sensor_channel, sub)
    ci.handle.set_channel_subset(ci.sensor_index, np.flatnonzero(ci.process_channel))
    ci.n_channels = int(ci.process_channel.sum())
    if err:
        print(f"CRTM_ChannelInfo_Subset(FAILURE): {err}")
        return FAILURE
    return SUCCESS


def CRTM_Init(sensor_ids: Sequence[str], channel_info: List[ChannelInfo], file_path: str = ".",
              precision: int = FP64, aerosol_model: Optional[str] = None,
              aerosolcoeff_file: Optional[str] = None, spccoeff_format: str = "Binary",
              taucoeff_format: str = "Binary", irwatercoeff_format: str = "Binary",
              cloudcoeff_format: str = "Binary", aerosolcoeff_format: str = "Binary",
              cloudcoeff_file: Optional[str] = None, cloud_model: Optional[str] = None,
              irwatercoeff_file: Optional[str] = None, nc_file_path: Optional[str] = None,
              load_cloudcoeff: bool = True, load_aerosolcoeff: bool = True) -> int:
    """CRTM_Init: load the coefficients of ``sensor_ids`` and fill ``channel_info``.
    The keyword arguments are the reference's optional arguments
    (src/CRTM_LifeCycle.f90:519-591) for the tables this path reads:
    Aerosol_Model, AerosolCoeff_Format / _File, Cloud_Model, CloudCoeff_Format
    / _File, SpcCoeff_Format, TauCoeff_Format, IRwaterCoeff_Format / _File,
    NC_File_Path, Load_CloudCoeff and Load_AerosolCoeff.

    - A format 'netCDF' reads <id>.SpcCoeff.nc / <id>.TauCoeff.nc from
      File_Path, and the cloud table (CloudCoeff_File, default CloudCoeff.nc),
      the aerosol table (AerosolCoeff_File, default AerosolCoeff.nc, in the
      Aerosol_Model's layout) and the IR water table (IRwaterCoeff_File,
      default Nalli.IRwater.EmisCoeff.nc) from NC_File_Path when given, else
      File_Path (:782-790, :811-815, :865-867).  They are converted to binary
      files in a private directory, which the library loads.
    - A binary CloudCoeff_File or IRwaterCoeff_File under another name is
      linked into that directory under the default name.
    - Load_CloudCoeff / Load_AerosolCoeff = False leave the table out
      (:653-656, :782, :811); a batch with clouds or aerosols is then refused.
    - Cloud_Model is accepted and, as in the reference, does not select the
      table: CRTM_CloudCoeff_Load reads the file CloudCoeff_File names
      (src/Coefficients/CRTM_CloudCoeff.f90:185-240)."""
    from . import netcdf_coeffs as ncc
    del cloud_model
    path = file_path
    nc_path = nc_file_path or file_path
    irwater_bin = ncc.IRWATER_FILE + ".bin"
    try:
        fmts = (spccoeff_format, taucoeff_format, irwatercoeff_format, cloudcoeff_format, aerosolcoeff_format)
        for fm in fmts:
            if fm.lower() not in ("binary", "netcdf"):
                raise ValueError(f"coefficient format must be 'Binary' or 'netCDF' (got {fm!r})")
        cloud_nc, ir_nc, aer_nc = (fm.lower() == "netcdf" for fm in
                                   (cloudcoeff_format, irwatercoeff_format, aerosolcoeff_format))
        cloud_renamed = not cloud_nc and cloudcoeff_file not in (None, "CloudCoeff.bin")
        ir_renamed = not ir_nc and irwatercoeff_file not in (None, irwater_bin)
        if not load_aerosolcoeff:
            aerosol_model = aerosolcoeff_file = None
        if (any(fm.lower() == "netcdf" for fm in fmts) or cloud_renamed or ir_renamed
                or not load_cloudcoeff or not load_aerosolcoeff):
            import tempfile
            path = tempfile.mkdtemp(prefix="crtm_coeffs_")
            for s in sensor_ids:
                ncc.convert_sensor(file_path, s, path, spccoeff_format, taucoeff_format)
            if load_cloudcoeff and cloud_nc:
                ncc.convert_cloud(nc_path, path, cloudcoeff_file or "CloudCoeff.nc")
            elif load_cloudcoeff and cloud_renamed:
                ncc._link(os.path.join(file_path, cloudcoeff_file), os.path.join(path, "CloudCoeff.bin"))
            if ir_nc:
                ncc.convert_irwater(nc_path, path, irwatercoeff_file or ncc.IRWATER_FILE + ".nc")
            elif ir_renamed:
                ncc._link(os.path.join(file_path, irwatercoeff_file), os.path.join(path, irwater_bin))
            if load_aerosolcoeff and aer_nc:
                aerosolcoeff_file = ncc.convert_aerosol(nc_path, path, aerosol_model or "CRTM",
                                                        aerosolcoeff_file or "AerosolCoeff.nc")
            names = [n for n in ncc.SHARED_FILES
                     if (load_cloudcoeff or n != "CloudCoeff.bin")
                     and (load_aerosolcoeff or not n.startswith("AerosolCoeff"))]
            ncc.link_shared_files(file_path, path, names=names,
                                  extra=(aerosolcoeff_file,) if aerosolcoeff_file else ())
    except (OSError, ValueError, KeyError) as e:
        print(f"CRTM_Init(FAILURE): {e}")
        return FAILURE
    try:
        h = CRTM(sensor_ids, path, precision, aerosol_model, aerosolcoeff_file)
    except RuntimeError as e:
        print(f"CRTM_Init(FAILURE): {e}")
        return FAILURE
    channel_info.clear()
    from .coefficients import read_spccoeff
    for i, s in enumerate(sensor_ids):
        sc = read_spccoeff(os.path.join(path, f"{s}.SpcCoeff.bin"))
        channel_info.append(ChannelInfo(s, i, h.n_channels[i], h, np.asarray(sc.sensor_channel),
                                        np.ones(h.n_channels[i], bool)))
    return SUCCESS


def CRTM_Destroy(channel_info: List[ChannelInfo]) -> int:
    handles = {id(ci.handle): ci.handle for ci in channel_info}
    for h in handles.values():
        h.close()
    channel_info.clear()
    return SUCCESS


def CRTM_IsInitialized(channel_info: Sequence[ChannelInfo]) -> bool:
    """CRTM_IsInitialized (src/CRTM_LifeCycle.f90:1291-1295): every ChannelInfo
    holds a live library handle (ALL() of an empty list is true, as in
    Fortran)."""
    return all(ci.handle is not None and getattr(ci.handle, "h", None) for ci in channel_info)


def CRTM_Forward(atmosphere: AtmosphereBatch, surface: SurfaceBatch, geometry: GeometryBatch,
                 channel_info: List[ChannelInfo], rts: List[RTSolutionBatch],
                 options: Optional[OptionsBatch] = None) -> int:
    """CRTM_Forward.  ``rts`` receives one RTSolutionBatch per sensor in ChannelInfo order.
    ``options.emissivity`` is (P, total channels) over all sensors."""
    rts.clear()
    atmosphere, added = _added_layers(atmosphere, "CRTM_Forward")
    if atmosphere is None:
        return FAILURE
    off = 0
    for ci in channel_info:
        opt = _sensor_options(options, off, ci.n_channels)
        try:
            r = ci.handle.forward(atmosphere, surface, geometry, opt, ci.sensor_index, components=True)
        except RuntimeError as e:
            print(f"CRTM_Forward(FAILURE): {e}")
            return FAILURE
        rts.append(_user_layer_components(added, r))
        off += ci.n_channels
    return SUCCESS


def _user_layer_components(added, r: RTSolutionBatch) -> RTSolutionBatch:
    """The layer components of an RTSolution on the user's layers
    (Layer_Optical_Depth(1:no) = the extended profile's na+1:nt,
    Common_RTSolution.f90:239,1206-1207)."""
    if not added.any:
        return r
    return dataclasses.replace(r, **{f: addlayers.user_layers(added, getattr(r, f))
                                     for f in RTS_LAYER_COMPONENTS if getattr(r, f) is not None})


def CRTM_K_Matrix(atmosphere, surface, rts_k: Optional[Sequence[np.ndarray]], geometry,
                  channel_info: List[ChannelInfo], atmosphere_k: List[KMatrixBatch],
                  rts: List[RTSolutionBatch], options: Optional[OptionsBatch] = None) -> int:
    """CRTM_K_Matrix.  ``rts_k[i]`` is the (P, L_i) brightness-temperature seed of sensor i
    (None: 1); ``atmosphere_k`` receives the K-matrix per sensor (the surface Jacobians
    are in its water_temperature / surface_emissivity fields).  As the
    reference's INTENT(IN OUT) Atmosphere_K / Surface_K (CRTM_K_Matrix_Module.f90:
    300-322; the adjoints add into them, CRTM_Atmosphere.f90:583-586): a list
    holding one KMatrixBatch per sensor on entry is accumulated into (zero it
    first for the plain K-matrix); an empty list is filled."""
    accumulate = len(atmosphere_k) > 0
    if accumulate and len(atmosphere_k) != len(channel_info):
        print("CRTM_K_Matrix(FAILURE): atmosphere_k holds %d structures for %d sensors"
              % (len(atmosphere_k), len(channel_info)))
        return FAILURE
    given = list(atmosphere_k)
    atmosphere_k.clear()
    rts.clear()
    atmosphere, added = _added_layers(atmosphere, "CRTM_K_Matrix")
    if atmosphere is None:
        return FAILURE
    off = 0
    for i, ci in enumerate(channel_info):
        opt = _sensor_options(options, off, ci.n_channels)
        seed = None if rts_k is None else rts_k[i]
        try:
            km, r = ci.handle.k_matrix(atmosphere, surface, geometry, opt, seed, ci.sensor_index, components=True)
        except RuntimeError as e:
            print(f"CRTM_K_Matrix(FAILURE): {e}")
            return FAILURE
        if added.any:
            km = dataclasses.replace(km, **{f: addlayers.user_layers(added, getattr(km, f))
                                             for f in LAYER_FIELDS})
        if accumulate:
            try:
                km = _accumulate(given[i], km)
            except ValueError as e:
                print(f"CRTM_K_Matrix(FAILURE): {e}")
                return FAILURE
        atmosphere_k.append(km)
        rts.append(_user_layer_components(added, r))
        off += ci.n_channels
    return SUCCESS


def CRTM_Adjoint(atmosphere, surface, rts_ad: Sequence[np.ndarray], geometry,
                 channel_info: List[ChannelInfo], atmosphere_ad: dict, rts: List[RTSolutionBatch],
                 options: Optional[OptionsBatch] = None) -> int:
    """CRTM_Adjoint: adjoints summed over the channels of all sensors into
    ``atmosphere_ad``; arrays it holds on entry are accumulated into, as the
    reference's INTENT(IN OUT) Atmosphere_AD / Surface_AD (zero them first for
    the plain adjoint)."""
    rts.clear()
    atmosphere, added = _added_layers(atmosphere, "CRTM_Adjoint")
    if atmosphere is None:
        return FAILURE
    off = 0
    tot: dict = {}
    for i, ci in enumerate(channel_info):
        opt = _sensor_options(options, off, ci.n_channels)
        try:
            out, r = ci.handle.adjoint(atmosphere, surface, geometry, opt, rts_ad[i], ci.sensor_index,
                                       components=True)
        except RuntimeError as e:
            print(f"CRTM_Adjoint(FAILURE): {e}")
            return FAILURE
        if added.any:
            out = {k: addlayers.user_layers(added, v) if k in LAYER_FIELDS else v for k, v in out.items()}
        for k, v in out.items():
            tot[k] = tot[k] + v if k in tot else v.copy()
        rts.append(_user_layer_components(added, r))
        off += ci.n_channels
    for k, v in tot.items():
        prev = atmosphere_ad.get(k)
        if prev is not None:
            if np.shape(prev) != v.shape:
                print(f"CRTM_Adjoint(FAILURE): atmosphere_ad['{k}'] has shape {np.shape(prev)}, not {v.shape}")
                return FAILURE
            v = prev + v
        atmosphere_ad[k] = v
    return SUCCESS


def _accumulate(given: KMatrixBatch, new: KMatrixBatch) -> KMatrixBatch:
    """The caller's K-matrix structure plus this call's (fields the caller's
    structure lacks are taken as returned)."""
    out = {}
    for f in dataclasses.fields(KMatrixBatch):
        a, b = getattr(given, f.name), getattr(new, f.name)
        if a is not None and b is not None:
            if np.shape(a) != np.shape(b):
                raise ValueError(f"atmosphere_k field {f.name} has shape {np.shape(a)}, not {np.shape(b)}")
            b = a + b
        out[f.name] = b
    return KMatrixBatch(**out)


def CRTM_Tangent_Linear(atmosphere, surface, atmosphere_tl, surface_tl, geometry,
                        channel_info: List[ChannelInfo], rts: List[RTSolutionBatch], rts_tl: List[np.ndarray],
                        options: Optional[OptionsBatch] = None) -> int:
    """CRTM_Tangent_Linear (src/CRTM_Tangent_Linear_Module.f90:271): forward
    RTSolution and the brightness-temperature perturbations, one (P, L) array
    per sensor, from the atmosphere and surface perturbations."""
    rts.clear()
    rts_tl.clear()
    atmosphere, added = _added_layers(atmosphere, "CRTM_Tangent_Linear")
    if atmosphere is None:
        return FAILURE
    if added.any and atmosphere_tl is not None:
        atmosphere_tl = types.SimpleNamespace(**{
            f: addlayers.extend_perturbation(added, getattr(atmosphere_tl, f, None)) for f in LAYER_FIELDS})
    off = 0
    for ci in channel_info:
        opt = _sensor_options(options, off, ci.n_channels)
        try:
            bt_tl, r = ci.handle.tangent_linear(atmosphere, surface, geometry, opt, atmosphere_tl, surface_tl,
                                                sensor=ci.sensor_index, components=True)
        except RuntimeError as e:
            print(f"CRTM_Tangent_Linear(FAILURE): {e}")
            return FAILURE
        rts.append(_user_layer_components(added, r))
        rts_tl.append(bt_tl)
        off += ci.n_channels
    return SUCCESS


# layer-indexed fields of the K-matrix, adjoint and tangent-linear structures
LAYER_FIELDS = ("temperature", "absorber", "cloud_water_content", "cloud_effective_radius", "cloud_fraction",
                "aerosol_concentration", "aerosol_effective_radius", "aerosol_effective_variance",
                "relative_humidity")


def _added_layers(atmosphere: AtmosphereBatch, routine: str):
    """CRTM_Atmosphere_AddLayers before the call (CRTM_Forward_Module.f90:595,
    CRTM_K_Matrix_Module.f90:693): (extended batch, AddedLayers), or (None,
    None) after printing the failure."""
    try:
        return addlayers.add_layers(atmosphere)
    except ValueError as e:
        print(f"{routine}(FAILURE): {e}")
        return None, None


def _sensor_options(options: Optional[OptionsBatch], off: int, n: int) -> OptionsBatch:
    """One sensor's options: its columns of Options%Emissivity and every
    per-profile option.  Without an emissivity the library's surface model
    supplies it (the IR sea-surface model)."""
    if options is None:
        return OptionsBatch()
    if options.emissivity is None:
        return options
    return dataclasses.replace(options, emissivity=np.ascontiguousarray(options.emissivity[:, off:off + n]))
