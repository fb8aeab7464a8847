"""ctypes binding of the CPU FP64 oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module; it is the checker, never the product.  Parity unpinned: see
crtm_oracle.h.
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess

import numpy as np
from typing import Optional

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

_dp = ct.POINTER(ct.c_double)
_ip = ct.POINTER(ct.c_int)


class OrBatch(ct.Structure):
    _fields_ = [("n_profiles", ct.c_int), ("max_layers", ct.c_int), ("n_layers", _ip),
                ("n_absorbers", ct.c_int), ("absorber_id", _ip),
                ("level_pressure", _dp), ("pressure", _dp), ("temperature", _dp),
                ("absorber", _dp),
                ("surface_land_coverage", _dp), ("surface_water_coverage", _dp),
                ("surface_snow_coverage", _dp), ("surface_ice_coverage", _dp),
                ("surface_land_temperature", _dp), ("surface_water_temperature", _dp),
                ("surface_snow_temperature", _dp), ("surface_ice_temperature", _dp),
                ("sensor_zenith_angle", _dp), ("source_zenith_angle", _dp),
                ("surface_altitude", _dp), ("emissivity", _dp), ("k_absorber_mask", _ip)]


class OrRtsExt(ct.Structure):
    _fields_ = [(f, ct.c_void_p) for f in (
        "tb_clear", "r_clear", "total_cloud_cover", "sod", "surface_emissivity", "up_radiance", "down_radiance",
        "surface_planck_radiance", "n_full_streams", "layer_optical_depth", "upwelling_radiance",
        "upwelling_overcast_radiance")]


class OrClouds(ct.Structure):
    _fields_ = [("max_clouds", ct.c_int), ("n_clouds", _ip), ("cloud_type", _ip),
                ("water_content", _dp), ("effective_radius", _dp), ("n_streams", _ip),
                ("rt_algorithm", _ip), ("max_aerosols", ct.c_int), ("n_aerosols", _ip),
                ("aerosol_type", _ip), ("aerosol_concentration", _dp), ("aerosol_effective_radius", _dp),
                ("cloud_fraction", _dp), ("overlap", _ip), ("aerosol_effective_variance", _dp),
                ("relative_humidity", _dp)]


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("crtm_oracle.c", "crtm_oracle.h", "oracle_scatter.inc",
                                             "oracle_scatter_k.inc", "oracle_optran.inc")]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(LIB) < os.path.getmtime(f) for f in srcs):
        subprocess.run(["make", "-C", HERE, "-B", "liboracle.so"], check=True,
                       stdout=subprocess.DEVNULL)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ct.CDLL(LIB)
        L.or_init.restype = ct.c_void_p
        L.or_init.argtypes = [ct.c_char_p, ct.c_char_p]
        L.or_destroy.argtypes = [ct.c_void_p]
        L.or_n_channels.argtypes = [ct.c_void_p]
        L.or_last_error.restype = ct.c_char_p
        L.or_forward.argtypes = [ct.c_void_p, ct.POINTER(OrBatch), _dp, _dp, _dp, ct.c_int]
        L.or_k_matrix.argtypes = [ct.c_void_p, ct.POINTER(OrBatch), _dp, _dp, _dp, _dp, _dp, _dp,
                                  _dp, ct.c_int]
        L.or_adjoint.argtypes = [ct.c_void_p, ct.POINTER(OrBatch), _dp, _dp, _dp, _dp, _dp, _dp,
                                 ct.c_int]
        L.or_tangent_fd.argtypes = [ct.c_void_p, ct.POINTER(OrBatch), _dp, _dp, _dp, ct.c_double,
                                    _dp, ct.c_int]
        L.or_cloud_init.restype = ct.c_void_p
        L.or_cloud_init.argtypes = [ct.c_char_p]
        L.or_cloud_destroy.argtypes = [ct.c_void_p]
        L.or_forward_scatter.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.POINTER(OrBatch),
                                         ct.POINTER(OrClouds), _dp, _dp, ct.c_int]
        L.or_forward_ext.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.POINTER(OrBatch),
                                     ct.POINTER(OrClouds), _dp, _dp, ct.POINTER(OrRtsExt), ct.c_int]
        L.or_k_matrix_scatter.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.POINTER(OrBatch),
                                          ct.POINTER(OrClouds)] + [_dp] * 11 + [ct.c_int]
        L.or_aerosol_init.restype = ct.c_void_p
        L.or_aerosol_init.argtypes = [ct.c_char_p]
        L.or_aerosol_init_scheme.restype = ct.c_void_p
        L.or_aerosol_init_scheme.argtypes = [ct.c_char_p, ct.c_char_p]
        L.or_aerosol_destroy.argtypes = [ct.c_void_p]
        L.or_irwater_init.restype = ct.c_void_p
        L.or_irwater_init.argtypes = [ct.c_char_p]
        L.or_irwater_destroy.argtypes = [ct.c_void_p]
        L.or_irssem.restype = ct.c_double
        L.or_irssem.argtypes = [ct.c_void_p, ct.c_double, ct.c_double, ct.c_double, ct.c_double]
        L.or_amom_layer.argtypes = [ct.c_int, ct.c_int, ct.c_double, ct.c_double, _dp, _dp, _dp, _dp,
                                    ct.c_double, _dp, _dp, _dp]
        L.or_phase_setup.argtypes = [ct.c_int, ct.c_double, _dp, _dp, _dp, _dp, _dp, _ip]
        L.or_add_layers.argtypes = [ct.c_int, _dp, _dp, _dp, ct.c_int, ct.c_double, _dp, _dp, _dp,
                                    _dp, _dp, _dp, _dp]
        _lib = L
    return _lib


def _p(a, t=_dp):
    return None if a is None else a.ctypes.data_as(t)


class Oracle:
    """One sensor's coefficients, loaded by the oracle from the binary files."""

    def __init__(self, coeff_dir: str, sensor_id: str):
        L = lib()
        self.h = L.or_init(coeff_dir.encode(), sensor_id.encode())
        if not self.h:
            raise IOError(L.or_last_error().decode())
        self.n_channels = L.or_n_channels(self.h)

    def close(self):
        if self.h:
            lib().or_destroy(self.h)
            self.h = None

    __del__ = close

    def _batch(self, atm, sfc, geo, opt):
        keep = []

        def c(a, dt=np.float64):
            a = np.ascontiguousarray(a, dtype=dt)
            keep.append(a)
            return a
        b = OrBatch()
        b.n_profiles = atm.n_profiles
        b.max_layers = atm.max_layers
        b.n_layers = _p(c(atm.n_layers, np.int32), _ip)
        b.n_absorbers = atm.n_absorbers
        b.absorber_id = _p(c(atm.absorber_id, np.int32), _ip)
        b.level_pressure = _p(c(atm.level_pressure))
        b.pressure = _p(c(atm.pressure))
        b.temperature = _p(c(atm.temperature))
        b.absorber = _p(c(atm.absorber))
        for f in ("land_coverage", "water_coverage", "snow_coverage", "ice_coverage",
                  "land_temperature", "water_temperature", "snow_temperature", "ice_temperature"):
            setattr(b, "surface_" + f, _p(c(getattr(sfc, f))))
        b.sensor_zenith_angle = _p(c(geo.sensor_zenith_angle))
        b.source_zenith_angle = _p(c(geo.source_zenith_angle))
        b.surface_altitude = _p(c(geo.surface_altitude))
        b.emissivity = _p(c(opt.emissivity))
        return b, keep

    def forward(self, atm, sfc, geo, opt, n_threads: int = 1, layer_od: bool = False):
        P, L, K = atm.n_profiles, self.n_channels, atm.max_layers
        b, keep = self._batch(atm, sfc, geo, opt)
        rad = np.zeros((P, L))
        bt = np.zeros((P, L))
        od = np.zeros((P, L, K)) if layer_od else None
        st = lib().or_forward(self.h, ct.byref(b), _p(rad), _p(bt), _p(od), n_threads)
        if st:
            raise RuntimeError(lib().or_last_error().decode())
        return (rad, bt, od) if layer_od else (rad, bt)

    def k_matrix(self, atm, sfc, geo, opt, bt_k=None, n_threads: int = 1, k_absorbers=None):
        """``k_absorbers``: user absorber indices whose Jacobians are computed
        (default all); the other absorbers' Jacobians are returned as zeros."""
        P, L, K, J = atm.n_profiles, self.n_channels, atm.max_layers, atm.n_absorbers
        b, keep = self._batch(atm, sfc, geo, opt)
        if k_absorbers is not None:
            mask = np.zeros(J, np.int32)
            mask[np.asarray(k_absorbers, int)] = 1
            keep.append(mask)
            b.k_absorber_mask = _p(mask, _ip)
        seed = None if bt_k is None else np.ascontiguousarray(bt_k, np.float64)
        rad, bt = np.zeros((P, L)), np.zeros((P, L))
        tk, ak = np.zeros((P, L, K)), np.zeros((P, L, J, K))
        tsk, ek = np.zeros((P, L)), np.zeros((P, L))
        st = lib().or_k_matrix(self.h, ct.byref(b), _p(seed), _p(rad), _p(bt), _p(tk), _p(ak),
                               _p(tsk), _p(ek), n_threads)
        if st:
            raise RuntimeError(lib().or_last_error().decode())
        return dict(radiance=rad, bt=bt, temperature_k=tk, absorber_k=ak,
                    water_temperature_k=tsk, surface_emissivity_k=ek)

    def adjoint(self, atm, sfc, geo, opt, bt_ad, n_threads: int = 1):
        P, L, K, J = atm.n_profiles, self.n_channels, atm.max_layers, atm.n_absorbers
        b, keep = self._batch(atm, sfc, geo, opt)
        seed = np.ascontiguousarray(bt_ad, np.float64)
        rad, bt = np.zeros((P, L)), np.zeros((P, L))
        ta, aa, wa = np.zeros((P, K)), np.zeros((P, J, K)), np.zeros(P)
        st = lib().or_adjoint(self.h, ct.byref(b), _p(seed), _p(rad), _p(bt), _p(ta), _p(aa),
                              _p(wa), n_threads)
        if st:
            raise RuntimeError(lib().or_last_error().decode())
        return dict(radiance=rad, bt=bt, temperature_ad=ta, absorber_ad=aa, water_temperature_ad=wa)

    @staticmethod
    def _clouds(atm, opt, keep):
        """The or_clouds structure of a batch (arrays kept alive in ``keep``)."""
        P = atm.n_profiles
        c = OrClouds()

        def arr(a, dt=np.float64):
            a = np.ascontiguousarray(a, dt)
            keep.append(a)
            return a
        if atm.cloud_type is not None and atm.cloud_type.shape[1] > 0:
            c.max_clouds = int(atm.cloud_type.shape[1])
            c.n_clouds = _p(arr(atm.n_clouds, np.int32), _ip)
            c.cloud_type = _p(arr(atm.cloud_type, np.int32), _ip)
            c.water_content = _p(arr(atm.cloud_water_content))
            c.effective_radius = _p(arr(atm.cloud_effective_radius))
        if atm.aerosol_type is not None and atm.aerosol_type.shape[1] > 0:
            c.max_aerosols = int(atm.aerosol_type.shape[1])
            c.n_aerosols = _p(arr(atm.n_aerosols, np.int32), _ip)
            c.aerosol_type = _p(arr(atm.aerosol_type, np.int32), _ip)
            c.aerosol_concentration = _p(arr(atm.aerosol_concentration))
            c.aerosol_effective_radius = _p(arr(atm.aerosol_effective_radius))
            if getattr(atm, "aerosol_effective_variance", None) is not None:
                c.aerosol_effective_variance = _p(arr(atm.aerosol_effective_variance))
            if getattr(atm, "relative_humidity", None) is not None:
                c.relative_humidity = _p(arr(atm.relative_humidity))
        if opt.n_streams is not None:
            use = opt.use_n_streams if opt.use_n_streams is not None else np.ones(P, bool)
            c.n_streams = _p(arr(np.where(use, opt.n_streams, 0), np.int32), _ip)
        if opt.rt_algorithm_id is not None:
            c.rt_algorithm = _p(arr(opt.rt_algorithm_id, np.int32), _ip)
        if c.max_clouds > 0 and atm.cloud_fraction is not None:
            c.cloud_fraction = _p(arr(atm.cloud_fraction))
        if getattr(opt, "overlap_id", None) is not None:
            c.overlap = _p(arr(opt.overlap_id, np.int32), _ip)
        return c

    @staticmethod
    def _luts(cloudcoeff_path, aerosolcoeff_path, aerosol_scheme):
        L = lib()
        ch = ah = None
        if cloudcoeff_path:
            ch = L.or_cloud_init(cloudcoeff_path.encode())
            if not ch:
                raise IOError(L.or_last_error().decode())
        if aerosolcoeff_path:
            ah = L.or_aerosol_init_scheme(aerosolcoeff_path.encode(), aerosol_scheme.encode())
            if not ah:
                if ch:
                    L.or_cloud_destroy(ch)
                raise IOError(L.or_last_error().decode())
        return ch, ah

    def forward_scatter(self, atm, sfc, geo, opt, cloudcoeff_path: Optional[str] = None,
                        aerosolcoeff_path: Optional[str] = None, n_threads: int = 1,
                        aerosol_scheme: str = "CRTM"):
        """Forward with clouds and aerosols (ADA or SOI per Options%RT_Algorithm_Id);
        profiles without either take the Emission solver.  aerosol_scheme is
        CRTM_Init's Aerosol_Model for the AerosolCoeff file."""
        L = lib()
        ch, ah = self._luts(cloudcoeff_path, aerosolcoeff_path, aerosol_scheme)
        try:
            P, nL = atm.n_profiles, self.n_channels
            b, keep = self._batch(atm, sfc, geo, opt)
            c = self._clouds(atm, opt, keep)
            rad, bt = np.zeros((P, nL)), np.zeros((P, nL))
            st = L.or_forward_scatter(self.h, ch, ah, ct.byref(b), ct.byref(c), _p(rad), _p(bt), n_threads)
            if st:
                raise RuntimeError(L.or_last_error().decode())
            return rad, bt
        finally:
            if ch:
                L.or_cloud_destroy(ch)
            if ah:
                L.or_aerosol_destroy(ah)

    def forward_components(self, atm, sfc, geo, opt, cloudcoeff_path: Optional[str] = None,
                           aerosolcoeff_path: Optional[str] = None, n_threads: int = 1,
                           aerosol_scheme: str = "CRTM") -> dict:
        """CRTM_Forward's radiance, brightness temperature and further
        RTSolution components (or_forward_ext) of a batch with or without
        clouds and aerosols: a dict of (P, L) arrays and (P, L, max_layers)
        layer arrays under the names of include/crtm_gpu.h."""
        L = lib()
        ch, ah = self._luts(cloudcoeff_path, aerosolcoeff_path, aerosol_scheme)
        try:
            P, nL, K = atm.n_profiles, self.n_channels, atm.max_layers
            b, keep = self._batch(atm, sfc, geo, opt)
            c = self._clouds(atm, opt, keep)
            out = dict(radiance=np.zeros((P, nL)), bt=np.zeros((P, nL)))
            x = OrRtsExt()
            for f, _ in OrRtsExt._fields_:
                shape = (P, nL, K) if f in ("layer_optical_depth", "upwelling_radiance",
                                            "upwelling_overcast_radiance") else (P, nL)
                a = np.zeros(shape, np.int32 if f == "n_full_streams" else np.float64)
                out[f] = a
                setattr(x, f, a.ctypes.data)
            st = L.or_forward_ext(self.h, ch, ah, ct.byref(b), ct.byref(c), _p(out["radiance"]), _p(out["bt"]),
                                  ct.byref(x), n_threads)
            if st:
                raise RuntimeError(L.or_last_error().decode())
            return out
        finally:
            if ch:
                L.or_cloud_destroy(ch)
            if ah:
                L.or_aerosol_destroy(ah)

    def k_matrix_scatter(self, atm, sfc, geo, opt, cloudcoeff_path: Optional[str] = None,
                         aerosolcoeff_path: Optional[str] = None, bt_k=None, n_threads: int = 1,
                         aerosol_scheme: str = "CRTM", k_absorbers=None):
        """K-matrix of a batch with clouds and aerosols through ADA (the
        oracle's reverse mode of the reference's ADA, MOM, phase, combine and
        LUT adjoints), dict with the clear-sky K-matrix keys plus
        cloud_water_content_k, cloud_effective_radius_k [P][L][NC][Kmax] and
        aerosol_concentration_k, aerosol_effective_radius_k [P][L][NA][Kmax]
        (the latter: relative humidity for 'GOCART-GEOS5' / 'NAAPS')."""
        L = lib()
        ch, ah = self._luts(cloudcoeff_path, aerosolcoeff_path, aerosol_scheme)
        try:
            P, nL, K, J = atm.n_profiles, self.n_channels, atm.max_layers, atm.n_absorbers
            b, keep = self._batch(atm, sfc, geo, opt)
            if k_absorbers is not None:
                mask = np.zeros(J, np.int32)
                mask[np.asarray(k_absorbers, int)] = 1
                keep.append(mask)
                b.k_absorber_mask = _p(mask, _ip)
            c = self._clouds(atm, opt, keep)
            NC, NA = max(c.max_clouds, 0), max(c.max_aerosols, 0)
            seed = None if bt_k is None else np.ascontiguousarray(bt_k, np.float64)
            o = dict(radiance=np.zeros((P, nL)), bt=np.zeros((P, nL)), temperature_k=np.zeros((P, nL, K)),
                     absorber_k=np.zeros((P, nL, J, K)), water_temperature_k=np.zeros((P, nL)),
                     surface_emissivity_k=np.zeros((P, nL)),
                     cloud_water_content_k=np.zeros((P, nL, NC, K)), cloud_effective_radius_k=np.zeros((P, nL, NC, K)),
                     aerosol_concentration_k=np.zeros((P, nL, NA, K)),
                     aerosol_effective_radius_k=np.zeros((P, nL, NA, K)))
            st = L.or_k_matrix_scatter(self.h, ch, ah, ct.byref(b), ct.byref(c), _p(seed), _p(o["radiance"]),
                                       _p(o["bt"]), _p(o["temperature_k"]), _p(o["absorber_k"]),
                                       _p(o["water_temperature_k"]), _p(o["surface_emissivity_k"]),
                                       _p(o["cloud_water_content_k"]) if NC else None,
                                       _p(o["cloud_effective_radius_k"]) if NC else None,
                                       _p(o["aerosol_concentration_k"]) if NA else None,
                                       _p(o["aerosol_effective_radius_k"]) if NA else None, n_threads)
            if st:
                raise RuntimeError(L.or_last_error().decode())
            return o
        finally:
            if ch:
                L.or_cloud_destroy(ch)
            if ah:
                L.or_aerosol_destroy(ah)

    def tangent_fd(self, atm, sfc, geo, opt, t_tl, a_tl, ts_tl, step=1e-4, n_threads: int = 1):
        P, L = atm.n_profiles, self.n_channels
        b, keep = self._batch(atm, sfc, geo, opt)
        t_tl = np.ascontiguousarray(t_tl, np.float64)
        a_tl = np.ascontiguousarray(a_tl, np.float64)
        ts_tl = np.ascontiguousarray(ts_tl, np.float64)
        out = np.zeros((P, L))
        st = lib().or_tangent_fd(self.h, ct.byref(b), _p(t_tl), _p(a_tl), _p(ts_tl), step, _p(out),
                                 n_threads)
        if st:
            raise RuntimeError(lib().or_last_error().decode())
        return out


def irwater_emissivity(path: str, sfc, geo, frequency) -> np.ndarray:
    """(P, L) IR sea-surface emissivities at each profile's sensor zenith angle
    (CRTM_IRSSEM through the oracle) from Surface%Water_Temperature and
    %Wind_Speed (5 m/s when absent) and the channel frequencies (cm^-1)."""
    L = lib()
    h = L.or_irwater_init(path.encode())
    if not h:
        raise IOError(L.or_last_error().decode())
    try:
        P = sfc.water_temperature.shape[0]
        wind = sfc.wind_speed if getattr(sfc, "wind_speed", None) is not None else np.full(P, 5.0)
        out = np.zeros((P, len(frequency)))
        for m in range(P):
            for c, f in enumerate(frequency):
                out[m, c] = L.or_irssem(h, float(sfc.water_temperature[m]), float(wind[m]), float(f),
                                        float(geo.sensor_zenith_angle[m]))
        return out
    finally:
        L.or_irwater_destroy(h)


def add_layers_profile(model_p, model_t, model_a, top, user_p, user_t, user_a):
    """The oracle's CRTM_Atmosphere_AddLayers for one profile: (pl (n+1,),
    p (n,), t (n,), a (J, n)); n = 0 gives empty arrays.  model_a (J, nlev):
    the climatology's rows for the profile's absorbers; user_p, user_t (2,) and
    user_a (J, 2): the profile's first two layers."""
    L = lib()
    mp = np.ascontiguousarray(model_p, np.float64)
    mt = np.ascontiguousarray(model_t, np.float64)
    ma = np.ascontiguousarray(model_a, np.float64)
    J, nlev = ma.shape
    up = np.ascontiguousarray(user_p[:2], np.float64)
    ut = np.ascontiguousarray(user_t[:2], np.float64)
    ua = np.ascontiguousarray(np.asarray(user_a, np.float64)[:, :2])
    pl = np.zeros(nlev)
    p = np.zeros(nlev)
    t = np.zeros(nlev)
    a = np.zeros(J * nlev)
    n = L.or_add_layers(nlev, _p(mp), _p(mt), _p(ma), J, float(top), _p(up), _p(ut), _p(ua),
                        _p(pl), _p(p), _p(t), _p(a))
    return pl[:n + 1] if n else pl[:0], p[:n], t[:n], a[:J * n].reshape(J, n)
