"""crtm_gpu_k_matrix_device_static: the K-matrix with its intermediates in the
library's fixed per-device scratch (no device allocation inside the call),
against crtm_gpu_k_matrix_device on the same inputs, two calls in a row.

Tolerance: the two entry points run the same kernels on the same per-profile
data, so they agree to 1e-12 relative (to the largest value of each output)
in either precision; only the chunking of the batch differs.
"""
import os

import numpy as np
import pytest

from crtmv3_gb300 import coefficients as co, synthetic as sy

pytestmark = pytest.mark.gpu

TOL = 1e-12
FIELDS = ("radiance", "bt", "temperature_k", "absorber_k", "water_temperature_k",
          "surface_emissivity_k")


def _device_inputs(torch, h, atm, sfc, geo, opt):
    dev = torch.device("cuda")
    t = {k: torch.from_numpy(np.ascontiguousarray(getattr(atm, k))).to(dev)
         for k in ("level_pressure", "pressure", "temperature", "absorber")}
    t["n_layers"] = torch.from_numpy(atm.n_layers.astype(np.int32)).to(dev)
    for f in ("land_coverage", "water_coverage", "snow_coverage", "ice_coverage", "land_temperature",
              "water_temperature", "snow_temperature", "ice_temperature"):
        t[f] = torch.from_numpy(np.ascontiguousarray(getattr(sfc, f))).to(dev)
    for f in ("sensor_zenith_angle", "source_zenith_angle", "surface_altitude"):
        t[f] = torch.from_numpy(np.ascontiguousarray(getattr(geo, f))).to(dev)
    t["emissivity"] = torch.from_numpy(np.ascontiguousarray(opt.emissivity)).to(dev)
    b, keep = h.device_batch(t, atm.absorber_id)
    return b, keep, t


def _outputs(torch, P, L, K, J):
    f = dict(dtype=torch.float64, device="cuda")
    return dict(radiance=torch.full((P, L), np.nan, **f), bt=torch.full((P, L), np.nan, **f),
                temperature_k=torch.full((P, L, K), np.nan, **f),
                absorber_k=torch.full((P, L, J, K), np.nan, **f),
                water_temperature_k=torch.full((P, L), np.nan, **f),
                surface_emissivity_k=torch.full((P, L), np.nan, **f),
                status=torch.full((P,), -1, dtype=torch.int32, device="cuda"))


def _close(a, b):
    for f in FIELDS:
        x, y = a[f], b[f]
        assert not x.isnan().any(), f
        scale = max(float(y.abs().max()), 1e-300)
        assert float((x - y).abs().max()) <= TOL * scale, f
    assert int(a["status"].abs().max()) == 0


@pytest.mark.parametrize("sensor,P,precision", [("irsynth_c616", 8, 0), ("irsynth_c616", 8, 1),
                                                ("mwsynth_c22", 5, 0),
                                                # several chunks of the 128 MiB scratch
                                                ("irsynth_c2211", 16, 0)])
def test_static_scratch_matches_device_entry(gpu_lib, coeff_dir, sensor, P, precision):
    import torch
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, P, 101 if sensor.startswith("ir") else 100, 71)
    K, J = atm.max_layers, atm.n_absorbers
    ref_h = gpu_lib.CRTM([sensor], coeff_dir, precision)
    L = ref_h.n_channels[0]
    b, keep, t = _device_inputs(torch, ref_h, atm, sfc, geo, opt)
    stream = torch.cuda.current_stream().cuda_stream
    ref = _outputs(torch, P, L, K, J)
    ref_h.k_matrix_device(b, ref, None, 0, stream)
    torch.cuda.synchronize()

    # a fresh handle: its own workspace is never grown by the static entry point
    h = gpu_lib.CRTM([sensor], coeff_dir, precision)
    outs = [_outputs(torch, P, L, K, J) for _ in range(2)]
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for o in outs:
        h.k_matrix_device(b, o, None, 0, stream, static_scratch=True)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    for o in outs:
        _close(o, ref)
    # the regular entry point would grow a workspace of tens to hundreds of MB here
    assert free0 - free1 < (16 << 20)


def test_static_scratch_with_seed_and_absorber_selection(gpu_lib, coeff_dir):
    import torch
    sensor = "irsynth_c616"
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, 6, 101, 72)
    h = gpu_lib.CRTM([sensor], coeff_dir, 0)
    L, K = h.n_channels[0], atm.max_layers
    b, keep, t = _device_inputs(torch, h, atm, sfc, geo, opt)
    seed = torch.from_numpy(np.random.default_rng(3).normal(size=(6, L))).cuda()
    ids = list(atm.absorber_id)
    sel = [ids.index(co.O3_ID), ids.index(co.H2O_ID)]
    stream = torch.cuda.current_stream().cuda_stream
    ref = _outputs(torch, 6, L, K, 2)
    h.k_matrix_device(b, ref, seed, 0, stream, k_absorbers=sel)
    for _ in range(2):
        o = _outputs(torch, 6, L, K, 2)
        h.k_matrix_device(b, o, seed, 0, stream, k_absorbers=sel, static_scratch=True)
        torch.cuda.synchronize()
        _close(o, ref)


def test_static_scratch_rejects_oversized_profiles(gpu_lib, tmp_path):
    """One profile of 14000 channels x 200 layers with 6 absorber Jacobians in FP64
    needs about 157 MB of intermediates: more than the scratch holds.  The call
    fails before launching anything and the handle stays usable."""
    import torch
    sid = "wide_c14000"
    tc = sy.generate_odps(3, 14000, 5, sid, co.INFRARED_SENSOR, max_predictors_per_channel=1)
    sc = sy.generate_spccoeff(sid, co.INFRARED_SENSOR, 14000, 6)
    co.write_odps(os.path.join(tmp_path, f"{sid}.TauCoeff.bin"), tc)
    co.write_spccoeff(os.path.join(tmp_path, f"{sid}.SpcCoeff.bin"), sc)
    h = gpu_lib.CRTM([sid], str(tmp_path), 0)
    L = h.n_channels[0]
    atm, sfc, geo = sy.generate_profiles(1, 200, sy.absorber_set(1), 9)
    opt = sy.OptionsBatch(emissivity=sy.emissivity_for(co.INFRARED_SENSOR, 1, L, 10))
    b, keep, t = _device_inputs(torch, h, atm, sfc, geo, opt)
    stream = torch.cuda.current_stream().cuda_stream
    out = _outputs(torch, 1, L, 200, atm.n_absorbers)
    launches = h.launch_count()
    with pytest.raises(RuntimeError, match="static scratch holds"):
        h.k_matrix_device(b, out, None, 0, stream, static_scratch=True)
    assert h.launch_count() == launches
    # fewer layers fit: the same handle then succeeds and matches the regular entry point
    atm, sfc, geo = sy.generate_profiles(2, 60, sy.absorber_set(1), 11)
    opt = sy.OptionsBatch(emissivity=sy.emissivity_for(co.INFRARED_SENSOR, 2, L, 12))
    b, keep, t = _device_inputs(torch, h, atm, sfc, geo, opt)
    ref = _outputs(torch, 2, L, 60, atm.n_absorbers)
    h.k_matrix_device(b, ref, None, 0, stream)
    o = _outputs(torch, 2, L, 60, atm.n_absorbers)
    h.k_matrix_device(b, o, None, 0, stream, static_scratch=True)
    torch.cuda.synchronize()
    _close(o, ref)


def test_static_scratch_with_emissivity_model(gpu_lib, coeff_dir, tmp_path):
    """No batch emissivity: the IR sea-surface emissivity model's e, de/dv and
    de/dT arrays come from the static scratch too, so the call still grows no
    device memory, and its outputs (with the wind-speed Jacobian) match the
    regular entry point's."""
    import shutil

    import torch
    sensor = "irsynth_c616"
    for f in os.listdir(coeff_dir):
        if f.startswith(sensor):
            shutil.copy(os.path.join(coeff_dir, f), tmp_path)
    sy.write_irwater_file(str(tmp_path), "Nalli")
    P = 6
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, P, 101, 73)
    sfc.land_coverage[:] = sfc.snow_coverage[:] = sfc.ice_coverage[:] = 0.0
    sfc.water_coverage[:] = 1.0
    ref_h = gpu_lib.CRTM([sensor], str(tmp_path), 0)
    L, K, J = ref_h.n_channels[0], atm.max_layers, atm.n_absorbers
    b, keep, t = _device_inputs(torch, ref_h, atm, sfc, geo, opt)
    t["wind_speed"] = torch.from_numpy(np.linspace(1.0, 12.0, P)).cuda()
    t.pop("emissivity")
    b, keep = ref_h.device_batch(t, atm.absorber_id)
    stream = torch.cuda.current_stream().cuda_stream

    def outs():
        o = _outputs(torch, P, L, K, J)
        o["wind_speed_k"] = torch.full((P, L), np.nan, dtype=torch.float64, device="cuda")
        return o

    ref = outs()
    ref_h.k_matrix_device(b, ref, None, 0, stream)
    torch.cuda.synchronize()
    h = gpu_lib.CRTM([sensor], str(tmp_path), 0)
    runs = [outs() for _ in range(2)]
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for o in runs:
        h.k_matrix_device(b, o, None, 0, stream, static_scratch=True)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    for o in runs:
        _close(o, ref)
        scale = float(ref["wind_speed_k"].abs().max())
        assert scale > 0.0
        assert float((o["wind_speed_k"] - ref["wind_speed_k"]).abs().max()) <= TOL * scale
    assert free0 - free1 < (16 << 20)


def test_static_scratch_cloudy_and_aerosol_batch(gpu_lib, coeff_dir, tmp_path):
    """Clouds and aerosols: the scattering intermediates (FP64 layer records,
    adding states, species slots) fit the static scratch chunk by chunk and
    the species Jacobians match the regular entry point's."""
    import shutil

    import torch
    sensor = "irsynth_c616"
    for f in os.listdir(coeff_dir):
        if f.startswith(sensor):
            shutil.copy(os.path.join(coeff_dir, f), tmp_path)
    sy.write_cloud_files(str(tmp_path))
    sy.write_aerosol_files(str(tmp_path))
    P = 4
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, P, 100, 74)
    sy.add_clouds(atm, (co.WATER_CLOUD, co.ICE_CLOUD), 75)
    sy.add_aerosols(atm, sy.AEROSOL_TYPES, 76)
    ref_h = gpu_lib.CRTM([sensor], str(tmp_path), 0)
    L, K, J = ref_h.n_channels[0], atm.max_layers, atm.n_absorbers
    b, keep, t = _device_inputs(torch, ref_h, atm, sfc, geo, opt)
    for k in ("cloud_water_content", "cloud_effective_radius", "cloud_fraction", "aerosol_concentration",
              "aerosol_effective_radius"):
        t[k] = torch.from_numpy(np.ascontiguousarray(getattr(atm, k), np.float64)).cuda()
    for k in ("n_clouds", "cloud_type", "n_aerosols", "aerosol_type"):
        t[k] = torch.from_numpy(np.ascontiguousarray(getattr(atm, k), np.int32)).cuda()
    b, keep = ref_h.device_batch(t, atm.absorber_id)
    stream = torch.cuda.current_stream().cuda_stream
    NC, NA = atm.cloud_type.shape[1], atm.aerosol_type.shape[1]
    species = {"cloud_water_content_k": NC, "cloud_effective_radius_k": NC,
               "aerosol_concentration_k": NA, "aerosol_effective_radius_k": NA}

    def outs():
        o = _outputs(torch, P, L, K, J)
        for f, n in species.items():
            o[f] = torch.full((P, L, n, K), np.nan, dtype=torch.float64, device="cuda")
        return o

    ref = outs()
    ref_h.k_matrix_device(b, ref, None, 0, stream)
    torch.cuda.synchronize()
    h = gpu_lib.CRTM([sensor], str(tmp_path), 0)
    runs = [outs() for _ in range(2)]
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for o in runs:
        h.k_matrix_device(b, o, None, 0, stream, static_scratch=True)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    for o in runs:
        _close(o, ref)
        for f in species:
            scale = float(ref[f].abs().max())
            assert scale > 0.0, f
            assert float((o[f] - ref[f]).abs().max()) <= TOL * scale, f
    assert free0 - free1 < (16 << 20)
