"""Pipeline tuning and the autotuner (crtm_gpu_set_tuning / crtm_gpu_get_tuning /
crtm_gpu_autotune_k_matrix_device) on device buffers.

The channels per map CTA and the cap on profiles per pipeline pass change only
the work decomposition, so a tuned handle gives the K-matrix of a default one:
1e-12 relative to the largest value of each output (in practice bit-equal).
"""
import numpy as np
import pytest

from crtmv3_gb300 import synthetic as sy

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


def _case(gpu_lib, coeff_dir, precision, P=8):
    import torch
    sensor = "irsynth_c616"
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, P, 101, 81)
    K, J = atm.max_layers, atm.n_absorbers
    ref_h = gpu_lib.CRTM([sensor], coeff_dir, precision)
    L = ref_h.n_channels[0]
    b, keep, t = _device_inputs(torch, ref_h, atm, sfc, geo, opt)
    stream = torch.cuda.current_stream().cuda_stream
    ref = _outputs(torch, P, L, K, J)
    ref_h.k_matrix_device(b, ref, None, 0, stream)
    torch.cuda.synchronize()
    return dict(sensor=sensor, P=P, L=L, K=K, J=J, b=b, keep=keep, t=t, stream=stream, ref=ref)


@pytest.mark.parametrize("precision", [0, 1])
def test_autotune_picks_a_measured_candidate_and_keeps_the_results(gpu_lib, coeff_dir, precision):
    import torch
    c = _case(gpu_lib, coeff_dir, precision)
    h = gpu_lib.CRTM([c["sensor"]], coeff_dir, precision)
    assert h.tuning() == dict(map_channels=16, chunk_profiles=0, ms_per_call=0.0)
    out = _outputs(torch, c["P"], c["L"], c["K"], c["J"])
    res = h.autotune_k_matrix_device(c["b"], out, None, 0, c["stream"], reps=1)
    torch.cuda.synchronize()
    _close(out, c["ref"])
    trials = res["trials"]
    # 8 profiles: caps none, 4 and 2 for each of 16, 8 and 32 channels per map CTA
    assert {(t["map_channels"], t["chunk_profiles"]) for t in trials} == \
        {(m, cap) for m in (16, 8, 32) for cap in (0, 4, 2)}
    assert all(t["ms_per_call"] > 0 for t in trials)
    best = res["chosen"]
    assert best["ms_per_call"] == min(t["ms_per_call"] for t in trials)
    assert h.tuning() == best
    # the other form keeps its default
    assert h.tuning(precision=1 - precision)["chunk_profiles"] == 0
    out2 = _outputs(torch, c["P"], c["L"], c["K"], c["J"])
    h.k_matrix_device(c["b"], out2, None, 0, c["stream"])
    torch.cuda.synchronize()
    _close(out2, c["ref"])


def test_set_tuning_splits_the_passes_without_changing_results(gpu_lib, coeff_dir):
    import torch
    c = _case(gpu_lib, coeff_dir, 0)
    h = gpu_lib.CRTM([c["sensor"]], coeff_dir, 0)
    out = _outputs(torch, c["P"], c["L"], c["K"], c["J"])
    n0 = h.launch_count()
    h.k_matrix_device(c["b"], out, None, 0, c["stream"])
    one_pass = h.launch_count() - n0
    h.set_tuning(map_channels=8, chunk_profiles=2)
    assert h.tuning() == dict(map_channels=8, chunk_profiles=2, ms_per_call=0.0)
    out = _outputs(torch, c["P"], c["L"], c["K"], c["J"])
    n0 = h.launch_count()
    h.k_matrix_device(c["b"], out, None, 0, c["stream"])
    torch.cuda.synchronize()
    assert h.launch_count() - n0 == 4 * one_pass   # 8 profiles in passes of 2
    _close(out, c["ref"])
    with pytest.raises(RuntimeError, match="map_channels"):
        h.set_tuning(map_channels=12)
    with pytest.raises(RuntimeError, match="chunk_profiles"):
        h.set_tuning(chunk_profiles=-1)
    assert h.tuning()["map_channels"] == 8
