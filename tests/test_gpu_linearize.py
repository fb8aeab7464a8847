"""The trajectory entry points for variational inner loops on the GPU
(crtm_gpu_linearize, crtm_gpu_tangent_linear_apply, crtm_gpu_adjoint_apply):
about one trajectory, the tangent linear and the adjoint applied from the
stored K-matrix give the same numbers as CRTM_Tangent_Linear and CRTM_Adjoint
on that trajectory (to rounding: the same Jacobians contracted in another
order), the forward of the trajectory is the forward, repeated applications
agree bit for bit, and a perturbation the trajectory holds no Jacobian for
is refused.  Clear sky, clouds with fractional cover and aerosols; FP64
form."""
import numpy as np
import pytest

from crtmv3_gb300 import coefficients as co, synthetic as sy

pytestmark = pytest.mark.gpu

ATM_TL = ("temperature", "absorber", "cloud_water_content", "cloud_effective_radius", "cloud_fraction",
          "aerosol_concentration", "aerosol_effective_radius")
SFC_TL = ("land_temperature", "water_temperature", "snow_temperature", "ice_temperature")


@pytest.fixture(scope="module")
def cloud_dir(coeff_dir):
    sy.write_cloud_files(coeff_dir)
    sy.write_aerosol_files(coeff_dir)
    return coeff_dir


def _case(kind):
    if kind == "clear":
        return ("irsynth_c616",) + sy.clear_sky_workload("irsynth_c616", 5, 101, 501)
    if kind == "clouds":
        sensor = "mwsynth_c16"
        atm, sfc, geo, opt = sy.cloudy_workload(sensor, 5, 100, 502, wc_scale=100.0)
        sy.add_clouds(atm, (co.WATER_CLOUD, co.RAIN_CLOUD, co.SNOW_CLOUD), 503, wc_scale=100.0, cover=(0.2, 0.9))
        atm.n_clouds[3] = 0
        return (sensor, atm, sfc, geo, opt)
    sensor = "irsynth_c616"
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, 4, 101, 504)
    sy.add_clouds(atm, (co.WATER_CLOUD, co.ICE_CLOUD), 505, wc_scale=30.0)
    sy.add_aerosols(atm, sy.AEROSOL_TYPES, 506, load_scale=20.0)
    return (sensor, atm, sfc, geo, opt)


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("kind", ["clear", "clouds", "aerosols"])
def test_apply_matches_tangent_linear_and_adjoint(gpu_lib, cloud_dir, kind):
    import torch
    import bench
    dev = torch.device("cuda")
    sensor, atm, sfc, geo, opt = _case(kind)
    h = gpu_lib.CRTM([sensor], cloud_dir, 0)
    P, L, K = atm.n_profiles, h.n_channels[0], atm.max_layers
    sfc.land_coverage[:] = 0.2
    sfc.water_coverage[:] = 0.6
    sfc.snow_coverage[:] = 0.1
    sfc.ice_coverage[:] = 0.1
    b, keep, t = bench.scatter_device_inputs(torch, h, atm, sfc, geo, opt, dev)
    f64 = dict(dtype=torch.float64, device=dev)
    traj = dict(radiance=torch.zeros((P, L), **f64), bt=torch.zeros((P, L), **f64),
                status=torch.full((P,), -1, dtype=torch.int32, device=dev))
    stream = torch.cuda.current_stream().cuda_stream
    h.linearize_device(b, traj, 0, stream)
    torch.cuda.synchronize()
    fw = h.forward(atm, sfc, geo, opt)
    assert np.abs(traj["bt"].cpu().numpy() - fw.brightness_temperature).max() < 1e-9
    assert not traj["status"].cpu().numpy().any()

    rng = np.random.Generator(np.random.PCG64(507))
    d = {}
    for f in ATM_TL:
        v = getattr(atm, f, None)
        if v is not None:
            d[f] = rng.uniform(-0.05, 0.05, v.shape) * (v if f != "temperature" else 20.0)
    if atm.cloud_fraction is not None:
        d["cloud_fraction"] = np.where(atm.cloud_fraction > 0, d["cloud_fraction"], 0.0)
    for f in SFC_TL:
        d[f] = rng.standard_normal(P)
    d["emissivity"] = rng.uniform(-0.01, 0.01, (P, L))

    class NS:
        pass
    atm_tl, sfc_tl = NS(), NS()
    for f in ATM_TL:
        setattr(atm_tl, f, d.get(f))
    for f in SFC_TL:
        setattr(sfc_tl, f, d[f])
    ref_tl, _ = h.tangent_linear(atm, sfc, geo, opt, atm_tl, sfc_tl, d["emissivity"])

    tl = {f: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for f, v in d.items()}
    bt_tl = torch.zeros((P, L), **f64)
    h.tangent_linear_apply_device(tl, bt_tl, stream)
    torch.cuda.synchronize()
    got = bt_tl.cpu().numpy()
    assert _rel(got, ref_tl) <= 1e-12
    # an inner loop applies it again: the same bits
    bt2 = torch.zeros((P, L), **f64)
    h.tangent_linear_apply_device(tl, bt2, stream)
    torch.cuda.synchronize()
    assert np.array_equal(bt2.cpu().numpy(), got)

    seed = rng.standard_normal((P, L))
    ref_ad, _ = h.adjoint(atm, sfc, geo, opt, seed)
    out = dict(temperature_ad=torch.zeros((P, K), **f64),
               absorber_ad=torch.zeros((P, atm.n_absorbers, K), **f64),
               water_temperature_ad=torch.zeros((P,), **f64))
    for f in ("land_temperature", "snow_temperature", "ice_temperature"):
        out[f + "_ad"] = torch.zeros((P,), **f64)
    if atm.cloud_type is not None:
        NC = atm.cloud_type.shape[1]
        out["cloud_water_content_ad"] = torch.zeros((P, NC, K), **f64)
        out["cloud_effective_radius_ad"] = torch.zeros((P, NC, K), **f64)
        out["cloud_fraction_ad"] = torch.zeros((P, K), **f64)
    if atm.aerosol_type is not None:
        NA = atm.aerosol_type.shape[1]
        out["aerosol_concentration_ad"] = torch.zeros((P, NA, K), **f64)
        out["aerosol_effective_radius_ad"] = torch.zeros((P, NA, K), **f64)
    h.adjoint_apply_device(torch.from_numpy(seed).to(dev), out, stream)
    torch.cuda.synchronize()
    pairs = [("temperature_ad", "temperature"), ("absorber_ad", "absorber"),
             ("water_temperature_ad", "water_temperature")]
    pairs += [(f + "_ad", f) for f in ("land_temperature", "snow_temperature", "ice_temperature",
                                       "cloud_water_content", "cloud_effective_radius", "cloud_fraction",
                                       "aerosol_concentration", "aerosol_effective_radius")]
    checked = 0
    for mine, ref in pairs:
        if mine in out and ref in ref_ad:
            assert _rel(out[mine].cpu().numpy(), ref_ad[ref]) <= 1e-12, mine
            checked += 1
    assert checked >= 3


def test_apply_refuses_jacobians_the_trajectory_lacks(gpu_lib, cloud_dir):
    import torch
    import bench
    dev = torch.device("cuda")
    sensor, atm, sfc, geo, opt = _case("clear")
    h = gpu_lib.CRTM([sensor], cloud_dir, 0)
    P, L = atm.n_profiles, h.n_channels[0]
    b, keep, t = bench.scatter_device_inputs(torch, h, atm, sfc, geo, opt, dev)
    f64 = dict(dtype=torch.float64, device=dev)
    with pytest.raises(RuntimeError, match="trajectory"):
        h.tangent_linear_apply_device({"temperature": torch.zeros(atm.temperature.shape, **f64)},
                                      torch.zeros((P, L), **f64))
    traj = dict(radiance=torch.zeros((P, L), **f64), bt=torch.zeros((P, L), **f64))
    h.linearize_device(b, traj)
    with pytest.raises(RuntimeError, match="cloud water content"):
        h.tangent_linear_apply_device({"cloud_water_content": torch.zeros((P, 1, atm.max_layers), **f64)},
                                      torch.zeros((P, L), **f64))
