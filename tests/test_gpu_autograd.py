"""The forward/adjoint pair behind torch.autograd (crtmv3_gb300.autograd):
torch's gradcheck (fast mode: random directional derivatives against central
differences) and the backward of a seeded sum against the K-matrix output."""
import numpy as np
import pytest

from crtmv3_gb300 import synthetic as sy

pytestmark = pytest.mark.gpu


def _setup(gpu_lib, coeff_dir, sensor, P, nl, seed):
    import torch
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, P, nl, seed)
    h = gpu_lib.CRTM([sensor], coeff_dir, 0)
    dev = torch.device("cuda", 0)
    t = {}
    for k in ("level_pressure", "pressure"):
        t[k] = torch.from_numpy(np.ascontiguousarray(getattr(atm, k))).to(dev)
    t["n_layers"] = torch.from_numpy(atm.n_layers.astype(np.int32)).to(dev)
    for f in ("land_coverage", "water_coverage", "snow_coverage", "ice_coverage", "land_temperature",
              "snow_temperature", "ice_temperature"):
        t[f] = torch.from_numpy(np.ascontiguousarray(getattr(sfc, f))).to(dev)
    for f in ("sensor_zenith_angle", "source_zenith_angle", "surface_altitude"):
        t[f] = torch.from_numpy(np.ascontiguousarray(getattr(geo, f))).to(dev)
    t["emissivity"] = torch.from_numpy(np.ascontiguousarray(opt.emissivity)).to(dev)
    T = torch.from_numpy(atm.temperature.copy()).to(dev).requires_grad_(True)
    A = torch.from_numpy(atm.absorber.copy()).to(dev).requires_grad_(True)
    W = torch.from_numpy(sfc.water_temperature.copy()).to(dev).requires_grad_(True)
    return h, t, atm, sfc, geo, opt, T, A, W


def test_gradcheck(gpu_lib, coeff_dir):
    import torch
    from crtmv3_gb300.autograd import brightness_temperature
    h, t, atm, sfc, geo, opt, T, A, W = _setup(gpu_lib, coeff_dir, "mwsynth_c16", 2, 60, 501)

    def f(T_, A_, W_):
        return brightness_temperature(h, t, atm.absorber_id, T_, A_, W_)
    assert torch.autograd.gradcheck(f, (T, A, W), eps=1e-6, atol=1e-6, rtol=1e-4, fast_mode=True)


def test_backward_equals_seeded_k_matrix(gpu_lib, coeff_dir):
    import torch
    from crtmv3_gb300.autograd import brightness_temperature
    h, t, atm, sfc, geo, opt, T, A, W = _setup(gpu_lib, coeff_dir, "irsynth_c616", 3, 101, 502)
    bt = brightness_temperature(h, t, atm.absorber_id, T, A, W)
    y = torch.randn(bt.shape, dtype=torch.float64, device=bt.device, generator=torch.Generator(bt.device).manual_seed(7))
    (bt * y).sum().backward()
    km, rts = h.k_matrix(atm, sfc, geo, opt)
    assert np.abs(bt.detach().cpu().numpy() - rts.brightness_temperature).max() < 1e-9
    yn = y.cpu().numpy()
    gT = np.einsum("pl,plk->pk", yn, km.temperature)
    gA = np.einsum("pl,pljk->pjk", yn, km.absorber)
    gW = np.einsum("pl,pl->p", yn, km.water_temperature)
    for got, ref in ((T.grad, gT), (A.grad, gA), (W.grad, gW)):
        got = got.cpu().numpy()
        assert np.abs(got - ref).max() <= 1e-10 * np.abs(ref).max()


def test_calls_on_other_streams_are_ordered(gpu_lib, coeff_dir):
    """A device call left running on one stream and a host call on the
    handle's own stream share the handle's workspace: the handle orders them."""
    import torch
    h, t, atm, sfc, geo, opt, T, A, W = _setup(gpu_lib, coeff_dir, "irsynth_c616", 3, 101, 503)
    P, K, L, J = atm.n_profiles, atm.max_layers, h.n_channels[0], atm.n_absorbers
    y = np.random.Generator(np.random.PCG64(5)).standard_normal((P, L))
    ref, _ = h.adjoint(atm, sfc, geo, opt, y)
    dev = dict(t, temperature=T.detach(), absorber=A.detach(), water_temperature=W.detach())
    b, keep = h.device_batch(dev, atm.absorber_id)
    f = dict(dtype=torch.float64, device="cuda")
    out = dict(radiance=torch.empty((P, L), **f), bt=torch.empty((P, L), **f),
               status=torch.empty((P,), dtype=torch.int32, device="cuda"),
               temperature_ad=torch.zeros((P, K), **f), absorber_ad=torch.zeros((P, J, K), **f),
               water_temperature_ad=torch.zeros((P,), **f))
    side = torch.cuda.Stream()
    h.adjoint_device(b, torch.from_numpy(y).cuda(), out, 0, side.cuda_stream)
    h.k_matrix(atm, sfc, geo, opt)          # host call on the handle's stream, no sync before it
    side.synchronize()
    assert np.abs(out["temperature_ad"].cpu().numpy() - ref["temperature"]).max() == 0.0
