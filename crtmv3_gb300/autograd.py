"""torch.autograd binding of the library's forward and adjoint (a thin harness).

``brightness_temperature(handle, batch, temperature, absorber, water_temperature)``
returns the (P, L) brightness temperatures of ``batch`` (a dict of device
tensors with the batch fields, as ``CRTM.device_batch`` takes them) with the
given temperature (P, K), absorber (P, J, K) and water temperature (P) in
place of the batch's; backward runs ``crtm_gpu_adjoint_device`` with the
incoming gradient as the brightness-temperature seed (CRTM_Adjoint,
src/CRTM_Adjoint_Module.f90:299-309).  Everything stays on the GPU.
"""
from __future__ import annotations

import numpy as np
import torch


def _run(handle, sensor, batch, absorber_id, temperature, absorber, water_temperature):
    dev = dict(batch)
    dev["temperature"] = temperature.contiguous()
    dev["absorber"] = absorber.contiguous()
    dev["water_temperature"] = water_temperature.contiguous()
    b, keep = handle.device_batch(dev, absorber_id)
    return dev, b, keep


class _BrightnessTemperature(torch.autograd.Function):
    @staticmethod
    def forward(ctx, temperature, absorber, water_temperature, handle, sensor, batch, absorber_id):
        dev, b, keep = _run(handle, sensor, batch, absorber_id, temperature, absorber, water_temperature)
        P, L = temperature.shape[0], handle.n_channels[sensor]
        f = dict(dtype=torch.float64, device=temperature.device)
        out = dict(radiance=torch.empty((P, L), **f), bt=torch.empty((P, L), **f),
                   status=torch.empty((P,), dtype=torch.int32, device=temperature.device))
        handle.forward_device(b, out, sensor, torch.cuda.current_stream(temperature.device).cuda_stream)
        ctx.save_for_backward(temperature, absorber, water_temperature)
        ctx.handle, ctx.sensor, ctx.batch, ctx.absorber_id = handle, sensor, batch, absorber_id
        return out["bt"]

    @staticmethod
    def backward(ctx, grad_bt):
        temperature, absorber, water_temperature = ctx.saved_tensors
        dev, b, keep = _run(ctx.handle, ctx.sensor, ctx.batch, ctx.absorber_id, temperature, absorber,
                            water_temperature)
        P, L = grad_bt.shape
        f = dict(dtype=torch.float64, device=temperature.device)
        out = dict(radiance=torch.empty((P, L), **f), bt=torch.empty((P, L), **f),
                   status=torch.empty((P,), dtype=torch.int32, device=temperature.device),
                   temperature_ad=torch.zeros_like(temperature), absorber_ad=torch.zeros_like(absorber),
                   water_temperature_ad=torch.zeros_like(water_temperature))
        seed = grad_bt.to(torch.float64).contiguous()
        ctx.handle.adjoint_device(b, seed, out, ctx.sensor,
                                  torch.cuda.current_stream(temperature.device).cuda_stream)
        return out["temperature_ad"], out["absorber_ad"], out["water_temperature_ad"], None, None, None, None


def brightness_temperature(handle, batch: dict, absorber_id: np.ndarray, temperature: torch.Tensor,
                           absorber: torch.Tensor, water_temperature: torch.Tensor, sensor: int = 0) -> torch.Tensor:
    """Differentiable brightness temperatures (P, L) with respect to the
    temperature, absorber amounts and water surface temperature."""
    return _BrightnessTemperature.apply(temperature, absorber, water_temperature, handle, sensor, batch,
                                        absorber_id)
