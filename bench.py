"""Benchmark: the K-matrix of the ragged mixed-sensor batch, mixed precision vs all-FP64, on one GB300.

Default workload (one step, --workload C5): 20000 profiles with layer counts
uniform in 60-137, each seen by one of 3 synthetic sensors (22 microwave, 616
and 2211 infrared channels), 30 % of them cloudy (liquid and ice clouds in the
infrared, 5 cloud types in the microwave) with the stream rule or
Options%n_Streams 8 / 16; forward + K-matrix through ADA with the Jacobians of
temperature, H2O and O3 per layer, skin temperature, emissivity and each
cloud's water content and effective radius.  Synthetic seeded inputs and
coefficient files (crtmv3_gb300.synthetic) stand in for real sensor data.

Reported value: profile*channels per second of the mixed-precision form with
inputs resident in HBM.  The same JSON line carries the all-FP64 GPU form,
the accuracy of both forms against the FP64 oracle (and of the mixed form
against the FP64 form), per-stage kernel times, the roofline of the dominant
kernel stage, the end-to-end rate through the host entry point and the CPU
baseline (the oracle on the host cores).  --workload C2 is the clear-sky IR
K-matrix (2000 x 101 x 2211); C3 and C4 the cloudy microwave adjoint and the
all-sky infrared K-matrix.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--workload C5|C2|C3|C4]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from crtmv3_gb300 import synthetic as sy  # noqa: E402
from crtmv3_gb300.replicas import max_over_ranks  # noqa: E402

SENSOR = "irsynth_c2211"
N_LAYERS = 101
METRIC = "K-matrix profile*channels/s (mixed precision, inputs in HBM)"
UNIT = "profile*channels/s"
COEFF_DIR = os.path.join(ROOT, "coeffs")


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    except OSError:
        return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi samples during the timed region (1 GPU: the one we run on)."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_workload(P: int, seed: int):
    atm, sfc, geo, opt = sy.clear_sky_workload(SENSOR, P, N_LAYERS, seed)
    return atm, sfc, geo, opt


def device_batch(torch, h, atm, sfc, geo, opt, dev):
    t = {}
    for k in ("level_pressure", "pressure", "temperature", "absorber"):
        t[k] = torch.from_numpy(np.ascontiguousarray(getattr(atm, k))).to(dev)
    t["n_layers"] = torch.from_numpy(atm.n_layers.astype(np.int32)).to(dev)
    for f in ("land_coverage", "water_coverage", "snow_coverage", "ice_coverage", "land_temperature",
              "water_temperature", "snow_temperature", "ice_temperature"):
        t[f] = torch.from_numpy(np.ascontiguousarray(getattr(sfc, f))).to(dev)
    t["sensor_zenith_angle"] = torch.from_numpy(geo.sensor_zenith_angle).to(dev)
    t["source_zenith_angle"] = torch.from_numpy(geo.source_zenith_angle).to(dev)
    t["surface_altitude"] = torch.from_numpy(geo.surface_altitude).to(dev)
    t["emissivity"] = torch.from_numpy(np.ascontiguousarray(opt.emissivity)).to(dev)
    b, keep = h.device_batch(t, atm.absorber_id)
    return b, keep, t


def k_outputs(torch, P, L, K, JK, dev):
    f = dict(dtype=torch.float64, device=dev)
    return dict(radiance=torch.empty((P, L), **f), bt=torch.empty((P, L), **f),
                temperature_k=torch.empty((P, L, K), **f), absorber_k=torch.empty((P, L, JK, K), **f),
                water_temperature_k=torch.empty((P, L), **f), surface_emissivity_k=torch.empty((P, L), **f),
                status=torch.empty((P,), dtype=torch.int32, device=dev))


def jacobian_sel(atm):
    """User absorber indices of the H2O and O3 Jacobians that the K-matrix returns."""
    ids = list(atm.absorber_id)
    return [ids.index(1), ids.index(3)]


def cpu_baseline(P_sample: int, threads: int, min_seconds: float = 10.0):
    """FP64 oracle (restatement of the reference's CPU path) on the host cores:
    K-matrix calls on batches of ``P_sample`` profiles of the workload with the
    same two absorber Jacobians as the GPU arm, repeated until at least
    ``min_seconds`` of CPU work; returns (p*c/s, seconds, calls, sample, oracle
    outputs of the sample)."""
    from oracle.pyoracle import Oracle
    atm, sfc, geo, opt = make_workload(P_sample, 2024)
    sel = jacobian_sel(atm)
    o = Oracle(COEFF_DIR, SENSOR)
    w = slice(0, min(2, P_sample))
    o.k_matrix(atm.subset(w), sfc.subset(w), geo.subset(w), opt.subset(w), n_threads=threads, k_absorbers=sel)
    calls, t0 = 0, time.perf_counter()
    while True:
        ref = o.k_matrix(atm, sfc, geo, opt, n_threads=threads, k_absorbers=sel)
        calls += 1
        dt = time.perf_counter() - t0
        if dt >= min_seconds:
            break
    return calls * P_sample * o.n_channels / dt, dt, calls, (atm, sfc, geo, opt), ref


def oracle_errors(h, sample, ref, prec):
    """Errors of one GPU form against the FP64 oracle on the CPU-baseline
    sample: max |dBT| (K) and, per Jacobian output, max |dK| / max |K_oracle|."""
    atm, sfc, geo, opt = sample
    sel = jacobian_sel(atm)
    h.set_precision(prec)
    km, rts = h.k_matrix(atm, sfc, geo, opt, k_absorbers=sel)

    def rel(x, y):
        return float(np.abs(x - y).max() / max(np.abs(y).max(), 1e-300))

    def over(x, y):   # entries off by more than 1e-3 of the largest (a clamp's kink crossed by rounding)
        return int((np.abs(x - y) > 1e-3 * max(np.abs(y).max(), 1e-300)).sum())
    n_over = {"temperature": over(km.temperature, ref["temperature_k"]),
              "h2o": over(km.absorber[:, :, 0], ref["absorber_k"][:, :, sel[0]]),
              "o3": over(km.absorber[:, :, 1], ref["absorber_k"][:, :, sel[1]])}
    return {"max_abs_bt_K": float(np.abs(rts.brightness_temperature - ref["bt"]).max()),
            "entries_over_1e-3": n_over, "entries": int(km.temperature.size),
            "max_rel_jacobian": {
                "temperature": rel(km.temperature, ref["temperature_k"]),
                "h2o": rel(km.absorber[:, :, 0], ref["absorber_k"][:, :, sel[0]]),
                "o3": rel(km.absorber[:, :, 1], ref["absorber_k"][:, :, sel[1]]),
                "water_temperature": rel(km.water_temperature, ref["water_temperature_k"]),
                "surface_emissivity": rel(km.surface_emissivity, ref["surface_emissivity_k"])},
            "profiles": int(atm.n_profiles)}


def workload_config(P: int, world: int) -> dict:
    return {"workload": f"clear-sky IR forward+K-matrix, {P} profiles x {N_LAYERS} layers x 2211 "
                        f"channels (ODPS group 1, Emission), Jacobians T/H2O/O3 + Tskin",
            "profiles": P, "layers": N_LAYERS, "channels": 2211, "parallelism": f"replicas x{world}",
            "l2": f"inputs larger than L2: {P * 2211 * (3 * N_LAYERS + 2) * 8 / 1e9:.1f} GB of "
                  f"K-matrix output per step, no flush"}


def run_reference(args):
    """The reference's CPU path (the FP64 oracle, a restatement of it: the
    Fortran reference cannot be built here) on the host cores: each step is
    a bounded sample of the workload (C2: args.cpu_profiles profiles; C3-C5:
    args.cpu_profiles profiles of each sensor group with the group's mix of
    clear and cloudy profiles and stream options)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    if args.workload == "C2":
        sy.write_sensor_files(COEFF_DIR, SENSOR)
        P_sample = args.cpu_profiles
        vals = []
        for _ in range(args.warmup):
            cpu_baseline(max(threads // 2, 1), threads, min_seconds=0.0)
        for _ in range(args.steps):
            v, dt, calls, _, _ = cpu_baseline(P_sample, threads, min_seconds=0.0)
            vals.append((v, dt))
        cfg = workload_config(args.profiles, 1)
        cfg["sample_profiles_per_step"] = P_sample
        metric = METRIC
        sample = (f"{P_sample} profiles x 2211 channels K-matrix per step, H2O and O3 Jacobians as the GPU arm "
                  f"(FP64 C oracle, OpenMP over profiles)")
    else:
        groups = scatter_groups(args.workload, 0, args.profiles if args.profiles != 2000 else 0)
        for sid, *_ in groups:
            sy.write_sensor_files(COEFF_DIR, sid)
        sy.write_cloud_files(COEFF_DIR)
        sy.write_aerosol_files(COEFF_DIR)
        samp = sample_groups(groups, args.cpu_profiles)
        small = sample_groups(groups, 2)
        for _ in range(args.warmup):
            oracle_scatter_k(small, threads)
        vals = []
        for _ in range(args.steps):
            _, pc, dt = oracle_scatter_k(samp, threads)
            vals.append((pc / dt, dt))
        cfg = {"workload": args.workload + ": " + SCATTER_WORKLOAD[args.workload],
               "groups": [{"sensor": g[0], "profiles": int(g[1].n_profiles)} for g in groups],
               "parallelism": "replicas x1", "sample_profiles_per_group_per_step": args.cpu_profiles}
        metric = SCATTER_METRIC[args.workload]
        sample = (f"{args.cpu_profiles} profiles of each sensor group per step whose mix of clear, stream-rule, "
                  f"8- and 16-stream cloudy profiles is the group's (the throughput of the sample stands for the "
                  f"whole workload's), K-matrix with the GPU arm's Jacobians"
                  f"{' (C3: the adjoint as the unit-seeded K-matrix, the same reverse pass per channel)' if args.workload == 'C3' else ''} "
                  f"(FP64 C oracle: clear-sky chain and the reverse mode of the ADA path, OpenMP over profiles)")
    value = statistics.median(v for v, _ in vals)
    ms = statistics.median(dt for _, dt in vals) * 1e3
    line = {"impl": "reference", "metric": metric,
            "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# Scattering workloads (optional: --workload C3 | C4 | C5)
# ---------------------------------------------------------------------------

SCATTER_WORKLOAD = {
    "C3": "5000 profiles x 100 layers x 16 MW channels, 5 cloud types, ADA, forward + adjoint",
    "C4": "1000 profiles x 100 layers x 616 IR channels, liquid + ice clouds and 3 aerosols, ADA, forward + "
          "K-matrix",
    "C5": "20000 profiles, layers U[60,137], one of 3 sensors each (22 MW / 616 IR / 2211 IR channels), 30% "
          "cloudy (liquid + ice in IR, 5 types in MW) with the stream rule or Options%n_Streams 8 / 16, ADA, "
          "forward + K-matrix with T / H2O / O3 per layer, skin T, emissivity, cloud water content and radius",
}
SCATTER_METRIC = {
    "C3": "forward+adjoint profile*channels/s (cloudy MW, ADA, mixed precision, inputs in HBM)",
    "C4": "forward+K-matrix profile*channels/s (all-sky IR with aerosols, ADA, mixed precision, inputs in HBM)",
    "C5": "forward+K-matrix profile*channels/s (ragged 3-sensor batch, 30% cloudy, mixed precision, "
          "inputs in HBM)",
}


def scatter_groups(name: str, rank: int, profiles: int = 0):
    """Per-sensor sub-batches [(sensor, atm, sfc, geo, opt)] of a scattering
    workload; ``profiles`` > 0 scales C3 / C4 down (profiling captures)."""
    from crtmv3_gb300 import coefficients as co
    if name == "C3":
        # 5000 x 100 x 16 MW, 5 cloud types (Cloud_Fraction 1 in cloudy layers),
        # stream rule with Options%n_Streams 8 / 16 on a tenth of the profiles each
        P = profiles or 5000
        atm, sfc, geo, opt = sy.cloudy_workload("mwsynth_c16", P, 100, 3100 + rank)
        rng = np.random.Generator(np.random.PCG64(3200 + rank))
        ns = rng.choice(np.array([0, 8, 16], np.int32), size=P, p=[0.8, 0.1, 0.1])
        opt.use_n_streams, opt.n_streams = ns > 0, ns
        return [("mwsynth_c16", atm, sfc, geo, opt)]
    if name == "C4":
        # 1000 x 100 x 616 IR, liquid + ice clouds, dust + sea salt + sulfate
        atm, sfc, geo, opt = sy.clear_sky_workload("irsynth_c616", profiles or 1000, 100, 3300 + rank)
        sy.add_clouds(atm, (co.WATER_CLOUD, co.ICE_CLOUD), 3301 + rank)
        sy.add_aerosols(atm, sy.AEROSOL_TYPES, 3302 + rank)
        return [("irsynth_c616", atm, sfc, geo, opt)]
    # C5: 20000 profiles, layers U[60,137], one of 3 sensors each, 30 % cloudy
    # with the stream rule or Options%n_Streams 8 / 16
    P = 20000
    rng = np.random.Generator(np.random.PCG64(3400 + rank))
    sensors = ("mwsynth_c22", "irsynth_c616", "irsynth_c2211")
    which = rng.integers(0, 3, P)
    nl = rng.integers(60, 138, P)
    groups = []
    for i, sid in enumerate(sensors):
        idx = np.nonzero(which == i)[0]
        atm, sfc, geo, opt = sy.clear_sky_workload(sid, idx.size, nl[idx], 3500 + 10 * rank + i)
        types = ((co.WATER_CLOUD, co.ICE_CLOUD, co.RAIN_CLOUD, co.SNOW_CLOUD, co.GRAUPEL_CLOUD)
                 if sid.startswith("mw") else (co.WATER_CLOUD, co.ICE_CLOUD))
        sy.add_clouds(atm, types, 3600 + 10 * rank + i)
        cloudy = rng.uniform(size=idx.size) < 0.3
        atm.n_clouds[~cloudy] = 0
        ns = np.where(cloudy, rng.choice(np.array([0, 8, 16], np.int32), size=idx.size, p=[0.6, 0.2, 0.2]), 0)
        opt.use_n_streams, opt.n_streams = ns > 0, ns.astype(np.int32)
        groups.append((sid, atm, sfc, geo, opt))
    return groups


def scatter_device_inputs(torch, h, atm, sfc, geo, opt, dev):
    t = {}
    for k in ("level_pressure", "pressure", "temperature", "absorber", "cloud_water_content",
              "cloud_effective_radius", "cloud_fraction", "aerosol_concentration", "aerosol_effective_radius"):
        v = getattr(atm, k)
        if v is not None:
            t[k] = torch.from_numpy(np.ascontiguousarray(v, np.float64)).to(dev)
    for k in ("n_layers", "n_clouds", "cloud_type", "n_aerosols", "aerosol_type"):
        v = getattr(atm, k)
        if v is not None:
            t[k] = torch.from_numpy(np.ascontiguousarray(v, np.int32)).to(dev)
    for f in ("land_coverage", "water_coverage", "snow_coverage", "ice_coverage", "land_temperature",
              "water_temperature", "snow_temperature", "ice_temperature"):
        t[f] = torch.from_numpy(np.ascontiguousarray(getattr(sfc, f))).to(dev)
    for f in ("sensor_zenith_angle", "source_zenith_angle", "surface_altitude"):
        t[f] = torch.from_numpy(np.ascontiguousarray(getattr(geo, f))).to(dev)
    t["emissivity"] = torch.from_numpy(np.ascontiguousarray(opt.emissivity)).to(dev)
    if opt.n_streams is not None:
        t["n_streams"] = torch.from_numpy(np.where(opt.use_n_streams, opt.n_streams, 0).astype(np.int32)).to(dev)
    if opt.rt_algorithm_id is not None:
        t["rt_algorithm_id"] = torch.from_numpy(opt.rt_algorithm_id.astype(np.int32)).to(dev)
    b, keep = h.device_batch(t, atm.absorber_id)
    return b, keep, t


def pinned_copy(torch, obj):
    """A copy of a batch dataclass with every numpy array in pinned host
    memory (the end-to-end legs copy their inputs from pinned memory)."""
    import dataclasses as dc
    vals = {}
    for f in dc.fields(obj):
        v = getattr(obj, f.name)
        if isinstance(v, np.ndarray) and v.dtype != object:
            t = torch.empty(v.shape, dtype=torch.from_numpy(np.zeros(1, v.dtype)).dtype, pin_memory=True).numpy()
            t[...] = v
            vals[f.name] = t
    return dc.replace(obj, **vals)


def pinned_rts(torch, P: int, L: int):
    from crtmv3_gb300.structures import RTSolutionBatch
    return RTSolutionBatch(torch.empty((P, L), dtype=torch.float64, pin_memory=True).numpy(),
                           torch.empty((P, L), dtype=torch.float64, pin_memory=True).numpy(),
                           status=torch.empty((P,), dtype=torch.int32, pin_memory=True).numpy())


def stratified_indices(atm, opt, n: int) -> np.ndarray:
    """n profile indices of a group whose mix of strata -- clear, cloudy on the
    stream rule, cloudy with Options%n_Streams 8, with 16 -- matches the
    group's (largest-remainder quotas; the first profiles of each stratum), so
    a throughput measured on the sample stands for the whole group's."""
    P = atm.n_profiles
    n = min(n, P)
    cloudy = np.zeros(P, bool)
    if atm.n_clouds is not None:
        cloudy |= atm.n_clouds > 0
    if atm.n_aerosols is not None:
        cloudy |= atm.n_aerosols > 0
    ns = opt.n_streams if opt.n_streams is not None and opt.use_n_streams is not None else np.zeros(P, np.int32)
    ns = np.where(opt.use_n_streams, ns, 0) if opt.use_n_streams is not None else ns
    key = np.where(~cloudy, 0, np.where(ns == 8, 2, np.where(ns == 16, 3, 1)))
    counts = np.bincount(key, minlength=4)
    exact = counts * n / P
    q = np.floor(exact).astype(int)
    for s_ in np.argsort(-(exact - q))[: n - q.sum()]:
        q[s_] += 1
    return np.sort(np.concatenate([np.nonzero(key == s_)[0][:q[s_]] for s_ in range(4)]))


def sample_groups(groups, n: int):
    """n profiles of each group with the group's own mix of clear and cloudy
    profiles and stream options (stratified_indices)."""
    out = []
    for sid, atm, sfc, geo, opt in groups:
        w = stratified_indices(atm, opt, n)
        out.append((sid, atm.subset(w), sfc.subset(w), geo.subset(w), opt.subset(w)))
    return out


def k_selection(atm):
    """User absorber indices of the H2O and O3 Jacobians that the K-matrix returns."""
    ids = list(atm.absorber_id)
    return [ids.index(j) for j in (1, 3) if j in ids]


def oracle_scatter_k(groups, threads: int):
    """The FP64 oracle's K-matrix (clear-sky chain + the reverse mode of the
    ADA path) of each group, with the Jacobians the GPU arm returns; returns
    (outputs per group, p*c, seconds)."""
    from oracle.pyoracle import Oracle
    outs, pc, t = [], 0, 0.0
    for sid, atm, sfc, geo, opt in groups:
        o = Oracle(COEFF_DIR, sid)
        t0 = time.perf_counter()
        r = o.k_matrix_scatter(atm, sfc, geo, opt, os.path.join(COEFF_DIR, "CloudCoeff.bin"),
                               os.path.join(COEFF_DIR, "AerosolCoeff.bin") if atm.aerosol_type is not None else None,
                               n_threads=threads, k_absorbers=k_selection(atm))
        t += time.perf_counter() - t0
        outs.append(r)
        pc += atm.n_profiles * o.n_channels
    return outs, pc, t


def scatter_errors(gpu, ref, atm):
    """Errors of one GPU form's outputs against the oracle's on the same
    profiles: max |dBT| (K) and, per Jacobian, max |dK| / max |K_oracle| (the
    cloud and aerosol Jacobians scaled by their variable)."""
    sel = k_selection(atm)

    def rel(x, y, scale=None):
        return float(np.abs(x - y).max() / max(np.abs(y if scale is None else scale).max(), 1e-300))
    e = {"max_abs_bt_K": float(np.abs(gpu["bt"] - ref["bt"]).max()),
         "temperature": rel(gpu["temperature_k"], ref["temperature_k"]),
         "water_temperature": rel(gpu["water_temperature_k"], ref["water_temperature_k"]),
         "surface_emissivity": rel(gpu["surface_emissivity_k"], ref["surface_emissivity_k"])}
    for i, j in enumerate(sel):
        e[f"absorber_{int(atm.absorber_id[j])}"] = rel(gpu["absorber_k"][:, :, i], ref["absorber_k"][:, :, j])
    for f in ("cloud_water_content", "cloud_effective_radius", "aerosol_concentration", "aerosol_effective_radius"):
        if f + "_k" in gpu and ref[f + "_k"].size:
            x = getattr(atm, f)[:, None]
            e[f] = rel(gpu[f + "_k"] * x, ref[f + "_k"] * x)
    return e


def merge_errors(acc, e):
    for k, v in e.items():
        acc[k] = max(acc.get(k, 0.0), v)
    return acc


def pipe_peaks(torch, dev):
    """cuBLAS FP64 and FP32 (TF32 off) matrix-multiply rates of this GPU
    through torch.matmul, best of 5, TFLOP/s: the measured ceilings for
    kernels bound by the FP64 or FP32 pipes."""
    out = {}
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    for name, dt, n in (("fp64", torch.float64, 4096), ("fp32", torch.float32, 8192)):
        a = torch.randn(n, n, dtype=dt, device=dev)
        b = torch.randn(n, n, dtype=dt, device=dev)
        torch.matmul(a, b)
        torch.cuda.synchronize(dev)
        best = 1e30
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize(dev)
            best = min(best, e0.elapsed_time(e1))
        out[name] = 2.0 * n ** 3 / (best * 1e-3) / 1e12
        del a, b
    torch.backends.cuda.matmul.allow_tf32 = prev
    return out


# Operations of one scattering layer's MOM work in the cloudy K-matrix's
# layer reverse sweep (scatter_reverse_kernel: phase blocks, the loss-form MOM
# forward and its reverse sweep, the phase blocks' adjoint) by its angle
# count nZ, counted by running the kernel's header code on an
# operation-counting number type (tests/harness/flop_count.cpp; every +, -,
# *, /, sqrt, exp counted, an FMA as two).  The species' LUT derivatives are
# not counted.
REVERSE_LAYER_OPS = {3: 3330, 4: 7660, 5: 14550, 6: 24700, 10: 113600}


def scattering_layer_sum(groups, n_channels, wavenumbers, per_layer):
    """Sum over the step's cloudy (profile, channel) pairs of their scattering
    layers' per_layer(nZ), with nZ the stream set's angles plus the sensor
    angle: Options%n_Streams, else the stream rule on the largest effective
    radius and the channel's wavenumber.  A scattering layer is one with an
    active cloud (water content above 1e-6)."""
    total = 0.0
    for (sid, atm, sfc, geo, opt), L, wn in zip(groups, n_channels, wavenumbers):
        for p in range(atm.n_profiles):
            nc = int(atm.n_clouds[p]) if atm.n_clouds is not None else 0
            if nc == 0:
                continue
            wc = atm.cloud_water_content[p, :nc]
            n_sl = int(((wc > 1e-6).any(axis=0)).sum())   # layers with an active cloud
            ns = int(opt.n_streams[p]) if opt.n_streams is not None and opt.use_n_streams[p] else 0
            if ns:
                nz = np.full(L, (ns + 2) // 2 + 1)
            else:
                mie = 2.0 * np.pi * atm.cloud_effective_radius[p, :nc].max() * wn / 1.0e4
                nleg = np.where(mie < 0.01, 2, np.where(mie < 1.0, 4, 6))
                nz = (nleg + 2) // 2 + 1
            total += n_sl * float(sum(per_layer(int(z)) * c for z, c in zip(*np.unique(nz, return_counts=True))))
    return total


def adding_flops(groups, n_channels, wavenumbers):
    """Algorithmic FP64 FLOPs of one step's adding and adding adjoint
    (scatter_adding): 38 nZ^3 per scattering layer and (profile, channel) --
    forward adding 10 nZ^3 (Gamma = (I - Rup R)^-1 by elimination, T Gamma,
    Rup T, T Gamma Rup T) and its adjoint 28 nZ^3 (Gamma again, and the
    products' transposes)."""
    return scattering_layer_sum(groups, n_channels, wavenumbers, lambda z: 38.0 * z ** 3)


def reverse_flops(groups, n_channels, wavenumbers):
    """Operations of one step's layer reverse sweeps (scatter_contract stage):
    REVERSE_LAYER_OPS[nZ] per scattering layer and (profile, channel)."""
    return scattering_layer_sum(groups, n_channels, wavenumbers, lambda z: float(REVERSE_LAYER_OPS[z]))


def run_scattering(args, torch, dev, rank, world, dist):
    from crtmv3_gb300 import api, coefficients as co
    name = args.workload
    # the K-matrix's scattering intermediates take ~0.4 GB per cloudy IR profile
    # on the stream rule and ~1.3 GB with 16 streams: a large work space keeps
    # the scattering kernels' grids full (the step's outputs take ~150 GB)
    os.environ.setdefault("CRTM_GPU_WORKSPACE_MB", "49152")
    groups = scatter_groups(name, rank, args.profiles if args.profiles != 2000 else 0)
    if rank == 0:
        for sid, *_ in groups:
            sy.write_sensor_files(COEFF_DIR, sid)
        sy.write_cloud_files(COEFF_DIR)
        sy.write_aerosol_files(COEFF_DIR)
    if dist:
        dist.barrier()
    sids = [g[0] for g in groups]
    h = api.CRTM(sids, COEFF_DIR, api.FP64)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    sptr = stream.cuda_stream
    f64 = dict(dtype=torch.float64, device=dev)
    calls = []
    for si, (sid, atm, sfc, geo, opt) in enumerate(groups):
        b, keep, t = scatter_device_inputs(torch, h, atm, sfc, geo, opt, dev)
        P, K, L = atm.n_profiles, atm.max_layers, h.n_channels[si]
        sel = k_selection(atm)
        o = dict(radiance=torch.empty((P, L), **f64), bt=torch.empty((P, L), **f64),
                 status=torch.empty((P,), dtype=torch.int32, device=dev))
        if name == "C3":
            o.update(temperature_ad=torch.empty((P, K), **f64),
                     absorber_ad=torch.empty((P, atm.n_absorbers, K), **f64),
                     water_temperature_ad=torch.empty((P,), **f64))
        else:
            o.update(temperature_k=torch.empty((P, L, K), **f64),
                     absorber_k=torch.empty((P, L, len(sel), K), **f64),
                     water_temperature_k=torch.empty((P, L), **f64),
                     surface_emissivity_k=torch.empty((P, L), **f64))
        # scattering Jacobians, as the reference's K-matrix / adjoint returns them
        sfx = "_ad" if name == "C3" else "_k"
        lead = (P,) if name == "C3" else (P, L)
        if atm.cloud_type is not None:
            NC = atm.cloud_type.shape[1]
            o["cloud_water_content" + sfx] = torch.empty(lead + (NC, K), **f64)
            o["cloud_effective_radius" + sfx] = torch.empty(lead + (NC, K), **f64)
        if atm.aerosol_type is not None:
            NA = atm.aerosol_type.shape[1]
            o["aerosol_concentration" + sfx] = torch.empty(lead + (NA, K), **f64)
            o["aerosol_effective_radius" + sfx] = torch.empty(lead + (NA, K), **f64)
        seed = torch.ones((P, L), **f64)
        calls.append(dict(si=si, b=b, keep=(keep, t), sel=sel, out=o, seed=seed, pc=P * L))

    def step(prec):
        h.set_precision(prec)
        for c in calls:
            if name == "C3":
                h.adjoint_device(c["b"], c["seed"], c["out"], c["si"], sptr)
            else:
                h.k_matrix_device(c["b"], c["out"], None, c["si"], sptr, k_absorbers=c["sel"])

    def timed(prec, n):
        torch.cuda.synchronize(dev)
        if dist:
            dist.barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            step(prec)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return max_over_ranks(e0.elapsed_time(e1), dist, dev)

    n_cmp = args.cpu_profiles
    samp_idx = [torch.from_numpy(stratified_indices(g[1], g[4], n_cmp)).to(dev) for g in groups]

    def sample_out():
        return [{f: v[ix].cpu().numpy() for f, v in c["out"].items()} for c, ix in zip(calls, samp_idx)]
    # the FP64 form's outputs: the mixed form's accuracy against it on the first
    # 512 profiles of each group, and both forms against the oracle on the sample
    step(0)
    torch.cuda.synchronize(dev)
    ref = [{f: v[:512].clone() for f, v in c["out"].items()} for c in calls]
    fp64_sample = sample_out()
    for _ in range(args.warmup):
        step(1)
    torch.cuda.synchronize(dev)
    launches0 = h.launch_count()
    h.set_profiling(True)
    h.stage_times(reset=True)
    with ClockSampler(local_rank()) as clk:
        ms_mixed = timed(1, args.steps)
    st = h.stage_times(reset=True)
    h.set_profiling(False)
    launches = h.launch_count() - launches0
    # a device entry point reports failed profiles in its status words only
    bad = sum(int((c["out"]["status"] != 0).sum()) for c in calls)
    if bad:
        raise RuntimeError(f"{bad} profiles failed in the timed mixed-form steps (status words)")
    mixed_sample = sample_out()
    bt_err, field_err = 0.0, {}
    for c, r in zip(calls, ref):
        a = c["out"]
        bt_err = max(bt_err, float((a["bt"][:512] - r["bt"]).abs().max()))
        for f in a:
            if f in ("radiance", "bt", "status"):
                continue
            e = float((a[f][:512] - r[f]).abs().max() / r[f].abs().max().clamp_min(1e-300))
            field_err[f] = max(field_err.get(f, 0.0), e)
    del ref
    jac_err = max(field_err.values()) if field_err else 0.0
    fp64_steps = max(1, min(args.steps, 2))
    ms_fp64 = timed(0, fp64_steps)
    bad = sum(int((c["out"]["status"] != 0).sum()) for c in calls)
    if bad:
        raise RuntimeError(f"{bad} profiles failed in the timed FP64-form steps (status words)")
    pc = sum(c["pc"] for c in calls) * world
    per_mixed, per_fp64 = ms_mixed / args.steps, ms_fp64 / fp64_steps
    value, fp64_value = pc / (per_mixed * 1e-3), pc / (per_fp64 * 1e-3)
    stage_ms = {k: v[0] / args.steps for k, v in st.items() if v[1] > 0}
    extra = {}
    # roofline of the step's dominant kernel stage
    roofline = None
    if rank == 0 and name in ("C4", "C5") and stage_ms:
        dom = max(stage_ms, key=stage_ms.get)
        pk = pipe_peaks(torch, dev)
        chans = [h.n_channels[i] for i in range(len(groups))]
        wns = [co.read_spccoeff(os.path.join(COEFF_DIR, f"{g[0]}.SpcCoeff.bin")).wavenumber for g in groups]
        if dom in ("scatter_adding", "scatter_contract"):
            fl = (adding_flops if dom == "scatter_adding" else reverse_flops)(groups, chans, wns)
            ach = fl / (stage_ms[dom] * 1e-3) / 1e12
            pipe = "fp32"   # the mixed form's adding and reverse sweep run in FP32
            roofline = {"bound": pipe, "achieved": ach, "peak": pk[pipe], "unit": "TFLOP/s",
                        "frac": ach / pk[pipe], "traffic": None,
                        "kernel": ("scatter_kmatrix_kernel (adding + adjoint)" if dom == "scatter_adding" else
                                   "scatter_reverse_kernel (MOM forward + reverse sweep per scattering layer)"),
                        "algorithmic_flops_per_step": fl,
                        "flop_count": ("38 nZ^3 per scattering layer" if dom == "scatter_adding" else
                                       "REVERSE_LAYER_OPS[nZ] per scattering layer, counted on an "
                                       "operation-counting number type"),
                        "peak_source": "measured in this run: cuBLAS FP32 GEMM (TF32 off) through torch.matmul"}
        else:
            roofline = {"bound": None, "kernel": dom, "note": "no algorithmic count for this stage"}
        extra["pipe_peaks_tflops"] = pk
    if name == "C4":   # SOI forward and K-matrix on the same inputs, ADA forward beside them
        sid, atm, sfc, geo, opt = groups[0]
        opt.rt_algorithm_id = np.full(atm.n_profiles, 168, np.int32)
        b, keep, t = scatter_device_inputs(torch, h, atm, sfc, geo, opt, dev)
        fo = calls[0]["out"]
        h.set_precision(1)
        h.forward_device(b, fo, 0, sptr)
        opt.rt_algorithm_id = np.full(atm.n_profiles, 56, np.int32)
        b2, keep2, t2 = scatter_device_inputs(torch, h, atm, sfc, geo, opt, dev)
        fo2 = {k: torch.empty_like(v) for k, v in fo.items() if k in ("radiance", "bt", "status")}
        for lab, bb, oo in (("soi", b, fo), ("ada", b2, fo2)):
            h.forward_device(bb, oo, 0, sptr)
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.steps):
                h.forward_device(bb, oo, 0, sptr)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            ms = e0.elapsed_time(e1) / args.steps
            extra[f"{lab}_forward_mixed"] = {"ms_per_step": ms, "value": calls[0]["pc"] / (ms * 1e-3)}
        extra["soi_vs_ada_max_abs_bt_K"] = float((fo["bt"] - fo2["bt"]).abs().max())
        # the SOI K-matrix of the same inputs (the orders' adjoint; FP64 in both
        # forms), against the ADA K-matrix step above
        c0 = calls[0]
        h.k_matrix_device(b, c0["out"], None, 0, sptr, k_absorbers=c0["sel"])
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        h.k_matrix_device(b, c0["out"], None, 0, sptr, k_absorbers=c0["sel"])
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1)
        extra["soi_k_matrix"] = {"ms_per_call": ms, "value": c0["pc"] / (ms * 1e-3),
                                 "vs_ada_k_matrix_mixed": ms / per_mixed}
        opt.rt_algorithm_id = None
    # end to end through the host entry point (pinned host outputs), mixed
    # form, on a sample of each group's profiles (the full step's ~150 GB of
    # Jacobians exceed what this process pins)
    e2e = None
    if not args.no_e2e and name != "C3":
        from crtmv3_gb300.structures import KMatrixBatch
        frac = 8
        sub = [(sid,) + tuple(pinned_copy(torch, x.subset(slice(0, a.n_profiles // frac)))
                              for x in (a, s_, g_, o_))
               for sid, a, s_, g_, o_ in groups]

        def pin(shape):
            return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
        outs, h2d, d2h, epc = [], 0, 0, 0
        for si, (sid, a, s_, g_, o_) in enumerate(sub):
            P, K, L = a.n_profiles, a.max_layers, h.n_channels[si]
            sel = k_selection(a)
            km = KMatrixBatch(pin((P, L, K)), pin((P, L, len(sel), K)), pin((P, L)), pin((P, L)))
            NC = a.cloud_type.shape[1] if a.cloud_type is not None else 0
            if NC:
                km.cloud_water_content = pin((P, L, NC, K))
                km.cloud_effective_radius = pin((P, L, NC, K))
            outs.append((km, sel, pinned_rts(torch, P, L)))
            h2d += sum(x.nbytes for x in (a.level_pressure, a.pressure, a.temperature, a.absorber, o_.emissivity,
                                          a.cloud_water_content, a.cloud_effective_radius, a.cloud_fraction)
                       if x is not None) + 14 * P * 8
            d2h += P * L * 8 * (2 + K * (1 + len(sel) + 2 * NC) + 2) + P * 4
            epc += P * L
        h.set_precision(1)

        def e2e_step():
            for si, ((sid, a, s_, g_, o_), (km, sel, rt)) in enumerate(zip(sub, outs)):
                h.k_matrix(a, s_, g_, o_, None, si, k_absorbers=sel, out=km, rts_out=rt)
        e2e_step()
        n_e2e = max(1, min(args.steps, 2))
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(n_e2e):
            e2e_step()
        dt = (time.perf_counter() - t0) / n_e2e
        e2e = {"value": epc * world / dt, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "ms_per_step": dt * 1e3, "sample": f"first 1/{frac} of each group's profiles per step, inputs and "
                                                 f"outputs in pinned host memory"}
        del outs
    # CPU baseline (the FP64 oracle on the host cores) and both GPU forms
    # against the oracle, on n_cmp profiles of each group (stratified_indices)
    cpu, vs_oracle = None, None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        samp = sample_groups(groups, n_cmp)
        ref_o, cpc, ct = oracle_scatter_k(samp, threads)
        cpu = {"value": cpc / ct, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{n_cmp} profiles of each sensor group ({cpc} profile*channels) whose mix of clear, "
                         f"stream-rule, 8- and 16-stream cloudy profiles is the group's, K-matrix with the same "
                         f"Jacobians as the GPU arm, FP64 C oracle with OpenMP over profiles, {ct:.1f} s"}
        if name == "C3":   # the adjoint (unit seed) is the oracle's K-matrix summed over the channels
            cpu["sample"] += "; the adjoint as the unit-seeded K-matrix summed over the channels"
        vs_oracle = {"fp64": {}, "mixed": {}, "profiles_per_group": n_cmp}
        for (sid, a, *_), r, g64, gmx in zip(samp, ref_o, fp64_sample, mixed_sample):
            if name == "C3":
                for form, g in (("fp64", g64), ("mixed", gmx)):
                    for key, ref in (("temperature_ad", r["temperature_k"].sum(axis=1)),
                                     ("cloud_water_content_ad", r["cloud_water_content_k"].sum(axis=1)),
                                     ("cloud_effective_radius_ad", r["cloud_effective_radius_k"].sum(axis=1))):
                        if key in g:
                            e = float(np.abs(g[key] - ref).max() / max(np.abs(ref).max(), 1e-300))
                            vs_oracle[form][key] = max(vs_oracle[form].get(key, 0.0), e)
                continue
            merge_errors(vs_oracle["fp64"], scatter_errors(g64, r, a))
            merge_errors(vs_oracle["mixed"], scatter_errors(gmx, r, a))
    if rank == 0:
        cfg = {"workload": name + ": " + SCATTER_WORKLOAD[name],
               "groups": [{"sensor": c_[0], "profiles": int(c_[1].n_profiles),
                           "layers_max": int(c_[1].max_layers),
                           "cloudy_profiles": int((c_[1].n_clouds > 0).sum())} for c_ in groups],
               "parallelism": f"replicas x{world}",
               "l2": "inputs and per-step intermediates far larger than L2, no flush"}
        line = {"metric": SCATTER_METRIC[name], "value": value, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_mixed,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "mixed f32/f64",
                "data": "synthetic", "config": cfg,
                "fp64_gpu": {"value": fp64_value, "ms_per_step": per_fp64, "steps": fp64_steps},
                "speedup_mixed_vs_fp64": value / fp64_value,
                "accuracy_mixed_vs_fp64": {"max_abs_bt_K": bt_err, "max_rel_jacobian": jac_err,
                                           "by_output": field_err, "profiles_compared_per_group": 512},
                "accuracy_vs_oracle": vs_oracle,
                "stages_ms_per_step": stage_ms,
                "stage_launches_per_step": {k: v[1] // args.steps for k, v in st.items() if v[1] > 0},
                "gpu_launches": int(launches), "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
                "clocks": clk.summary(), **extra}
        print(json.dumps(line))
    return 0


def run_case(args, torch, dev) -> int:
    """Fixed cases for kernel captures and trajectory timing, one JSON line each.

    cloudy-k48: one mixed-form K-matrix of 48 ``irsynth_c616`` profiles, 100
    layers, liquid and ice clouds (``cloudy_workload(..., wc_scale=3.0)``),
    stream rule -- the small case on which the scattering kernels are captured.
    trajectory: ``linearize_device`` of ``--profiles`` clear-sky
    ``irsynth_c2211`` profiles (101 layers, mixed form), then the tangent
    linear (temperature and absorber perturbations) and the adjoint (a seed of
    ones) applied from the stored Jacobians; CUDA events on the calling
    stream, one untimed call first, linearize averaged over 3 calls and the
    applications over 10."""
    from crtmv3_gb300 import api, coefficients as co
    d = tempfile.mkdtemp(prefix="crtm_case_")
    if args.workload == "cloudy-k48":
        sensor, P = "irsynth_c616", 48
        sy.write_sensor_files(d, sensor)
        sy.write_cloud_files(d)
        atm, sfc, geo, opt = sy.cloudy_workload(sensor, P, 100, 7, cloud_types=(co.WATER_CLOUD, co.ICE_CLOUD),
                                                wc_scale=3.0)
        h = api.CRTM([sensor], d, api.MIXED)
        km, rts = h.k_matrix(atm, sfc, geo, opt)
        print(json.dumps({"workload": "cloudy-k48", "sensor": sensor, "profiles": P,
                          "max_bt": float(np.abs(rts.brightness_temperature).max()),
                          "status": int(np.abs(rts.status).max())}))
        return 0
    sensor, P = SENSOR, args.profiles
    sy.write_sensor_files(d, sensor)
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, P, N_LAYERS, 11)
    h = api.CRTM([sensor], d, api.MIXED)
    L, K, J = h.n_channels[0], atm.max_layers, atm.n_absorbers
    b, keep, t = scatter_device_inputs(torch, h, atm, sfc, geo, opt, dev)
    f64 = dict(dtype=torch.float64, device=dev)
    traj = dict(radiance=torch.zeros((P, L), **f64), bt=torch.zeros((P, L), **f64),
                status=torch.zeros((P,), dtype=torch.int32, device=dev))
    st = torch.cuda.current_stream(dev)
    sp = st.cuda_stream
    rng = np.random.default_rng(1)
    tl = dict(temperature=torch.from_numpy(rng.standard_normal((P, K))).to(dev),
              absorber=torch.from_numpy(rng.standard_normal((P, J, K)) * 0.01).to(dev))
    bt_tl = torch.zeros((P, L), **f64)
    seed = torch.ones((P, L), **f64)
    out = dict(temperature_ad=torch.zeros((P, K), **f64), absorber_ad=torch.zeros((P, J, K), **f64),
               water_temperature_ad=torch.zeros((P,), **f64))

    def timed(fn, n):
        fn()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(n):
            fn()
        e1.record(st)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / n
    t_lin = timed(lambda: h.linearize_device(b, traj, 0, sp), 3)
    t_tl = timed(lambda: h.tangent_linear_apply_device(tl, bt_tl, sp), 10)
    t_ad = timed(lambda: h.adjoint_apply_device(seed, out, sp), 10)
    kbytes = P * L * (K * (1 + J) + 5) * 8     # stored T, absorber and surface Jacobians
    print(json.dumps({"workload": "trajectory", "sensor": sensor, "profiles": P, "channels": L, "layers": K,
                      "absorbers": J, "stored_jacobian_gb": kbytes / 1e9, "linearize_ms": t_lin,
                      "tl_apply_ms": t_tl, "tl_apply_gbs": kbytes / t_tl / 1e6,
                      "ad_apply_ms": t_ad, "ad_apply_gbs": kbytes / t_ad / 1e6,
                      "status": int(traj["status"].abs().max().item())}))
    return 0


def local_rank() -> int:
    return int(os.environ.get("LOCAL_RANK", "0"))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--profiles", type=int, default=2000)
    ap.add_argument("--cpu-profiles", type=int, default=0,
                    help="CPU-baseline / oracle sample: profiles (C2, default 256) or profiles per sensor "
                         "group (C3-C5, default 32)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--workload", default="C5", choices=["C2", "C3", "C4", "C5", "cloudy-k48", "trajectory"],
                    help="C5 (default): the ragged mixed-sensor batch, 30%% cloudy, forward + K-matrix; "
                         "C2: clear-sky IR K-matrix; C3, C4: cloudy MW adjoint, all-sky IR K-matrix; "
                         "cloudy-k48, trajectory: the fixed cases of run_case (not bench lines)")
    ap.add_argument("--autotune", action="store_true",
                    help="C2: pick the map tile and profiles per pass of each form with the "
                         "library's autotuner before the warm-up (default: the built-in 16 channels "
                         "per map CTA, no pass cap)")
    args = ap.parse_args()
    if not args.cpu_profiles:
        args.cpu_profiles = 256 if args.workload == "C2" else 32
    if args.impl == "reference":
        if args.workload in ("cloudy-k48", "trajectory"):
            print(json.dumps({"impl": "reference", "unavailable": f"{args.workload} is a kernel-capture case, "
                              "not a bench workload"}))
            return 0
        return run_reference(args)

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from crtmv3_gb300 import api, build
    build.build()
    if args.workload in ("cloudy-k48", "trajectory"):
        return run_case(args, torch, dev)
    if args.workload != "C2":
        rc = run_scattering(args, torch, dev, rank, world, dist)
        if dist:
            dist.destroy_process_group()
        return rc
    if rank == 0:
        sy.write_sensor_files(COEFF_DIR, SENSOR)
    if dist:
        dist.barrier()

    P, K, L = args.profiles, N_LAYERS, 2211
    atm, sfc, geo, opt = make_workload(P, 3000 + rank)
    sel = jacobian_sel(atm)     # H2O, O3 Jacobians
    JK = len(sel)
    h = api.CRTM([SENSOR], COEFF_DIR, api.FP64)
    b, keep, dev_in = device_batch(torch, h, atm, sfc, geo, opt, dev)
    # a dedicated stream: the library enqueues on it and the CUDA events below time it
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    sptr = stream.cuda_stream
    out = {0: k_outputs(torch, P, L, K, JK, dev), 1: k_outputs(torch, P, L, K, JK, dev)}

    def step(prec):
        h.set_precision(prec)
        h.k_matrix_device(b, out[prec], None, 0, sptr, k_absorbers=sel)

    def timed(prec, n):
        torch.cuda.synchronize(dev)
        if dist:
            dist.barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            step(prec)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return max_over_ranks(e0.elapsed_time(e1), dist, dev)

    tuning = None
    if args.autotune:   # untimed: each candidate runs the full K-matrix three times
        tuning = {}
        for prec, form in ((1, "mixed"), (0, "fp64")):
            h.set_precision(prec)
            r = h.autotune_k_matrix_device(b, out[prec], None, 0, sptr, reps=2, k_absorbers=sel)
            tuning[form] = dict(r["chosen"], trials=r["trials"])
    for _ in range(args.warmup):
        step(1)
    for _ in range(max(1, min(args.warmup, 2))):
        step(0)
    torch.cuda.synchronize(dev)
    launches0 = h.launch_count()
    # per-stage kernel times: CUDA events around every launch on the launching
    # stream, recorded by the library during the timed steps themselves
    h.set_profiling(True)
    h.stage_times(reset=True)
    with ClockSampler(local) as clk:
        ms_mixed = timed(1, args.steps)
    st = h.stage_times(reset=True)
    h.set_profiling(False)
    launches_mixed = (h.launch_count() - launches0) // args.steps
    fp64_steps = max(1, min(args.steps, 3))
    ms_fp64 = timed(0, fp64_steps)
    per_mixed = ms_mixed / args.steps
    per_fp64 = ms_fp64 / fp64_steps
    pc = P * L * world
    value = pc / (per_mixed * 1e-3)
    fp64_value = pc / (per_fp64 * 1e-3)

    # accuracy of the mixed form against the all-FP64 form (same inputs, full workload)
    a, r = out[1], out[0]
    bt_err = float((a["bt"] - r["bt"]).abs().max())

    def rel(x, y):
        return float((x - y).abs().max() / y.abs().max().clamp_min(1e-300))
    jac_err = max(rel(a["temperature_k"], r["temperature_k"]), rel(a["absorber_k"], r["absorber_k"]),
                  rel(a["water_temperature_k"], r["water_temperature_k"]))

    stage_ms = {k: v[0] / args.steps for k, v in st.items() if v[1] > 0}
    stage_launch = {k: v[1] // args.steps for k, v in st.items() if v[1] > 0}
    hbm, bf16, peak_kind = peaks()
    # Algorithmic bytes per profile*channel of each stage in the mixed form (FP32
    # intermediates, FP64 outputs; K_r = 100 reference layers, K_u = 101 user
    # layers, 2 absorber Jacobians), and the DRAM bytes per profile*channel that
    # ncu measured for the same kernels on a 192-profile case of this workload
    # (profiles/kmatrix_c2_kernels.md).
    kr, ku = 100, K
    algo_pc = {
        "map_out": (1 + JK) * kr * 4 + ku * 4 + 4 + (1 + JK) * ku * 8,
        "column": kr * 4 + 2 * 2 * ku * 4 + kr * 4 + kr * 4 + ku * 4 + 36,
        "absorb_ad": kr * 4 + 4 + (1 + JK) * kr * 4,
        "absorb_fwd": kr * 4,
    }
    ncu_pc = {"map_out": 3908.0, "column": 2568.0, "absorb_ad": 1934.0, "absorb_fwd": 495.0}
    kernels = {}
    for st_name, ms in stage_ms.items():
        if st_name not in algo_pc:
            continue
        kernels[st_name] = {"ms_per_step": ms,
                            "achieved_gbs": algo_pc[st_name] * P * L / (ms * 1e-3) / 1e9,
                            "algorithmic_bytes_per_pc": algo_pc[st_name]}
    dom = max(kernels, key=lambda k: kernels[k]["ms_per_step"])
    n_launch = stage_launch[dom]
    pc_launch = P * L / n_launch
    achieved = kernels[dom]["achieved_gbs"]
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "traffic": ncu_pc[dom] * pc_launch,
                "algorithmic_bytes": algo_pc[dom] * pc_launch, "kernel": dom,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"}

    # end to end through the C-ABI with host (pinned) buffers, mixed form
    e2e = None
    if not args.no_e2e:
        from crtmv3_gb300.structures import KMatrixBatch

        def pin(shape):
            return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
        kout = KMatrixBatch(pin((P, L, K)), pin((P, L, JK, K)), pin((P, L)), pin((P, L)))
        patm, psfc, pgeo, popt = (pinned_copy(torch, x) for x in (atm, sfc, geo, opt))
        prts = pinned_rts(torch, P, L)
        h.set_precision(1)
        h.k_matrix(patm, psfc, pgeo, popt, None, 0, k_absorbers=sel, out=kout, rts_out=prts)
        n_e2e = max(1, min(args.steps, 3))
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(n_e2e):
            h.k_matrix(patm, psfc, pgeo, popt, None, 0, k_absorbers=sel, out=kout, rts_out=prts)
        dt = (time.perf_counter() - t0) / n_e2e
        h2d = sum(x.nbytes for x in (atm.level_pressure, atm.pressure, atm.temperature, atm.absorber,
                                     opt.emissivity)) + 10 * P * 8 + P * 4
        d2h = P * L * 8 * (2 + K + JK * K + 2) + P * 4
        # the host link bounds this figure: plain pinned device-to-host copy rate
        nb = 1 << 28
        dsrc = torch.empty(nb, dtype=torch.float64, device=dev)
        hdst = torch.empty(nb, dtype=torch.float64, pin_memory=True)
        hdst.copy_(dsrc)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(3):
            hdst.copy_(dsrc, non_blocking=True)
        torch.cuda.synchronize(dev)
        d2h_gbs = 3 * nb * 8 / (time.perf_counter() - t0) / 1e9
        del dsrc, hdst
        e2e = {"value": pc / dt, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": dt * 1e3,
               "d2h_copy_gbs": d2h_gbs, "d2h_bound_ms": d2h / d2h_gbs / 1e6}

    cpu = None
    vs_oracle = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v, dt, calls, sample, ref = cpu_baseline(args.cpu_profiles, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{calls} K-matrix calls of {args.cpu_profiles} profiles x 2211 channels x "
                         f"{N_LAYERS} layers (H2O and O3 Jacobians, as the GPU arm), FP64 C oracle "
                         f"with OpenMP over profiles, {dt:.1f} s"}
        # both GPU forms against the oracle on the same sample (untimed)
        vs_oracle = {"mixed": oracle_errors(h, sample, ref, 1), "fp64": oracle_errors(h, sample, ref, 0)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": per_mixed, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "mixed f32/f64", "data": "synthetic",
            "config": dict(workload_config(P, world),
                           tuning="autotuned" if tuning else "default (16 channels per map CTA, no pass cap)"),
            "fp64_gpu": {"value": fp64_value, "ms_per_step": per_fp64, "steps": fp64_steps},
            "speedup_mixed_vs_fp64": value / fp64_value,
            "accuracy_mixed_vs_fp64": {"max_abs_bt_K": bt_err, "max_rel_jacobian": jac_err},
            "accuracy_vs_oracle": vs_oracle,
            "stages_ms_per_step": stage_ms, "stage_launches_per_step": stage_launch,
            "kernels": kernels, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": int(launches_mixed * args.steps),
            "clocks": clk.summary(),
        }
        if tuning:
            line["tuning"] = tuning
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
