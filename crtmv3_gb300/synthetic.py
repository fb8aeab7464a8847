"""Seeded synthetic profiles and coefficient tables for the benchmark workloads.

No real coefficient files or profile sets are used: every input is generated
here from the distributions below and written with the repository's own
coefficient writers (``coefficients.py``), so the oracle and the GPU library
read identical files.

Profiles (all workloads): levels log-spaced from 0.005 hPa (the reference's
``TOA_PRESSURE``, ``src/CRTM_Parameters.f90:157``) to the surface; temperature a
US-standard lapse profile plus Gaussian noise; water vapour exponential with a
2 km scale height (surface 5-20 g/kg); ozone a Chapman-shaped layer peaking
near 10 hPa; CO2 400 +- 10 ppmv; CH4, N2O and CO near background values.
Ocean surface with skin temperature U[270, 305] K, sensor zenith U[0, 60] deg.

ODPS coefficients: for each channel and each active component a column
optical depth is drawn log-uniformly; the component's layer optical depth at
the reference profile is that column spread over layers by a physical shape
(pressure-broadened dry air, water vapour, ozone, well-mixed trace gases).
The leading predictor of each component carries that optical depth and the
remaining predictors add small Gaussian perturbations, so layer optical depths
span about 1e-4 to 2 and occasionally go negative (exercising the clamp).
"""
from __future__ import annotations

import os
from typing import Dict, Optional, Sequence, Tuple

import numpy as np

from . import coefficients as co
from .structures import AtmosphereBatch, GeometryBatch, OptionsBatch, SurfaceBatch

TOA_PRESSURE = 0.005
SURFACE_PRESSURE = 1100.0
C1_RADIATION = 1.191042722e-05   # 2hc^2 in mW/(m2.sr.cm-4)
C2_RADIATION = 1.4387752         # hc/k in K.cm
TSPACE = 2.7253                  # ``src/CRTM_Parameters.f90:173``

# background mixing ratios (ppmv) and the water vapour floor (g/kg)
BACKGROUND_PPMV = {co.CO2_ID: 400.0, co.N2O_ID: 0.32, co.CO_ID: 0.10, co.CH4_ID: 1.80}
H2O_FLOOR = 3.0e-3


def height_km(p: np.ndarray) -> np.ndarray:
    return -7.0 * np.log(np.asarray(p) / 1013.25)


def us_standard_temperature(z: np.ndarray) -> np.ndarray:
    """Piecewise-linear US standard atmosphere temperature (K) at height z (km)."""
    zs = np.array([0.0, 11.0, 20.0, 32.0, 47.0, 51.0, 71.0, 86.0, 200.0])
    ts = np.array([288.15, 216.65, 216.65, 228.65, 270.65, 270.65, 214.65, 186.87, 186.87])
    return np.interp(np.clip(z, 0.0, 200.0), zs, ts)


def layer_mean_pressure(lev: np.ndarray) -> np.ndarray:
    return (lev[..., 1:] - lev[..., :-1]) / np.log(lev[..., 1:] / lev[..., :-1])


def h2o_profile(p: np.ndarray, q_sfc) -> np.ndarray:
    q = np.asarray(q_sfc)[..., None] * np.exp(-np.clip(height_km(p), 0.0, None) / 2.0)
    return np.maximum(q, H2O_FLOOR)


def o3_profile(p: np.ndarray, amp) -> np.ndarray:
    """Chapman layer in height with its peak at the 10 hPa height."""
    x = (height_km(p) - height_km(10.0)) / 5.0
    return np.asarray(amp)[..., None] * np.exp(1.0 - x - np.exp(-x)) + 0.03


def ref_level_pressure(n_layers: int = 100) -> np.ndarray:
    """The ODPS reference grid: p^(1/3.5) quadratic in the level index."""
    s0, s1 = TOA_PRESSURE ** (1 / 3.5), SURFACE_PRESSURE ** (1 / 3.5)
    x = np.arange(n_layers + 1) / n_layers
    return (s0 + (s1 - s0) * (0.35 * x + 0.65 * x * x)) ** 3.5


def absorber_set(group: int) -> Tuple[int, ...]:
    return co.ABSORBER_ID_G[group]


def _profile_absorber(aid: int, p: np.ndarray, rng, P: int, q_sfc, o3_amp) -> np.ndarray:
    if aid == co.H2O_ID:
        return h2o_profile(p, q_sfc)
    if aid == co.O3_ID:
        return o3_profile(p, o3_amp)
    base = BACKGROUND_PPMV[aid]
    if aid == co.CO2_ID:
        col = base + rng.uniform(-10.0, 10.0, size=P)
    else:
        col = base * rng.uniform(0.9, 1.1, size=P)
    return np.broadcast_to(col[:, None], p.shape) * (1.0 + 0.01 * rng.standard_normal(p.shape))


def generate_profiles(n_profiles: int, n_layers, absorber_ids: Sequence[int], seed: int,
                      p_sfc: float = SURFACE_PRESSURE):
    """Profiles, ocean surfaces and view geometries.

    ``n_layers`` is an int or a (P,) array for ragged batches.
    Returns (AtmosphereBatch, SurfaceBatch, GeometryBatch).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    P = n_profiles
    nl = np.broadcast_to(np.asarray(n_layers, dtype=np.int32), (P,)).copy()
    K = int(nl.max())
    lev = np.zeros((P, K + 1))
    for m in range(P):
        n = int(nl[m])
        lev[m, :n + 1] = np.geomspace(TOA_PRESSURE, p_sfc, n + 1)
        lev[m, n + 1:] = p_sfc
    lev_pad = lev.copy()
    # padding levels past a short profile's surface keep positive thickness
    for m in range(P):
        n = int(nl[m])
        if n < K:
            lev_pad[m, n + 1:] = p_sfc * (1.0 + 0.01 * np.arange(1, K - n + 1))
    lay = layer_mean_pressure(lev_pad)
    temp = us_standard_temperature(height_km(lay)) + rng.normal(0.0, 5.0, size=lay.shape)
    temp = np.clip(temp, 160.0, 340.0)
    q_sfc = rng.uniform(5.0, 20.0, size=P)
    o3_amp = rng.uniform(4.0, 9.0, size=P)
    absorbers = np.stack([_profile_absorber(a, lay, rng, P, q_sfc, o3_amp)
                          for a in absorber_ids], axis=1)
    units = np.array([co.MASS_MIXING_RATIO_UNITS if a == co.H2O_ID else co.VOLUME_MIXING_RATIO_UNITS
                      for a in absorber_ids], np.int32)
    for m in range(P):
        n = int(nl[m])
        lev[m, n + 1:] = 0.0
        lay[m, n:] = 0.0
        temp[m, n:] = 0.0
        absorbers[m, :, n:] = 0.0
    atm = AtmosphereBatch(nl, lev, lay, temp, np.ascontiguousarray(absorbers),
                          np.asarray(absorber_ids, np.int32), units)
    sfc = SurfaceBatch.ocean(rng.uniform(270.0, 305.0, size=P))
    geo = GeometryBatch.nadir_like(rng.uniform(0.0, 60.0, size=P))
    return atm, sfc, geo


# ---------------------------------------------------------------------------
# Coefficients
# ---------------------------------------------------------------------------

def _ref_profile(group: int, lev: np.ndarray):
    lay = layer_mean_pressure(lev)
    T = us_standard_temperature(height_km(lay))
    ab = []
    for a in absorber_set(group):
        if a == co.H2O_ID:
            ab.append(h2o_profile(lay[None], np.array([10.0]))[0])
        elif a == co.O3_ID:
            ab.append(o3_profile(lay[None], np.array([6.0]))[0])
        else:
            ab.append(np.full(lay.shape, BACKGROUND_PPMV[a]))
    return lay, T, np.stack(ab, axis=1)


def predictors_numpy(group: int, T, A, Tref, Aref, lev, secang):
    """Predictors X[..., k, i, j] of ``ODPS_Predictor.f90:645-1095`` for arrays
    T (..., K), A (..., K, Jm); used only to scale synthetic coefficients."""
    K = T.shape[-1]
    pdp = np.empty(K)
    pdp[0] = lev[0] * (lev[1] - lev[0])
    pdp[1:] = lev[1:K] * (lev[1:K] - lev[0:K - 1])
    Tz = np.cumsum(T, -1) / np.cumsum(Tref)
    Tzp = np.cumsum(pdp * T, -1) / np.cumsum(pdp * Tref)
    GAzp = np.cumsum(pdp[:, None] * A, -2) / np.cumsum(pdp[:, None] * Aref, 0)
    GATzp = np.cumsum(pdp[:, None] * A * T[..., None], -2) / np.cumsum(pdp[:, None] * Aref * Tref[:, None], 0)
    dT = T - Tref
    t = T / Tref
    t2 = t * t
    dT2 = dT * np.abs(dT)
    s = secang
    R = A / Aref
    nmax = max(co.N_PREDICTORS_G[group])
    X = np.zeros(T.shape + (nmax, co.N_COMPONENTS_G[group]))
    h2o = R[..., 0]
    h2o_a = s * h2o
    h2o_r = np.sqrt(h2o_a)
    h2o_s = h2o_a * h2o_a
    dry = [s + 0 * t, s * t, s * t2, t, s * s + 0 * t, t2, Tz]
    for i, v in enumerate(dry):
        X[..., i, 0] = v
    if group == 3:
        h2otz = h2o / GATzp[..., 0]
        wet = [h2o_a / t, h2o_a / t * h2o, h2o_a / t2 * h2o / t2, h2o_a / t2, h2o_a / t2 * h2o,
               h2o_a / t2 ** 2, h2o_a, h2o_a * dT, (s * GAzp[..., 0]) ** 2, s * GAzp[..., 0],
               s + 0 * t, h2o_s * h2o_a, h2o_s * h2o_s, h2otz]
        for i, v in enumerate(wet):
            X[..., i, 1] = v
        return X
    o3 = R[..., 1]
    co2 = R[..., 2]
    o3_a = s * o3
    o3_r = np.sqrt(o3_a)
    g_o3 = GAzp[..., 1]
    h2otz = h2o / GATzp[..., 0]
    wco = [h2o_a / t, h2o_a / t * h2o, h2o_a / t2 * h2o / t2, h2o_a / t2, h2o_a / t2 * h2o,
           h2o_a / t2 ** 2, h2o_a]
    ozo = [o3_a, o3_a * dT, o3_a * o3 * g_o3, o3_a * o3_a, o3_a * g_o3, o3_a * np.sqrt(s * g_o3),
           o3_r * dT, o3_r, o3_r * o3 / g_o3, s * g_o3, (s * g_o3) ** 2]
    co2p = [s * t, s * t2, t, t2, s + 0 * t, s * co2, s * Tzp, (s * GAzp[..., 2]) ** 2, Tzp ** 3,
            s * Tzp * np.sqrt(t)]
    wlo = [h2o_a, h2o_a * dT, h2o_s, h2o_a * dT2, np.sqrt(h2o_r), h2o_s * h2o_a, h2o_r,
           h2o_r * dT, h2o_s * h2o_s, h2otz, h2o_r * h2otz, (s * GAzp[..., 0]) ** 2,
           s * GAzp[..., 0], s + 0 * t, s * co2]
    for i, v in enumerate(wlo):
        X[..., i, 1] = v
    for i, v in enumerate(wco):
        X[..., i, 2] = v
    for i, v in enumerate(ozo):
        X[..., i, 3] = v
    for i, v in enumerate(co2p):
        X[..., i, 4] = v
    if group == 1:
        n2o, co_, ch4 = R[..., 3], R[..., 4], R[..., 5]
        n2o_a, co_a, ch4_a = s * n2o, s * co_, s * ch4
        n2o_r, co_r, ch4_r = np.sqrt(n2o_a), np.sqrt(co_a), np.sqrt(ch4_a)
        g_co, g_ch4, g_n2o = GAzp[..., 4], GAzp[..., 5], GAzp[..., 3]
        co_ac = co_a * co_ / g_co
        ch4_z = s * g_ch4
        X[..., 10, 4] = co_a
        X[..., 15, 1] = ch4_a
        X[..., 16, 1] = ch4_a * ch4_a * dT
        X[..., 17, 1] = co_a
        cop = [co_a, co_a * dT, np.sqrt(co_r), co_r * dT, co_a * co_a, co_r, co_a * dT2, co_ac,
               co_ac / co_r, co_ac * np.sqrt(g_co)]
        ch4p = [ch4_a * dT, ch4_r, ch4_a * ch4_a, ch4_a, ch4 * dT, ch4_z, ch4_z ** 2, np.sqrt(ch4_r),
                GATzp[..., 5], s * GATzp[..., 5], ch4_r * ch4 / g_ch4]
        n2op = [n2o_a * dT, n2o_r, n2o * dT, n2o_a ** 0.25, n2o_a, s * g_n2o, s * GATzp[..., 3],
                n2o_a * n2o_a, GATzp[..., 3], n2o_r * n2o / g_n2o, ch4_a, ch4_a * g_ch4, co_a,
                co_a * s * g_co]
        for i, v in enumerate(n2op):
            X[..., i, 5] = v
        for i, v in enumerate(cop):
            X[..., i, 6] = v
        for i, v in enumerate(ch4p):
            X[..., i, 7] = v
    return X


# Probability that a component is active in a channel, and its column-OD range.
_COMPONENT_RULES = {
    # group: list over components of (probability, (lo, hi) column optical depth)
    1: [(1.0, (0.005, 3.0)), (1.0, (0.001, 20.0)), (1.0, (0.001, 2.0)), (0.3, (0.01, 8.0)),
        (0.5, (0.01, 30.0)), (0.2, (0.005, 2.0)), (0.15, (0.005, 2.0)), (0.2, (0.005, 2.0))],
    2: [(1.0, (0.005, 3.0)), (0.8, (0.001, 15.0)), (0.5, (0.001, 1.5)), (0.3, (0.01, 6.0)),
        (0.3, (0.01, 20.0))],
    3: [(1.0, (0.005, 6.0)), (1.0, (0.001, 10.0))],
}


def _component_shapes(group: int, lev: np.ndarray, lay: np.ndarray, A: np.ndarray) -> np.ndarray:
    """Fraction of each component's column optical depth in each reference layer."""
    dp = np.diff(lev)
    broad = np.sqrt(lay / SURFACE_PRESSURE)
    J = co.N_COMPONENTS_G[group]
    ids = absorber_set(group)
    f = np.zeros((J, lay.size))
    f[0] = dp * broad
    if group == 3:
        f[1] = dp * A[:, 0] * broad
    else:
        f[1] = dp * A[:, 0] * broad
        f[2] = dp * A[:, 0] ** 2 * lay / SURFACE_PRESSURE
        f[3] = dp * A[:, ids.index(co.O3_ID)]
        f[4] = dp * broad
        for j in range(5, J):
            f[j] = dp * broad
    return f / f.sum(axis=1, keepdims=True)


def generate_odps(group: int, n_channels: int, seed: int, sensor_id: str, sensor_type: int,
                  n_ref_layers: int = 100, max_predictors_per_channel: Optional[int] = None) -> co.ODPSCoeff:
    """A synthetic ODPS TauCoeff for ``n_channels`` channels of predictor ``group``."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lev = ref_level_pressure(n_ref_layers)
    lay, Tref, Aref = _ref_profile(group, lev)
    K = n_ref_layers
    J = co.N_COMPONENTS_G[group]
    ncp = co.N_PREDICTORS_G[group]
    # typical predictor values over sample states near the reference
    ns = 48
    srng = np.random.Generator(np.random.PCG64(seed + 7))
    Ts = Tref[None] + srng.normal(0.0, 5.0, (ns, K))
    As = Aref[None] * np.exp(srng.normal(0.0, 0.3, (ns, K, Aref.shape[1])))
    sec = 1.0 / np.cos(np.deg2rad(30.0))
    Xs = predictors_numpy(group, Ts, As, Tref, Aref, lev, sec)
    x_mean = Xs.mean(axis=0)
    x_rms = np.sqrt((Xs ** 2).mean(axis=0)) + 1e-30
    shapes = _component_shapes(group, lev, lay, Aref)
    rules = _COMPONENT_RULES[group]
    npred = np.zeros((J, n_channels), np.int32)
    pos = np.zeros((J, n_channels), np.int32)
    blocks = []
    cursor = 1
    for l in range(n_channels):
        budget = max_predictors_per_channel
        for j in range(J):
            prob, (lo, hi) = rules[j]
            if j > 0 and rng.uniform() >= prob:
                continue
            n = int(rng.integers(max(1, ncp[j] - 4), ncp[j] + 1))
            if budget is not None:
                n = min(n, budget - (0 if j > 0 else 0))
                if j == 0:
                    n = min(ncp[0], budget)
                if n <= 0:
                    continue
                budget -= n
            col = np.exp(rng.uniform(np.log(lo), np.log(hi)))
            od = col * shapes[j]
            c = np.empty((n, K))
            c[0] = od / x_mean[:, 0, j]
            if n > 1:
                c[1:] = (od[None, :] / x_rms[:, 1:n, j].T) * rng.normal(0.0, 0.05, (n - 1, K)) / np.sqrt(n - 1)
            npred[j, l] = n
            pos[j, l] = cursor
            cursor += n * K
            blocks.append(c.astype(np.float32).ravel())
    cvec = np.concatenate(blocks) if blocks else np.zeros(0, np.float32)
    ids = absorber_set(group)
    amin = Aref * 0.001
    amax = Aref * 50.0
    for jj, a in enumerate(ids):
        if a != co.H2O_ID:
            amin[:, jj] = Aref[:, jj] * 0.02
            amax[:, jj] = Aref[:, jj] * 20.0
    return co.ODPSCoeff(group, sensor_id, sensor_type, np.arange(1, n_channels + 1, dtype=np.int32),
                        lev, lay, Tref, Aref, amin, amax, npred, pos, cvec)


def generate_spccoeff(sensor_id: str, sensor_type: int, n_channels: int, seed: int) -> co.SpcCoeff:
    rng = np.random.Generator(np.random.PCG64(seed))
    L = n_channels
    if sensor_type == co.MICROWAVE_SENSOR:
        freq = np.sort(rng.uniform(23.0, 190.0, L))           # GHz
        wn = freq / 29.9792458
        b1 = np.zeros(L)
        b2 = np.ones(L)
    else:
        wn = np.sort(rng.uniform(650.0, 2550.0, L))
        freq = wn * 29.9792458
        b1 = rng.uniform(0.0, 0.3, L)
        b2 = rng.uniform(0.9995, 1.0, L)
    c1 = C1_RADIATION * wn ** 3
    c2 = C2_RADIATION * wn
    cbr = np.zeros(L)
    if sensor_type == co.MICROWAVE_SENSOR:
        cbr = c1 / (np.exp(c2 / (b1 + b2 * TSPACE)) - 1.0)
    return co.SpcCoeff(sensor_id, sensor_type, np.arange(1, L + 1, dtype=np.int32), freq, wn,
                       c1, c2, b1, b2, cbr, np.zeros(L))


# ---------------------------------------------------------------------------
# Workloads
# ---------------------------------------------------------------------------

SENSORS = {
    # sensor id: (group, channels, sensor type, seed)
    "mwsynth_c22": (2, 22, co.MICROWAVE_SENSOR, 11),
    "irsynth_c2211": (1, 2211, co.INFRARED_SENSOR, 12),
    "mwsynth_c16": (3, 16, co.MICROWAVE_SENSOR, 13),
    "irsynth_c616": (1, 616, co.INFRARED_SENSOR, 14),
    "irsynth_o120": (1, 120, co.INFRARED_SENSOR, 15),   # with a compact-OPTRAN water-vapour-line term
}
OPTRAN_SENSORS = ("irsynth_o120",)


def generate_optran(tc: co.ODPSCoeff, seed: int, fraction: float = 0.6) -> co.OPTRANCoeff:
    """A synthetic compact-OPTRAN term (ODPS_Define.f90:186-203) for the water
    vapour line component (component 2) of ``fraction`` of the channels that
    have one: 2-6 predictors among T, P, P^(1/4), the water vapour amount, its
    ratio to T^2 and the integrated T* and P*, and polynomials of order 2-5 in
    the transformed integrated water vapour Ap = ln((A - C2) / C1) / Alpha,
    scaled so that ln(chi) stays near -4 +- 1 over the workload's profiles."""
    rng = np.random.Generator(np.random.PCG64(seed))
    L = tc.n_channels
    nu = co.N_PREDICTOR_USED_OPTRAN + 1
    sig = np.zeros(L, np.int32)
    order = np.zeros(L, np.int32)
    opi = np.zeros((nu, L), np.int32)
    opos = np.zeros(L, np.int32)
    # typical magnitudes of OX 1-14 (T, P, T^2, P^2, TP, T^2P, TP^2, T^2P^2, P^1/4, V, V/T^2, T*, P*, sec)
    typ = np.array([250.0, 500.0, 6.0e4, 3.0e5, 1.2e5, 3.0e7, 6.0e7, 1.5e10, 4.0, 3.0, 5.0e-5, 500.0, 800.0, 1.3])
    pool = np.array([1, 2, 9, 10, 11, 12, 13])
    blocks = []
    cursor = 1
    for l in range(L):
        if tc.n_predictors[1, l] <= 0 or rng.uniform() >= fraction:
            continue
        npred = int(rng.integers(2, co.N_PREDICTOR_USED_OPTRAN + 1))
        preds = np.sort(rng.choice(pool, size=min(npred, pool.size), replace=False))
        npred = preds.size
        n_ord = int(rng.integers(2, 6))
        c = np.zeros((npred + 1, n_ord + 1))
        c[0, 0] = rng.uniform(-4.5, -3.5)
        c[0, 1:] = rng.normal(0.0, 0.3, n_ord) / 3.0 ** np.arange(1, n_ord + 1)
        for i, ii in enumerate(preds, start=1):
            c[i, 0] = rng.normal(0.0, 0.4) / typ[ii - 1]
            c[i, 1:] = rng.normal(0.0, 0.1, n_ord) / (typ[ii - 1] * 3.0 ** np.arange(1, n_ord + 1))
        sig[l] = co.SIGNIFICANCE_OPTRAN
        order[l] = n_ord
        opi[0, l] = npred
        opi[1:npred + 1, l] = preds
        opos[l] = cursor
        cursor += c.size
        blocks.append(c.ravel())
    oc = np.concatenate(blocks) if blocks else np.zeros(0)
    return co.OPTRANCoeff(sig, order, opi, opos, oc, 2.0, 1.0, -1.0e-4, 2)


def write_sensor_files(coeff_dir: str, sensor_id: str) -> None:
    """Write ``<sensor>.TauCoeff.bin`` and ``<sensor>.SpcCoeff.bin`` if missing."""
    os.makedirs(coeff_dir, exist_ok=True)
    tau = os.path.join(coeff_dir, f"{sensor_id}.TauCoeff.bin")
    spc = os.path.join(coeff_dir, f"{sensor_id}.SpcCoeff.bin")
    if os.path.exists(tau) and os.path.exists(spc):
        return
    group, L, stype, seed = SENSORS[sensor_id]
    budget = 20 if sensor_id == "mwsynth_c22" else None
    tc = generate_odps(group, L, seed, sensor_id, stype, max_predictors_per_channel=budget)
    if sensor_id in OPTRAN_SENSORS:
        tc.optran = generate_optran(tc, seed + 50)
    sc = generate_spccoeff(sensor_id, stype, L, seed + 100)
    co.write_odps(tau + ".tmp", tc)
    co.write_spccoeff(spc + ".tmp", sc)
    os.replace(tau + ".tmp", tau)
    os.replace(spc + ".tmp", spc)


def emissivity_for(sensor_type: int, n_profiles: int, n_channels: int, seed: int) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    if sensor_type == co.MICROWAVE_SENSOR:
        return rng.uniform(0.5, 0.7, (n_profiles, n_channels))
    return rng.uniform(0.95, 0.99, (n_profiles, n_channels))


def clear_sky_workload(sensor_id: str, n_profiles: int, n_layers, seed: int):
    """Profiles + options for a clear-sky run of one synthetic sensor."""
    group, L, stype, _ = SENSORS[sensor_id]
    atm, sfc, geo = generate_profiles(n_profiles, n_layers, absorber_set(group)
                                      if group != 2 or sensor_id != "mwsynth_c22"
                                      else (co.H2O_ID, co.O3_ID), seed)
    opt = OptionsBatch(emissivity=emissivity_for(stype, n_profiles, L, seed + 1))
    return atm, sfc, geo, opt


# ---------------------------------------------------------------------------
# Clouds: synthetic CloudCoeff LUT and cloudy profiles
# ---------------------------------------------------------------------------

CLOUD_N_LEGENDRE = 38       # >= 21 + 16 + 1: the 16-stream offset plus 16 terms fit


def _phase_terms(g: np.ndarray, n_leg: int) -> np.ndarray:
    """Legendre terms 0.5*g**l of a Henyey-Greenstein phase function in the
    reference's normalisation (term 0 is 1/2), shape g.shape + (n_leg+1,)."""
    return 0.5 * g[..., None] ** np.arange(n_leg + 1)


def generate_cloudcoeff(seed: int = 7) -> co.CloudCoeff:
    """Smooth synthetic cloud optical properties on the reference's LUT axes:
    8 MW frequencies x 30 radii x 6 temperatures (liquid) or 3 densities
    (frozen), 20 IR wavenumbers x 30 radii x 4 densities, 38 Legendre terms."""
    rng = np.random.Generator(np.random.PCG64(seed))
    f_mw = np.array([10.0, 19.0, 23.8, 31.4, 50.3, 89.0, 150.0, 190.0])
    r_mw = np.geomspace(5.0, 1000.0, 30)
    temp = np.array([233.0, 248.0, 263.0, 278.0, 293.0, 308.0])
    dens = np.array([100.0, 400.0, 900.0])
    f_ir = np.linspace(500.0, 3000.0, 20)
    r_ir = np.geomspace(2.0, 1000.0, 30)
    nl = CLOUD_N_LEGENDRE
    jit = lambda shape: 1.0 + 0.02 * rng.standard_normal(shape)   # noqa: E731
    # microwave liquid: size parameter x = 2 pi r f / c
    x = 2.0 * np.pi * r_mw[None, :, None] * f_mw[:, None, None] / 3.0e5
    tfac = 1.0 + 0.004 * (300.0 - temp[None, None, :])
    ke_l = 0.08 * (f_mw[:, None, None] / 10.0) ** 1.8 * (1.0 + 3.0 * x ** 2 / (1.0 + x ** 2)) * tfac
    w_l = np.clip(0.9 * x ** 2 / (1.0 + x ** 2) * np.ones_like(tfac), 0.0, 0.99)
    g_l = 0.8 * x / (1.0 + x) * np.ones_like(tfac)
    ke_l, w_l = ke_l * jit(ke_l.shape), w_l * jit(w_l.shape).clip(0.0, 1.0)
    pc_l = _phase_terms(g_l, nl)[..., None]
    # microwave frozen: density axis
    xs = 2.0 * np.pi * r_mw[None, :, None] * f_mw[:, None, None] / 3.0e5 * np.ones((1, 1, dens.size))
    dfac = 1.0 + 0.2 * np.arange(dens.size)[None, None, :]
    ke_s = 0.03 * (f_mw[:, None, None] / 10.0) ** 1.5 * (1.0 + 2.0 * xs ** 2 / (1.0 + xs ** 2)) * dfac
    w_s = np.clip(0.97 * xs ** 2 / (1.0 + xs ** 2), 0.0, 0.99)
    g_s = 0.75 * xs / (1.0 + xs)
    ke_s = ke_s * jit(ke_s.shape)
    pc_s = _phase_terms(g_s, nl)[..., None]
    # infrared: density axis 1..4 (1 liquid, 2-4 frozen)
    xi = 2.0 * np.pi * r_ir[None, :, None] * f_ir[:, None, None] / 1.0e4 * np.ones((1, 1, dens.size + 1))
    q = 2.0 - 1.5 / (1.0 + xi)
    ke_ir = 1.5e3 / r_ir[None, :, None] * q * (1.0 + 0.1 * np.arange(dens.size + 1)[None, None, :])
    band = 0.1 * np.sin(f_ir / 300.0)[:, None, None]
    w_ir = np.clip(0.5 + 0.45 * xi / (1.0 + xi) - band, 0.05, 0.999)
    g_ir = 0.85 * xi / (1.0 + xi)
    ke_ir = ke_ir * jit(ke_ir.shape)
    pc_ir = _phase_terms(g_ir, nl)[..., 1:, None]
    return co.CloudCoeff(f_mw, f_ir, r_mw, r_ir, temp, dens, ke_l, w_l, g_l, pc_l, ke_s, w_s, g_s,
                         pc_s, ke_ir, w_ir, g_ir, pc_ir)


def write_cloud_files(coeff_dir: str) -> str:
    """Write ``CloudCoeff.bin`` (the reference's default file name) if missing."""
    os.makedirs(coeff_dir, exist_ok=True)
    path = os.path.join(coeff_dir, "CloudCoeff.bin")
    if not os.path.exists(path):
        co.write_cloudcoeff(path + ".tmp", generate_cloudcoeff())
        os.replace(path + ".tmp", path)
    return path


# effective radius ranges (microns) by cloud type
REFF_RANGE = {co.WATER_CLOUD: (5.0, 20.0), co.ICE_CLOUD: (20.0, 200.0), co.RAIN_CLOUD: (100.0, 1000.0),
              co.SNOW_CLOUD: (100.0, 1000.0), co.GRAUPEL_CLOUD: (200.0, 1000.0),
              co.HAIL_CLOUD: (300.0, 1000.0)}


def add_clouds(atm: AtmosphereBatch, cloud_types: Sequence[int], seed: int, max_fraction: float = 0.3,
               wc_scale: float = 1.0, cover=None) -> AtmosphereBatch:
    """Give every profile the clouds ``cloud_types``: each active in a random
    0-``max_fraction`` of the layers, water content lognormal with geometric
    mean 0.05 g/m^2 x ``wc_scale`` and sigma_ln 1.2 (stored in kg/m^2, the
    reference's unit), effective radius uniform in the type's range.
    Cloud_Fraction is 1 in the cloudy layers (``cover`` None), or uniform in
    ``cover`` = (lo, hi) there; 0 elsewhere.  The reference drops clouds
    where the fraction is below 1e-12, and mixes a clear and a cloudy column
    by the overlap scheme's total cover when a cloudy layer's fraction is
    above 1e-6 (with fraction 1 the total cover is 1: one cloudy column)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    P, K = atm.n_profiles, atm.max_layers
    NC = len(cloud_types)
    wc = np.zeros((P, NC, K))
    reff = np.zeros((P, NC, K))
    for m in range(P):
        n = int(atm.n_layers[m])
        for c, t in enumerate(cloud_types):
            frac = rng.uniform(0.0, max_fraction)
            mask = rng.uniform(size=n) < frac
            wc[m, c, :n][mask] = 5.0e-5 * wc_scale * np.exp(1.2 * rng.standard_normal(mask.sum()))
            lo, hi = REFF_RANGE[t]
            reff[m, c, :n][mask] = rng.uniform(lo, hi, mask.sum())
    atm.n_clouds = np.full(P, NC, np.int32)
    atm.cloud_type = np.tile(np.asarray(cloud_types, np.int32), (P, 1))
    atm.cloud_water_content = wc
    atm.cloud_effective_radius = reff
    cloudy = (wc > 0).any(axis=1)
    if cover is None:
        atm.cloud_fraction = np.where(cloudy, 1.0, 0.0)
    else:
        rc = np.random.Generator(np.random.PCG64(seed + 1000003))
        atm.cloud_fraction = np.where(cloudy, rc.uniform(cover[0], cover[1], (P, K)), 0.0)
    return atm


def cloudy_workload(sensor_id: str, n_profiles: int, n_layers, seed: int,
                    cloud_types=(co.WATER_CLOUD, co.ICE_CLOUD, co.RAIN_CLOUD, co.SNOW_CLOUD,
                                 co.GRAUPEL_CLOUD), wc_scale: float = 1.0, n_streams=None):
    """A cloudy run of one synthetic sensor (``n_streams``: None for the
    reference's stream rule, or a per-profile array for Options%Use_N_Streams)."""
    atm, sfc, geo, opt = clear_sky_workload(sensor_id, n_profiles, n_layers, seed)
    add_clouds(atm, cloud_types, seed + 17, wc_scale=wc_scale)
    if n_streams is not None:
        ns = np.broadcast_to(np.asarray(n_streams, np.int32), (n_profiles,)).copy()
        opt.use_n_streams = ns > 0
        opt.n_streams = ns
    return atm, sfc, geo, opt


# ---------------------------------------------------------------------------
# Aerosols: synthetic AerosolCoeff LUT (scheme 'CRTM') and aerosol profiles
# ---------------------------------------------------------------------------

# the reference's aerosol type ids (CRTM_Parameters.f90:286-294), all eight in
# the synthetic table; the synthetic workloads load dust, sea salt (SSAM) and
# sulfate
(DUST_AEROSOL, SEASALT_SSAM_AEROSOL, SEASALT_SSCM1_AEROSOL, SEASALT_SSCM2_AEROSOL, SEASALT_SSCM3_AEROSOL,
 ORGANIC_CARBON_AEROSOL, BLACK_CARBON_AEROSOL, SULFATE_AEROSOL) = range(1, 9)
SEASALT_AEROSOL = SEASALT_SSAM_AEROSOL
AEROSOL_TABLE_TYPES = tuple(range(1, 9))
AEROSOL_TABLE_NAMES = ["Dust", "SeaSalt(SSAM)", "SeaSalt(SSCM1)", "SeaSalt(SSCM2)", "SeaSalt(SSCM3)",
                       "Organic carbon", "Black carbon", "Sulfate"]
AEROSOL_TYPES = (DUST_AEROSOL, SEASALT_AEROSOL, SULFATE_AEROSOL)
AEROSOL_REFF = {DUST_AEROSOL: (0.5, 5.0), SEASALT_AEROSOL: (0.3, 3.0), SULFATE_AEROSOL: (0.05, 0.5)}


def generate_aerosolcoeff(seed: int = 9, scheme: str = "CRTM") -> co.AerosolCoeff:
    """Synthetic AerosolCoeff table for one scheme, 20 wavelengths
    (frequencies increasing) x the reference's 8 types, 38 Legendre terms, smooth Mie-like
    optics (extinction efficiency 2x^2/(1+x^2) of the size parameter x):

    - 'CRTM': 10 RH x 40 radii x 1 sigma; the scheme reads the first RH;
    - 'CMAQ': 1 RH x 40 radii x 6 log-normal widths sigma; broader size
      distributions act as larger particles;
    - 'GOCART-GEOS5' / 'NAAPS': 8 RH x 1 radius x 1 sigma; hygroscopic growth
      (kappa per type) swells the dry radius with relative humidity."""
    wl = np.geomspace(25.0, 0.3, 20)                      # microns, decreasing
    nu = 1.0e4 / wl                                        # cm^-1, increasing
    nl = CLOUD_N_LEGENDRE
    #                    dust  SSAM SSCM1 SSCM2 SSCM3  OC    BC   sulfate
    DENS = np.array([2.6, 2.2, 2.2, 2.2, 2.2, 1.8, 1.0, 1.7])            # g/cm^3
    W0 = np.array([0.75, 0.98, 0.98, 0.98, 0.98, 0.9, 0.3, 0.95])
    RDRY = np.array([1.5, 1.0, 0.5, 2.0, 4.0, 0.1, 0.05, 0.15])          # dry radius (RH schemes)
    KAPPA = np.array([0.05, 1.0, 1.0, 1.0, 1.0, 0.2, 0.0, 0.6])

    def tables(sel, rng):
        """The scheme's axes and (w, rh, r, sigma, type) tables of the types
        at positions sel of the parameter arrays."""
        nt, dens, w0 = len(sel), DENS[sel], W0[sel]

        def optics(r_eff, r_mass):
            """r_eff (..., type) optical radius, r_mass the radius of the dry
            mass: ke [m^2/kg], w, g with the wavelength axis first."""
            x = 2.0 * np.pi * r_eff[None] * nu.reshape((-1,) + (1,) * r_eff.ndim) / 1.0e4
            q = 2.0 * x ** 2 / (1.0 + x ** 2)
            ke = 0.75 * q * (r_eff / r_mass)[None] ** 2 / (dens * 1.0e3 * r_mass[None] * 1.0e-6)
            w = np.clip(w0 * x / (1.0 + x) + 0.02, 0.01, 0.995)
            g = 0.7 * x / (1.0 + x)
            return ke * (1.0 + 0.02 * rng.standard_normal(ke.shape)), w, g

        if scheme in ("CRTM", "CMAQ"):
            nrh, nr = (10, 40) if scheme == "CRTM" else (1, 40)
            reff = np.stack([np.geomspace(0.01, 20.0, nr)] * nt, axis=1)            # (r, type)
            rh = np.linspace(0.0, 0.99, nrh) if scheme == "CRTM" else np.zeros(1)
            if scheme == "CRTM":
                rsig = np.ones((1, nt))
                ke, w, g = optics(reff, reff)                                        # (w, r, type)
                ke5, w5, g5 = (np.repeat(a[:, None, :, None, :], nrh, axis=1) for a in (ke, w, g))
            else:
                ns = 6
                rsig = np.stack([np.linspace(1.1, 2.6, ns)] * nt, axis=1)            # (sigma, type)
                broad = np.exp(0.5 * np.log(rsig) ** 2)                              # (sigma, type)
                r_opt = reff[:, None, :] * broad[None, :, :]                         # (r, sigma, type)
                ke, w, g = optics(r_opt, np.broadcast_to(reff[:, None, :], r_opt.shape))
                ke5, w5, g5 = (a[:, None] for a in (ke, w, g))                       # (w, 1, r, sigma, type)
        else:
            rh = np.array([0.0, 0.5, 0.7, 0.8, 0.9, 0.95, 0.98, 0.99])
            rdry, kappa = RDRY[sel], KAPPA[sel]
            gf = (1.0 + kappa[None, :] * rh[:, None] / (1.0 - rh[:, None])) ** (1.0 / 3.0)   # (rh, type)
            r_wet = rdry[None, :] * gf
            ke, w, g = optics(r_wet, np.broadcast_to(rdry[None, :], r_wet.shape))           # (w, rh, type)
            reff = rdry[None, :].copy()
            rsig = np.ones((1, nt))
            ke5, w5, g5 = (a[:, :, None, None, :] for a in (ke, w, g))                      # (w, rh, 1, 1, type)
        return reff, rsig, rh, ke5, w5, g5

    # dust, sea salt (SSAM) and sulfate from the seed's own stream, the other
    # five types from a second one, so the workloads' three types keep their
    # tables whatever else the file holds
    first = [0, 1, 7]
    rest = [2, 3, 4, 5, 6]
    a = tables(first, np.random.Generator(np.random.PCG64(seed)))
    b = tables(rest, np.random.Generator(np.random.PCG64(seed + 1000)))
    out = []
    for x, y in zip(a[:2], b[:2]):          # reff, rsig: type last
        z = np.empty(x.shape[:-1] + (8,))
        z[..., first], z[..., rest] = x, y
        out.append(z)
    rh = a[2]
    for x, y in zip(a[3:], b[3:]):
        z = np.empty(x.shape[:-1] + (8,))
        z[..., first], z[..., rest] = x, y
        out.append(z)
    reff, rsig, ke5, w5, g5 = out
    pc = 0.5 * g5[..., None] ** np.arange(nl + 1)
    return co.AerosolCoeff(np.array(AEROSOL_TABLE_TYPES, np.int32), AEROSOL_TABLE_NAMES, wl, reff,
                           rsig, rh, np.ascontiguousarray(ke5), np.ascontiguousarray(w5),
                           np.ascontiguousarray(g5), pc[..., None])


def aerosol_file_name(scheme: str = "CRTM") -> str:
    """``AerosolCoeff.bin`` (the reference's default name) for 'CRTM', else
    ``AerosolCoeff.<scheme>.bin``."""
    return "AerosolCoeff.bin" if scheme == "CRTM" else f"AerosolCoeff.{scheme}.bin"


def write_aerosol_files(coeff_dir: str, scheme: str = "CRTM") -> str:
    """Write the scheme's synthetic AerosolCoeff file if missing."""
    os.makedirs(coeff_dir, exist_ok=True)
    path = os.path.join(coeff_dir, aerosol_file_name(scheme))
    if not os.path.exists(path):
        co.write_aerosolcoeff(path + ".tmp", generate_aerosolcoeff(scheme=scheme), scheme=scheme)
        os.replace(path + ".tmp", path)
    return path


def add_aerosol_scheme_inputs(atm: AtmosphereBatch, seed: int) -> AtmosphereBatch:
    """Effective_Variance (the 'CMAQ' table's sigma, uniform in [1.2, 2.4] per
    aerosol and profile) and Relative_Humidity (0.3-0.95 at the surface,
    falling with height) for the aerosol schemes that read them."""
    rng = np.random.Generator(np.random.PCG64(seed))
    P, K = atm.n_profiles, atm.max_layers
    NA = atm.aerosol_type.shape[1]
    atm.aerosol_effective_variance = np.repeat(rng.uniform(1.2, 2.4, (P, NA))[:, :, None], K, axis=2)
    z = height_km(np.maximum(atm.pressure, 1e-3))
    atm.relative_humidity = np.clip(rng.uniform(0.3, 0.95, (P, 1)) * np.exp(-z / 8.0), 0.0, 0.99)
    return atm


def add_aerosols(atm: AtmosphereBatch, aerosol_types: Sequence[int], seed: int,
                 load_scale: float = 1.0) -> AtmosphereBatch:
    """Aerosols of ``aerosol_types`` in every profile: lognormal column loading
    in 0.01-1 g/m^2 (x ``load_scale``), exponential vertical profile with a
    1-3 km scale height, effective radius uniform in the type's range
    (concentration stored in kg/m^2 per layer)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    P, K = atm.n_profiles, atm.max_layers
    NA = len(aerosol_types)
    conc = np.zeros((P, NA, K))
    reff = np.zeros((P, NA, K))
    for m in range(P):
        n = int(atm.n_layers[m])
        z = height_km(np.maximum(atm.pressure[m, :n], 1e-3))
        dz = np.abs(np.gradient(z))
        for a, t in enumerate(aerosol_types):
            col = np.exp(rng.uniform(np.log(0.01), np.log(1.0))) * 1.0e-3 * load_scale   # kg/m^2
            prof = np.exp(-z / rng.uniform(1.0, 3.0)) * dz
            conc[m, a, :n] = col * prof / prof.sum()
            lo, hi = AEROSOL_REFF[t]
            reff[m, a, :n] = rng.uniform(lo, hi)
    atm.n_aerosols = np.full(P, NA, np.int32)
    atm.aerosol_type = np.tile(np.asarray(aerosol_types, np.int32), (P, 1))
    atm.aerosol_concentration = conc
    atm.aerosol_effective_radius = reff
    return atm


IRWATER_FILE = "Nalli.IRwater.EmisCoeff.bin"   # the reference's default IRwaterCoeff_File


def generate_irwatercoeff(classification: str = "Nalli") -> co.IRwaterCoeff:
    """Synthetic IR sea-surface emissivity table: 18 angles (0-85 deg) x 61
    frequencies (600-3000 cm^-1) x 16 wind speeds (0-15 m/s) x 1 temperature
    (5, 270-310 K, for 'Nalli2').  Emissivity 1 - R with a Schlick-type
    Fresnel reflectance R(theta) = R0 + (1 - R0)(1 - cos theta)^5 of a
    frequency-dependent refractive index, reduced at slant angles by wind
    roughness, and a weak temperature dependence."""
    ang = np.arange(0.0, 86.0, 5.0)
    nu = np.arange(600.0, 3001.0, 40.0)
    wind = np.arange(0.0, 16.0, 1.0)
    temp = np.array([270.0, 280.0, 290.0, 300.0, 310.0]) if classification == "Nalli2" else np.array([290.0])
    n = 1.28 + 0.05 * np.sin(nu / 300.0)
    r0 = ((n - 1.0) / (n + 1.0)) ** 2
    c = np.cos(np.deg2rad(ang))
    R = r0[None, :] + (1.0 - r0[None, :]) * (1.0 - c[:, None]) ** 5            # (angle, frequency)
    s2 = (1.0 - c ** 2)[:, None, None]
    Rv = R[:, :, None] * (1.0 - 0.02 * wind[None, None, :] * s2)              # (angle, frequency, wind)
    e = 1.0 - Rv
    e4 = e[..., None] * (1.0 + 1.0e-4 * (temp[None, None, None, :] - 290.0))
    return co.IRwaterCoeff(classification, ang, nu, wind, temp, np.clip(e4, 0.0, 1.0))


def write_irwater_file(coeff_dir: str, classification: str = "Nalli", name: str = IRWATER_FILE) -> str:
    """Write the synthetic IR water emissivity table if missing."""
    os.makedirs(coeff_dir, exist_ok=True)
    path = os.path.join(coeff_dir, name)
    if not os.path.exists(path):
        co.write_irwatercoeff(path + ".tmp", generate_irwatercoeff(classification))
        os.replace(path + ".tmp", path)
    return path
