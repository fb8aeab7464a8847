"""The GPU library's __host__ __device__ physics headers, compiled for the CPU.

Checks, without a GPU: the per-profile prep (layer averaging, mapped
profile, predictors) against the oracle, the hand-derived predictor partial
derivatives against finite differences, and the column-by-column layer
averaging against the sequential form.
"""
import ctypes as ct
import os
import shutil
import subprocess

import numpy as np
import pytest

from crtmv3_gb300 import coefficients as co, synthetic as sy

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
MAX_BAND = 32


@pytest.fixture(scope="module")
def hx(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    out = str(tmp_path_factory.mktemp("hx") / "libhx.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I",
                    os.path.join(ROOT, "crtmv3_gb300", "csrc"), "-o", out,
                    os.path.join(HERE, "harness", "physics_harness.cpp")], check=True)
    return ct.CDLL(out)


def _ptr(a):
    return a.ctypes.data_as(ct.c_void_p)


def _extended(atm, cut):
    """The batch without its top `cut` layers, extended again by AddLayers."""
    import dataclasses
    from crtmv3_gb300 import addlayers as al
    m = atm.n_layers - cut
    cutb = dataclasses.replace(
        atm, n_layers=m.astype(np.int32), level_pressure=np.ascontiguousarray(atm.level_pressure[:, cut:]),
        pressure=np.ascontiguousarray(atm.pressure[:, cut:]), temperature=np.ascontiguousarray(atm.temperature[:, cut:]),
        absorber=np.ascontiguousarray(atm.absorber[:, :, cut:]))
    ext, info = al.add_layers(cutb)
    assert info.any
    return ext


@pytest.mark.parametrize("sensor,nl,cut", [("mwsynth_c22", 100, 0), ("irsynth_c616", 101, 0), ("mwsynth_c16", 77, 0),
                                           # profile tops below 0.005 hPa, extended by AddLayers
                                           ("irsynth_c616", 101, 9), ("mwsynth_c22", 100, 25)])
def test_prep_matches_oracle(hx, coeff_dir, sensor, nl, cut):
    from oracle import pyoracle as po
    o = po.Oracle(coeff_dir, sensor)
    tc = co.read_odps(f"{coeff_dir}/{sensor}.TauCoeff.bin")
    G, K, Jm, J = tc.group_index, tc.n_layers, tc.n_absorbers, tc.n_components
    NS = {1: 89, 2: 50, 3: 21}[G]
    nnz = hx.hx_nnz(G)
    atm, sfc, geo, opt = sy.clear_sky_workload(sensor, 2, nl, 40)
    if cut:
        atm = _extended(atm, cut)
    b, keep = o._batch(atm, sfc, geo, opt)
    L = po.lib()
    L.or_profile_state.argtypes = [ct.c_void_p, ct.POINTER(po.OrBatch), ct.c_int] + [po._dp] * 4
    tabs = [np.ascontiguousarray(x, np.float64) for x in
            (tc.ref_level_pressure, tc.ref_pressure, tc.ref_temperature, tc.ref_absorber.T,
             tc.min_absorber.T, tc.max_absorber.T)]
    h2o = Jm - 1 if tc.absorber_id[-1] == 1 else 0
    ids = list(atm.absorber_id)
    idx = np.array([ids.index(a) if a in ids else -1 for a in tc.absorber_id], np.int32)
    for m in range(2):
        T, A, sec, X = np.zeros(K), np.zeros(Jm * K), np.zeros(K), np.zeros(K * J * 18)
        L.or_profile_state(o.h, ct.byref(b), m, po._p(T), po._p(A), po._p(sec), po._p(X))
        X = X.reshape(K, J, 18)
        Ku = int(atm.n_layers[m])
        out = [np.zeros(K * NS), np.zeros(K * nnz), np.zeros(K), np.zeros(Jm * K),
               np.zeros(Jm * K, np.uint8), np.zeros(K, np.int32), np.zeros(K, np.int32),
               np.zeros(K * MAX_BAND), np.zeros(Ku + 1, np.int32), np.zeros(Ku + 1, np.int32),
               np.zeros(Ku + 1), np.zeros(Ku, np.int32), np.zeros(Ku, np.int32), np.zeros(4)]
        prof = [np.ascontiguousarray(x) for x in (atm.level_pressure[m], atm.pressure[m],
                                                  atm.temperature[m], atm.absorber[m])]
        args = [ct.c_int(G), ct.c_int(K)] + [_ptr(x) for x in tabs]
        args += [ct.c_int(h2o), ct.c_int(Ku), _ptr(prof[0]), _ptr(prof[1]), _ptr(prof[2]),
                 ct.c_int(atm.n_absorbers), _ptr(prof[3]), ct.c_int(atm.max_layers), _ptr(idx),
                 ct.c_double(geo.sensor_zenith_angle[m])]
        args += [_ptr(x) for x in out]
        assert hx.hx_prep(*args) == 0
        Xo = np.concatenate([X[:, j, :co.N_PREDICTORS_G[G][j]] for j in range(J)], axis=1)
        assert np.array_equal(out[2], T)
        assert np.array_equal(out[3], A)
        assert np.array_equal(out[0].reshape(K, NS), Xo)


@pytest.mark.parametrize("G,NS,Jm", [(1, 89, 6), (2, 50, 3), (3, 21, 1)])
def test_partials_match_finite_differences(hx, G, NS, Jm):
    nnz = hx.hx_nnz(G)
    slot, q = np.zeros(nnz, np.int32), np.zeros(nnz, np.int32)
    hx.hx_pattern(G, _ptr(slot), _ptr(q))
    NV = 3 + 3 * Jm
    rng = np.random.default_rng(G)
    for _ in range(10):
        st = np.zeros(44)
        st[0] = rng.uniform(1, 2.2); st[2] = rng.uniform(200, 280); st[1] = st[2] + rng.normal(0, 8)
        st[3] = rng.uniform(1, 100); st[6] = rng.uniform(100, 5000); st[7] = rng.uniform(100, 5000)
        st[4] = rng.uniform(.9, 1.1); st[5] = rng.uniform(.9, 1.1)
        st[14:20] = rng.uniform(0.1, 10, 6); st[8:14] = st[14:20] * rng.uniform(0.3, 3, 6)
        st[20:26] = rng.uniform(0.5, 2, 6); st[26:32] = rng.uniform(0.5, 2, 6)
        st[32:38] = rng.uniform(10, 1e4, 6); st[38:44] = rng.uniform(10, 1e4, 6)

        def ev(s):
            X, D = np.zeros(NS), np.zeros(nnz)
            hx.hx_layer(G, _ptr(s), _ptr(X), _ptr(D))
            return X, D
        X0, D0 = ev(st)
        Jan = np.zeros((NS, NV))
        for e in range(nnz):
            Jan[slot[e], q[e]] += D0[e]
        for v in range(NV):
            if v == 0: i, mul = 1, 1.0
            elif v <= Jm: i, mul = 8 + v - 1, 1.0
            elif v == 1 + Jm: i, mul = 4, 1 / st[6]
            elif v == 2 + Jm: i, mul = 5, 1 / st[7]
            elif v < 3 + 2 * Jm: a = v - 3 - Jm; i, mul = 20 + a, 1 / st[32 + a]
            else: a = v - 3 - 2 * Jm; i, mul = 26 + a, 1 / st[38 + a]
            h = 1e-6 * abs(st[i])
            s1, s2 = st.copy(), st.copy()
            s1[i] += h
            s2[i] -= h
            fd = (ev(s1)[0] - ev(s2)[0]) / (2 * h) * mul
            err = np.abs(Jan[:, v] - fd) / (np.abs(fd) + 1e-6 * np.abs(X0) + 1e-12)
            assert err.max() < 1e-5, (v, int(err.argmax()))


def test_layer_average_columns_are_independent(hx):
    ref = np.log(sy.layer_mean_pressure(sy.ref_level_pressure(100)))
    rng = np.random.default_rng(1)
    for trial in range(400):
        n = int(rng.integers(20, 200))
        top = np.exp(rng.uniform(np.log(0.001), np.log(0.05)))
        sfc = rng.uniform(500, 1200)
        lev = np.geomspace(top, sfc, n + 1)
        if trial % 2:
            x = np.sort(rng.uniform(np.log(top), np.log(sfc), n - 1))
            lev = np.exp(np.concatenate([[np.log(top)], x, [np.log(sfc)]]))
        lay = np.log(sy.layer_mean_pressure(lev))
        mb = ct.c_int(0)
        assert hx.hx_layer_avg_compare(_ptr(ref), 100, _ptr(lay), n, ct.byref(mb)) == 0
        assert mb.value <= MAX_BAND


def test_exact_float_to_double_conversion(hx):
    """The integer-pipe float->double conversion used for FP64 stores of FP32
    results equals the hardware conversion, including zeros, subnormals,
    infinities and the largest finite values."""
    hx.hx_f32_to_f64.argtypes = [ct.c_float]
    hx.hx_f32_to_f64.restype = ct.c_double
    rng = np.random.default_rng(7)
    bits = np.concatenate([rng.integers(0, 2**32, 200000, dtype=np.uint64).astype(np.uint32),
                           np.arange(0, 70000, dtype=np.uint32),                    # subnormals
                           np.arange(0x7f7f0000, 0x7f800001, 97, dtype=np.uint32),  # large, inf
                           np.array([0x80000000, 0x80000001, 0xff800000], np.uint32)])
    f = bits.view(np.float32)
    f = f[~np.isnan(f)]
    got = np.array([hx.hx_f32_to_f64(float(x)) for x in f])
    assert np.array_equal(got.view(np.uint64), f.astype(np.float64).view(np.uint64))
