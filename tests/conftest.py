import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def coeff_dir(tmp_path_factory):
    from crtmv3_gb300 import synthetic as sy
    d = str(tmp_path_factory.mktemp("coeffs"))
    for s in sy.SENSORS:
        sy.write_sensor_files(d, s)
    return d


@pytest.fixture(scope="session")
def gpu_lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crtmv3_gb300 import build
    build.build()
    from crtmv3_gb300 import api
    api.library()
    return api


def reference_profiles(sensor_id, clouds=False, aerosols=False, seed=5):
    """The reference's two unit-test profiles (tests/golden/reference_profiles.json,
    from Load_Atm_Data.inc / Load_Sfc_Data.inc and test_AD.f90's geometry) as
    batches for a synthetic sensor: 92 layers, H2O (mass mixing ratio) and O3
    (volume mixing ratio), tops at 0.714 hPa (so AddLayers extends them), each
    profile's Climatology; with ``clouds`` the file's one snow cloud per
    profile (layers k1..k2, 5 kg/m^2, 20 and 1000 microns, Cloud_Fraction 1
    and 0.5), with ``aerosols`` its three aerosols per profile.  The surface
    is the file's four-cover surface; the emissivity is the sensor type's
    seeded synthetic one (the path takes the emissivity as an input)."""
    import json

    import numpy as np

    from crtmv3_gb300 import structures as st, synthetic as sy
    with open(os.path.join(ROOT, "tests", "golden", "reference_profiles.json")) as f:
        doc = json.load(f)
    prof, sfcs, g = doc["atmosphere"], doc["surface"], doc["geometry"]
    P, K = len(prof), len(prof[0]["pressure"])
    atm = st.AtmosphereBatch(
        n_layers=np.full(P, K, np.int32),
        level_pressure=np.array([p["level_pressure"] for p in prof]),
        pressure=np.array([p["pressure"] for p in prof]),
        temperature=np.array([p["temperature"] for p in prof]),
        absorber=np.array([p["absorber"] for p in prof]),
        absorber_id=np.array(prof[0]["absorber_id"], np.int32),
        absorber_units=np.array([3, 1], np.int32),
        climatology=np.array([p["climatology"] for p in prof], np.int32))
    if clouds:
        atm.n_clouds = np.ones(P, np.int32)
        atm.cloud_type = np.array([[p["cloud"]["type"]] for p in prof], np.int32)
        atm.cloud_water_content = np.zeros((P, 1, K))
        atm.cloud_effective_radius = np.zeros((P, 1, K))
        atm.cloud_fraction = np.zeros((P, K))
        for i, p in enumerate(prof):
            c = p["cloud"]
            sl = slice(c["k1"] - 1, c["k2"])
            atm.cloud_water_content[i, 0, sl] = c["water_content"]
            atm.cloud_effective_radius[i, 0, sl] = c["effective_radius"]
            # Atmosphere%Cloud_Fraction is set whole-profile by the file
            atm.cloud_fraction[i, :] = c["cloud_fraction"]
    if aerosols:
        NA = max(len(p["aerosols"]) for p in prof)
        atm.n_aerosols = np.array([len(p["aerosols"]) for p in prof], np.int32)
        atm.aerosol_type = np.zeros((P, NA), np.int32)
        atm.aerosol_concentration = np.zeros((P, NA, K))
        atm.aerosol_effective_radius = np.zeros((P, NA, K))
        for i, p in enumerate(prof):
            for j, a in enumerate(p["aerosols"]):
                atm.aerosol_type[i, j] = a["type"]
                atm.aerosol_concentration[i, j] = a["concentration"]
                atm.aerosol_effective_radius[i, j] = a["effective_radius"]

    def col(key, default):
        return np.array([s[key] if s[key] is not None else default for s in sfcs], np.float64)
    sfc = st.SurfaceBatch(col("land_coverage", 0.0), col("water_coverage", 0.0), col("snow_coverage", 0.0),
                          col("ice_coverage", 0.0), col("land_temperature", 280.0),
                          col("water_temperature", 280.0), col("snow_temperature", 260.0),
                          col("ice_temperature", 260.0))
    geo = st.GeometryBatch(np.full(P, g["sensor_zenith_angle"]), np.full(P, g["sensor_scan_angle"]),
                           np.zeros(P), np.full(P, 100.0), np.zeros(P), np.zeros(P))
    _, L, stype, _ = sy.SENSORS[sensor_id]
    opt = st.OptionsBatch(emissivity=sy.emissivity_for(stype, P, L, seed))
    return atm, sfc, geo, opt
