"""Writes model_profiles.json: the six climatological model profiles that
CRTM_Atmosphere_AddLayers places above a profile whose top level is below
0.005 hPa, on the 101 AIRS pressure levels.

The numbers are read from the reference's DATA statements in
src/Atmosphere/CRTM_Model_Profiles.f90 (MODEL_LEVEL_PRESSURE :80-100,
Level_Temperature :107-239, Level_Absorber :241-1038).  The added layers are
defined by this table, so it must be the same table.  The script runs in a
checkout that has the reference tree; the JSON it writes is what the library
reads.

    python crtmv3_gb300/data/extract_model_profiles.py <reference root>
"""
import json
import os
import re
import sys

MODELS = ["TROPICAL", "MIDLATITUDE_SUMMER", "MIDLATITUDE_WINTER", "SUBARCTIC_SUMMER",
          "SUBARCTIC_WINTER", "US_STANDARD_ATMOSPHERE"]
# index order of the absorber axis in the reference's table (CRTM_Model_Profiles.f90:56-61)
ABSORBERS = ["H2O", "O3", "CO2", "N2O", "CO", "CH4"]
NUM = re.compile(r"[-+]?\d+\.\d*(?:[eEdD][-+]?\d+)?(?=_fp)")


def numbers(text: str) -> list:
    return [float(v.replace("d", "e").replace("D", "e")) for v in NUM.findall(text)]


def main(root: str) -> None:
    src = open(os.path.join(root, "src", "Atmosphere", "CRTM_Model_Profiles.f90")).read()
    src = "\n".join(line.split("!")[0] for line in src.split("\n"))
    m = re.search(r"MODEL_LEVEL_PRESSURE\(0:N_MODEL_LAYERS\)\s*=\s*&?\s*\(/(.*?)/\)", src, re.S)
    pressure = numbers(m.group(1))
    temperature = {}
    absorber = {}
    for m in re.finditer(r"DATA\s+Level_Temperature\(:,(\w+)\)\s*/(.*?)/", src, re.S):
        temperature[m.group(1)] = numbers(m.group(2))
    for m in re.finditer(r"DATA\s+Level_Absorber\(:,(\w+),(\w+)\)\s*/(.*?)/", src, re.S):
        absorber.setdefault(m.group(2), {})[m.group(1)] = numbers(m.group(3))
    assert len(pressure) == 101, len(pressure)
    out = {"source": "CRTM_Model_Profiles.f90 (JCSDA/CRTMv3 src/Atmosphere)",
           "models": MODELS, "absorbers": ABSORBERS,
           "absorber_units": "H2O g/kg, others ppmv",
           "level_pressure_hpa": pressure,
           "level_temperature_k": [temperature[name] for name in MODELS],
           "level_absorber": [[absorber[name][a] for a in ABSORBERS] for name in MODELS]}
    for t in out["level_temperature_k"]:
        assert len(t) == 101
    for per_model in out["level_absorber"]:
        for a in per_model:
            assert len(a) == 101
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "model_profiles.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
