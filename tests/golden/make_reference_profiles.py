"""Writes ``reference_profiles.json``: the reference's own unit-test profiles
(two 92-layer atmospheres with their clouds and aerosols, and their
surfaces), read from the reference tree's Fortran include files

    test/mains/unit/Unit_Test/Load_Atm_Data.inc
    test/mains/unit/Unit_Test/Load_Sfc_Data.inc

and the test programs' geometry (``test_AD.f90``: Sensor_Zenith_Angle 30,
Sensor_Scan_Angle 26.37293341421) and sizes (92 layers, 2 absorbers).  The
named constants the files use (climatology models, cloud and aerosol types)
are resolved from the reference's own definitions
(``src/Atmosphere/CRTM_Atmosphere_Define.f90``,
``src/Atmosphere/Cloud/CRTM_Cloud_Define.f90``, ``src/CRTM_Parameters.f90``).

Run once where the reference tree is present:

    python tests/golden/make_reference_profiles.py [reference root]

The JSON is committed; the tests read only the JSON.
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
UNIT = os.path.join("test", "mains", "unit", "Unit_Test")


def _strip_comments(text):
    return "\n".join(line.split("!")[0] for line in text.splitlines())


def _number(tok):
    return float(tok.strip().replace("_fp", "").replace("D", "E").replace("d", "e"))


def _constants(root):
    """Integer PARAMETERs of the files that define the names used."""
    out = {}
    for rel in (("src", "Atmosphere", "CRTM_Atmosphere_Define.f90"),
                ("src", "Atmosphere", "Cloud", "CRTM_Cloud_Define.f90"),
                ("src", "CRTM_Parameters.f90")):
        with open(os.path.join(root, *rel)) as f:
            for m in re.finditer(r"INTEGER\s*,.*?PARAMETER\s*::\s*(\w+)\s*=\s*(-?\d+)\s*$",
                                 _strip_comments(f.read()), re.M | re.I):
                out.setdefault(m.group(1).upper(), int(m.group(2)))
    return out


def _arrays(text):
    """Every ``lhs = (/ ... /)`` assignment: {lhs: [values]}."""
    out = {}
    for m in re.finditer(r"(\w+\(\d\)%[\w%():,]+?)\s*=\s*&?\s*\(/(.*?)/\)", text, re.S):
        vals = [v for v in m.group(2).replace("&", " ").split(",") if v.strip()]
        try:
            out[m.group(1)] = [_number(v) for v in vals]
        except ValueError:
            out[m.group(1)] = [v.strip() for v in vals]
    return out


def _scalars(text):
    """``lhs = value`` assignments (not arrays): {lhs: token}."""
    out = {}
    for m in re.finditer(r"^\s*(\w+\(\d\)%[\w%():,]+|\w+)\s*=\s*([^(&\n][^\n]*)$", text, re.M):
        out.setdefault(m.group(1).strip(), m.group(2).strip())
    return out


def atmosphere(root, const):
    with open(os.path.join(root, UNIT, "Load_Atm_Data.inc")) as f:
        text = _strip_comments(f.read())
    parts = re.split(r"\n\s*atm\(2\)%Climatology", text, maxsplit=1)
    parts[1] = "atm(2)%Climatology" + parts[1]
    profiles = []
    for p, part in enumerate(parts, start=1):
        arr, sca = _arrays(part), _scalars(part)
        a = f"atm({p})%"
        prof = {
            "climatology": const[sca[a + "Climatology"].upper()],
            "absorber_id": [const.get(t.upper(), t) for t in arr[a + "Absorber_Id(1:2)"]],
            "level_pressure": arr[a + "Level_Pressure"],
            "pressure": arr[a + "Pressure"],
            "temperature": arr[a + "Temperature"],
            "absorber": [arr[a + "Absorber(:,1)"], arr[a + "Absorber(:,2)"]],
        }
        co2 = arr.get(a + "Absorber(:,3)")
        prof["co2"] = co2 if co2 is not None else [_number(sca[a + "Absorber(:,3)"])] * len(prof["pressure"])
        # one cloud: the loop body sets every cloud alike (k1:k2, 1-based)
        k1, k2 = int(sca["k1"]), int(sca["k2"])
        prof["cloud"] = {
            "type": const[sca[a + "Cloud(nc)%Type"].upper()],
            "k1": k1, "k2": k2,
            "effective_radius": _number(sca[a + "Cloud(nc)%Effective_Radius(k1:k2)"]),
            "water_content": _number(sca[a + "Cloud(nc)%Water_Content(k1:k2)"]),
            "cloud_fraction": _number(sca[a + "Cloud_Fraction"]),
        }
        aer = []
        for i in (1, 2, 3):
            t = sca.get(f"{a}Aerosol({i})%Type")
            if t is None:
                continue
            aer.append({"type": const[t.upper()],
                        "effective_radius": arr[f"{a}Aerosol({i})%Effective_Radius"],
                        "concentration": arr[f"{a}Aerosol({i})%Concentration"]})
        prof["aerosols"] = aer
        n = len(prof["pressure"])
        assert len(prof["level_pressure"]) == n + 1 and len(prof["temperature"]) == n
        assert all(len(x) == n for x in prof["absorber"]) and len(prof["co2"]) == n
        assert all(len(x["effective_radius"]) == n and len(x["concentration"]) == n for x in aer)
        profiles.append(prof)
    return profiles


def surface(root):
    with open(os.path.join(root, UNIT, "Load_Sfc_Data.inc")) as f:
        text = _strip_comments(f.read())
    sca = _scalars(text)
    out = []
    for p in (1, 2):
        s = {}
        for kind in ("Land", "Water", "Snow", "Ice"):
            c = sca.get(f"sfc({p})%{kind}_Coverage")
            t = sca.get(f"sfc({p})%{kind}_Temperature")
            s[kind.lower() + "_coverage"] = _number(c) if c else 0.0
            s[kind.lower() + "_temperature"] = _number(t) if t else None
        out.append(s)
    return out


def geometry(root):
    with open(os.path.join(root, UNIT, "test_AD.f90")) as f:
        text = _strip_comments(f.read())
    z = re.search(r"ZENITH_ANGLE\s*=\s*([\d.Ee+-]+_fp)", text).group(1)
    s = re.search(r"SCAN_ANGLE\s*=\s*([\d.Ee+-]+_fp)", text).group(1)
    return {"sensor_zenith_angle": _number(z), "sensor_scan_angle": _number(s)}


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    const = _constants(root)
    doc = {
        "source": [os.path.join(UNIT, "Load_Atm_Data.inc"), os.path.join(UNIT, "Load_Sfc_Data.inc"),
                   os.path.join(UNIT, "test_AD.f90")],
        "atmosphere": atmosphere(root, const),
        "surface": surface(root),
        "geometry": geometry(root),
    }
    path = os.path.join(HERE, "reference_profiles.json")
    with open(path, "w") as f:
        json.dump(doc, f, indent=None, separators=(",", ":"))
        f.write("\n")
    a = doc["atmosphere"]
    print(path, [len(p["pressure"]) for p in a], [np.round(p["level_pressure"][0], 3) for p in a],
          [[x["type"] for x in p["aerosols"]] for p in a], doc["surface"], doc["geometry"])


if __name__ == "__main__":
    main()
