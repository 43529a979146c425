"""Generates the golden fixtures in this folder from the reference's source text.

Run with the environment variable REFERENCE naming a checkout of the
reference; the outputs are committed so the tests never need the reference
at run time.

  velocity_sets.json  -- the (c, w) tables of
                         BoltzmannFluids/Source/LBMConstants/VelocitySet.cpp,
                         parsed from the get_velosity_vectors() switch cases,
                         weights evaluated from their literal fractions.
  lbm_defaults.json   -- default knob values read from
                         BoltzmannFluids/Source/LBM/LBM.h and the thermal
                         relaxation time that LBM.cpp's initialize_fields sets.
"""
import json
import os
import re
import sys
from fractions import Fraction

REFERENCE = os.environ.get("REFERENCE")
HERE = os.path.dirname(os.path.abspath(__file__))


def parse_velocity_sets(text):
    sets = {}
    # every "case NAME:" followed by "return{ glm::vec4(...), ... };"
    for m in re.finditer(r"case\s+(D\dQ\d+)\s*:\s*return\s*\{(.*?)\};", text, re.S):
        name, body = m.group(1), m.group(2)
        rows = []
        for v in re.finditer(r"glm::vec4\(\s*([-\d]+)\s*,\s*([-\d]+)\s*,\s*([-\d]+)\s*,\s*([\d.]+)\s*/\s*(\d+)\s*\)", body):
            cx, cy, cz = int(v.group(1)), int(v.group(2)), int(v.group(3))
            num = Fraction(v.group(4)).limit_denominator(1000)
            w = num / int(v.group(5))
            rows.append({"c": [cx, cy, cz], "w_num": w.numerator, "w_den": w.denominator,
                         "w_float": float(w)})
        sets[name] = rows
    return sets


def parse_defaults(h_text, cpp_text):
    def num(pattern, text):
        m = re.search(pattern, text)
        return float(m.group(1).rstrip("f")) if m else None

    return {
        "velocity_limit": num(r"float velocity_limit\s*=\s*([\d.]+f?)", h_text),
        "velocity_limit_extreme": num(r"float velocity_limit_extreme\s*=\s*([\d.]+f?)", h_text),
        "relaxation_time": num(r"float relaxation_time\s*=\s*([\d.]+f?)", h_text),
        "thermal_expension_coeficient": num(r"float thermal_expension_coeficient\s*=\s*([\d.]+f?)", h_text),
        "intermolecular_interaction_strength": num(r"float intermolecular_interaction_strength\s*=\s*(-?[\d.]+f?)",
                                                   h_text),
        "max_boundry_count": num(r"max_boundry_count\s*=\s*(\d+)", h_text),
        "initialize_fields_thermal_relaxation_time": num(r"thermal_relaxation_time\s*=\s*([\d.]+f?)\s*;", cpp_text),
    }


def main():
    if not REFERENCE:
        sys.exit("set REFERENCE to a checkout of the reference")
    src = os.path.join(REFERENCE, "BoltzmannFluids", "Source")
    vs_text = open(os.path.join(src, "LBMConstants", "VelocitySet.cpp")).read()
    sets = parse_velocity_sets(vs_text)
    want = {"D2Q9": 9, "D3Q15": 15, "D3Q19": 19, "D3Q27": 27, "D2Q5": 5, "D3Q7": 7}
    for k, n in want.items():
        if len(sets.get(k, [])) != n:
            sys.exit(f"parse failure for {k}: {len(sets.get(k, []))} rows")
    with open(os.path.join(HERE, "velocity_sets.json"), "w") as f:
        json.dump({"source": "BoltzmannFluids/Source/LBMConstants/VelocitySet.cpp", "sets": sets}, f, indent=1)
    h_text = open(os.path.join(src, "LBM", "LBM.h")).read()
    cpp_text = open(os.path.join(src, "LBM", "LBM.cpp")).read()
    d = parse_defaults(h_text, cpp_text)
    with open(os.path.join(HERE, "lbm_defaults.json"), "w") as f:
        json.dump({"source": "BoltzmannFluids/Source/LBM/LBM.h, LBM.cpp", "defaults": d}, f, indent=1)
    print("wrote", sorted(sets), d)


if __name__ == "__main__":
    main()
