"""Writes tests/golden/reference_pins.json from two output files the reference repository
ships (read as text where the reference is checked out; the JSON is what the tests use):

* software/trunk/bin/reference_values.txt, written by write_reference_values_to_file
  (trunk/src/solver/scaling.f90:203-237) for argon at n = 1e20 m^-3, T = 273 K, Kn = 1.091;
* software/shock_calculator/normal_shock_parameters.txt, written by the reference's
  shock calculator (software/shock_calculator/normal_shock.f90) for a 3 % Xe / 97 % He
  mixture, stationary shock at Mach 3.9.

    python tests/golden/make_reference_pins.py [reference checkout]
"""
import json
import os
import re
import sys

ROOT = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
HERE = os.path.dirname(os.path.abspath(__file__))


def _values(path, pattern=r"^\s*([^=]+?)\s*=\s*([-+0-9.Ee]+)"):
    out = {}
    for line in open(path):
        m = re.match(pattern, line)
        if m:
            out[m.group(1).strip()] = float(m.group(2))
    return out


def main():
    ref = _values(os.path.join(ROOT, "software", "trunk", "bin", "reference_values.txt"))
    shock_txt = os.path.join(ROOT, "software", "shock_calculator", "normal_shock_parameters.txt")
    shock = _values(shock_txt)
    he = re.search(r"He: *([0-9.]+)\s+mass = *([0-9.]+)", open(shock_txt).read())
    shock["He fraction"], shock["He mass ratio"] = float(he.group(1)), float(he.group(2))
    xe = re.search(r"Xe: *([0-9.]+)", open(shock_txt).read())
    shock["Xe fraction"] = float(xe.group(1))
    shock["Mach"] = float(re.search(r"Mach number \(shock reference frame\) = *([0-9.]+)",
                                    open(shock_txt).read()).group(1))
    with open(os.path.join(HERE, "reference_pins.json"), "w") as fh:
        json.dump({"reference_values": ref, "normal_shock": shock}, fh, indent=1, sort_keys=True)
        fh.write("\n")


if __name__ == "__main__":
    main()
