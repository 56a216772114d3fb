"""Extract the reference's multigroup decks into JSON fixtures.

The reference verifies its multigroup path with analytic benchmark decks whose
expected multiplication factor is written in the deck header
(input_files/PUa-1-0-IN.yaml:2, PUb-1-0-IN.yaml:2, PUa-1-0-SL.yaml:2,
PUb-1-0-SL.yaml:2), plus decks used as regression inputs: Ua-1-1-IN.yaml
(an infinite medium with P1 scattering),
Ua-1-1-CY.yaml (P1 scattering), UD2O-2-1-SL.yaml (two groups), PUa-1-1-SL.yaml
and PUa-1-2-SL.yaml (P1 and P2 scattering in a slab), and c5g7.yaml, the
seven-group C5G7 benchmark core (nested rectangular lattices of 17x17 pin
cells in 2x2 assemblies with seven materials).

Usage: python make_reference_decks.py REFERENCE_ROOT
(or with the ABEILLE_REFERENCE environment variable set to the reference's
source tree).  The decks are parsed with the package's own deck reader
(abeille_gb300.deck.parse_yaml) and written to reference_decks.json next to
this script; the tests read only the JSON.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from abeille_gb300 import deck as deck_io  # noqa: E402

DECKS = ["PUa-1-0-IN", "PUb-1-0-IN", "PUa-1-0-SL", "PUb-1-0-SL", "Ua-1-1-CY", "UD2O-2-1-SL",
         "PUa-1-1-SL", "PUa-1-2-SL", "Ua-1-1-IN", "c5g7"]


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ABEILLE_REFERENCE")
    if not ref:
        sys.exit("usage: make_reference_decks.py REFERENCE_ROOT (or set ABEILLE_REFERENCE)")
    out = {}
    for name in DECKS:
        path = os.path.join(ref, "input_files", name + ".yaml")
        with open(path) as f:
            text = f.read()
        header = " | ".join(text.splitlines()[:2])
        m = re.search(r"k(?:_inf)?\s*=\s*([0-9.]+)", header)
        d = deck_io.parse_yaml(text)
        d["_expected_k"] = float(m.group(1)) if m else None
        d["_source"] = f"input_files/{name}.yaml"
        out[name] = d
    with open(os.path.join(HERE, "reference_decks.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(HERE, "reference_decks.json"))


if __name__ == "__main__":
    main()
