"""Extract the golden vectors this repository's tests pin against from the reference checkout.

Reads (paths within KronFreeCircuits.jl):
  test/fixtures/scqubits_reference.json   energies computed by scqubits 4.3.1 (the reference's goldens)
  test/fixtures/{transmon,two_transmons,fluxonium,zero_pi,two_zero_pi}.json   the circuit specs

and writes `reference_goldens.json` beside this script: the spec dictionaries and, per golden,
its parameters and energies, unchanged.  Run once where the reference is mounted:

    python tests/golden/make_golden.py /path/to/KronFreeCircuits.jl

The output is committed; nothing at test time reads the reference checkout.
"""
import json
import os
import sys

SPECS = ["transmon", "two_transmons", "fluxonium", "zero_pi", "two_zero_pi"]
GOLDENS = ["transmon", "two_transmons", "fluxonium", "zero_pi_small", "two_zero_pi_small",
           "two_zero_pi_small_ng0"]


def main(ref_root):
    fx = os.path.join(ref_root, "test", "fixtures")
    with open(os.path.join(fx, "scqubits_reference.json")) as f:
        sc = json.load(f)
    out = {"source": "KronFreeCircuits.jl test/fixtures (scqubits %s goldens)" % sc.get("scqubits_version"),
           "specs": {}, "goldens": {}}
    for name in SPECS:
        with open(os.path.join(fx, name + ".json")) as f:
            out["specs"][name] = json.load(f)
    for name in GOLDENS:
        g = sc[name]
        out["goldens"][name] = {"params": g["params"], "energies": g["energies"],
                                "scqubits_params": g.get("scqubits_params")}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_goldens.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path to a KronFreeCircuits.jl checkout>")
    main(sys.argv[1])
