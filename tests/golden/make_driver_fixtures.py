"""Golden vectors for the spin-boson driver, taken from the reference's own examples.

Reads the reference's input files (inputs/<case>.in) and the outputs its driver wrote
for them (example_outputs/<case>.out) and stores, per case, the input document and the
first rows of the output: t, the observables, the expansion counts, the H applications
per node and (when printed) every bond dimension.  Run in a checkout that has the
reference next to it:

    python tests/golden/make_driver_fixtures.py /path/to/reference

and commit the resulting tests/golden/driver_examples.json.
"""
import json
import os
import sys

# every printed row (t, observables, expansion counts, H applications per node) of these
LONG = ["beta_10/ohmic/spin_boson_sudden", "beta_10/ohmic/spin_boson_debye"]
CASES = [
    "beta_10/ohmic/spin_boson_debye",
    "beta_10/ohmic/spin_boson_exponential",
    "beta_10/ohmic/spin_boson_sudden",
    "beta_10/superohmic/spin_boson_exponential",
    "zero_temperature/subohmic/spin_boson_exponential",
]
ROWS = 4


def parse_row(line, nops):
    f = line.split()
    row = {"t": float(f[0]), "values": [float(x) for x in f[1:1 + nops]]}
    rest = f[1 + nops:]
    row["counts"] = [int(rest[0]), int(rest[1])]
    row["nh_per_node"] = float(rest[2])
    row["hrank"] = [int(x) for x in rest[3:]]
    return row


def main(ref):
    out = {}
    for case in CASES:
        with open(os.path.join(ref, "inputs", case + ".in")) as f:
            doc = json.load(f)
        doc.pop("output file", None)
        nops = len(doc["ops"])
        with open(os.path.join(ref, "example_outputs", case + ".out")) as f:
            lines = [ln for ln in f.read().splitlines() if ln.strip() and not ln.startswith("nh_app")]
        rows = [parse_row(ln, nops) for ln in lines[:ROWS]]
        out[case] = {"input": doc, "rows": rows, "text": [ln + "\n" for ln in lines[:2]]}
        if case in LONG:
            out[case]["trajectory"] = [[r["t"]] + r["values"] + r["counts"] + [r["nh_per_node"]]
                                       for r in (parse_row(ln, nops) for ln in lines)]
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "driver_examples.json")
    with open(dst, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print("wrote", dst, os.path.getsize(dst), "bytes")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_driver_fixtures.py <path of the ttns_lib checkout>")
    main(sys.argv[1])
