"""Writes tests/golden/minimal_ecp5.json: the parts of the reference's ECP5
device fixture (crates/texo-target-ecp5/fixtures/minimal-ecp5.json, schema
version 7) that the device adapter reads: the header, the location grid and
the location types' wires, BELs and pips. Package pins and speed grades are
left out (the adapter does not read them). Run from the repository root
where the reference tree is present:

    python tests/golden/make_ecp5_fixture.py /root/reference
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
KEYS = ("schema_version", "provenance", "family", "device", "width", "height", "location_types", "locations")


def main(reference_root):
    src = os.path.join(reference_root, "crates", "texo-target-ecp5", "fixtures", "minimal-ecp5.json")
    with open(src) as f:
        data = json.load(f)
    out = {k: data[k] for k in KEYS}
    with open(os.path.join(HERE, "minimal_ecp5.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"), sort_keys=False)
        f.write("\n")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
