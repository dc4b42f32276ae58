"""Regenerate the golden fixtures in this folder from the reference checkout.

Reads the reference's regression data for the 4x4x4-cell tension test
(tests/Solid/reference/{linear-cubic,affine-cubic}.dat of the reference
project: columns time, disp_xhi_x, trac_xhi_x) and stores the two series as
solid_trac_xhi.json, so the tests never need the reference tree at run time.

    python tests/golden/make_golden.py /root/reference
"""
import json
import os
import sys


def load(path):
    with open(path) as f:
        head = f.readline().split()
        rows = [[float(v) for v in line.split()] for line in f if line.strip()]
    return {h: [r[i] for r in rows] for i, h in enumerate(head)}


def main(ref_root):
    out = {}
    for name in ["linear-cubic", "affine-cubic"]:
        d = load(os.path.join(ref_root, "tests", "Solid", "reference", name + ".dat"))
        out[name] = {"time": d["time"], "disp_xhi_x": d["disp_xhi_x"], "trac_xhi_x": d["trac_xhi_x"]}
    out["_source"] = "reference tests/Solid/reference/*.dat (regression data of the 4^3-cell tension test)"
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "solid_trac_xhi.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=0)
    print("wrote", dst)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
