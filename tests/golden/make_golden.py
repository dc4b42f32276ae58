"""Regenerate the golden fixtures in this folder from the reference checkout.

* solid_trac_xhi.json: the regression data of the 4x4x4-cell tension test
  (tests/Solid/reference/{linear-cubic,affine-cubic,affine-hexagonal,
  transverselyisotropic,neo-hookean}.dat of the reference project: columns
  time, disp_xhi_x, trac_xhi_x).
* eshelby.json: the analytic Eshelby curves the reference's Eshelby test
  compares with (tests/Eshelby/reference/Eshelby_displacement.csv, columns
  z, u1..u3 in units of 1e-4; Eshelby_sigma_normal.csv, columns z,
  sigma11..sigma33 in units of E/1000), along the ray x = y = 0.25.

The tests never need the reference tree at run time.

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


def load_csv(path):
    with open(path) as f:
        head = f.readline().strip().split(",")
        rows = [[float(v) for v in line.split(",")] for line in f if line.strip()]
    return {h: [r[i] for r in rows] for i, h in enumerate(head)}


def write(name, out):
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), name)
    with open(dst, "w") as f:
        json.dump(out, f, indent=0)
    print("wrote", dst)


def main(ref_root):
    out = {}
    for name in ["linear-cubic", "affine-cubic", "affine-hexagonal", "transverselyisotropic", "neo-hookean"]:
        d = load(os.path.join(ref_root, "tests", "Solid", "reference", name + ".dat"))
        out[name] = {"time": d["time"], "disp_xhi_x": d["disp_xhi_x"], "trac_xhi_x": d["trac_xhi_x"]}
    out["_source"] = "reference tests/Solid/reference/*.dat (regression data of the 4^3-cell tension test)"
    write("solid_trac_xhi.json", out)

    out = {}
    for name in ["displacement", "sigma_normal"]:
        out[name] = load_csv(os.path.join(ref_root, "tests", "Eshelby", "reference", "Eshelby_" + name + ".csv"))
    out["_source"] = ("reference tests/Eshelby/reference/Eshelby_{displacement,sigma_normal}.csv "
                      "(analytic Eshelby solution along x = y = 0.25)")
    write("eshelby.json", out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
