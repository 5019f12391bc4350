"""Generates tests/golden/*.json from the reference's own shipped files.

Run where a checkout of the reference is available, with its path as the
only argument (or in the HYB_REFERENCE environment variable):
    python tests/golden/make_golden.py <reference checkout>
Nothing at test time reads the reference; the tests read only the JSON
written here.

flow2d_gkua_step0.json
    Hybrid2D/output/flow2d-GKUA.dat is the moment field the reference wrote
    at step 0 of its shipped cylinder case (IO.f90:369-386): every cell holds
    the Gauss-Legendre moments of the initial Maxwellian (GKUA_sudufenbu.f90
    :22-53) for the inputs in Hybrid2D/input/control.in and
    Quadrature_Para.dat.  The file is uniform; one row plus the inputs that
    produced it are stored.

gauss_hermite_half_range.json
    The node / weight table of the reference's "modified (half-range)
    Gauss-Hermite" velocity grid (GaussHermite in
    Hybrid2D/src/GKUA_lisansudu.f90:364-440): nodes a_k and weights H_k of
    the quadrature of integral_0^inf exp(-v^2) g(v) dv for 7, 8 and 16 nodes,
    as printed in that routine.
"""
import json
import os
import re
import sys

ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("HYB_REFERENCE")
if not ref:
    sys.exit("usage: make_golden.py <reference checkout>  (or set HYB_REFERENCE)")
here = os.path.dirname(os.path.abspath(__file__))
src = os.path.join(ref, "Hybrid2D", "output", "flow2d-GKUA.dat")
rows = []
with open(src) as fh:
    lines = fh.readlines()
for line in lines[2:]:
    rows.append([float(x) for x in line.split()])
first = rows[0]
assert all(r[2:] == first[2:] for r in rows), "step-0 field is expected to be uniform"
names = ["d", "u", "v", "T", "p", "txx", "tyy", "txy", "qx", "qy", "tzz", "cf"]
out = {
    "source": "Hybrid2D/output/flow2d-GKUA.dat (columns x,y,d,u,v,T,p,txx,tyy,txy,qx,qy,tzz,cf)",
    "cells": len(rows),
    "values": dict(zip(names, first[2:])),
    "printed_decimals": 10,
    # inputs read by the reference (Hybrid2D/input/control.in, Quadrature_Para.dat)
    "inputs": {
        "mole_mass": 28.0, "gamma": 1.6667, "khs": 0, "alpha": 1.0, "omega": 0.81,
        # read_parameter reads vis_ref and Tref from the VHS, Sutherland and
        # LJ lines in turn (opencfd_ec2d.f90:128-132); the LJ line's values
        # are the ones left for the VHS viscosity law
        "vis_ref": 1.66414e-05, "tref": 273.0, "ma": 3.0, "nd_inf": 1.18117e20,
        "t_inf": 260.771, "lref": 1.0, "aoa": 0.0,
        "quadrature": "gauss-legendre", "dv": 1.2, "intervals": 15, "vdown": -9.0, "kgln": 4,
    },
}
with open(os.path.join(here, "flow2d_gkua_step0.json"), "w") as fh:
    json.dump(out, fh, indent=1)
print("wrote", os.path.join(here, "flow2d_gkua_step0.json"))


# ---- half-range Gauss-Hermite table -------------------------------------------
src = os.path.join(ref, "Hybrid2D", "src", "GKUA_lisansudu.f90")
with open(src, errors="replace") as fh:
    text = fh.read()
body = text[text.index("SUBROUTINE GaussHermite(AGH,HGH,NV)"):]
body = body[:body.index("END IF")]
tables, cur = {}, None
for line in body.splitlines():
    m = re.search(r"NV\.EQ\.(\d+)", line)
    if m:
        cur = int(m.group(1))
        tables[cur] = {"a": {}, "h": {}}
        continue
    m = re.match(r"\s*(AGH|HGH)\((\d+)\)\s*=\s*([-+0-9.EeDd]+)", line)
    if m and cur is not None:
        key = "a" if m.group(1) == "AGH" else "h"
        tables[cur][key][int(m.group(2))] = float(m.group(3).replace("D", "E").replace("d", "e"))
out = {"source": "Hybrid2D/src/GKUA_lisansudu.f90, SUBROUTINE GaussHermite",
       "weight": "exp(-v^2) on [0, inf)",
       "tables": {str(n): {"nodes": [t["a"][k] for k in range(1, n + 1)],
                           "weights": [t["h"][k] for k in range(1, n + 1)]} for n, t in sorted(tables.items())}}
with open(os.path.join(here, "gauss_hermite_half_range.json"), "w") as fh:
    json.dump(out, fh, indent=1)
print("wrote", os.path.join(here, "gauss_hermite_half_range.json"))
