"""Loader for the reference-generated fixtures in tests/golden/."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names(kind=None):
    out = []
    for f in sorted(os.listdir(GOLDEN)):
        if f.endswith(".npz"):
            n = f[:-4]
            if kind is None or load(n)["kind"] in (kind if isinstance(kind, tuple) else (kind,)):
                out.append(n)
    return out


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = {k: z[k] for k in z.files}
    p = json.loads(str(d.pop("params")))
    d["kind"] = p["kind"]
    if p["kind"] == "heli":
        d["heli"] = p["heli"]
        d["expect"] = p["expect"]
    else:
        d["geom"] = p["geom"]
    return d


def heli(case):
    from oracle import Heli
    return Heli(**case["heli"])


def geom(case):
    from oracle import Geom
    return Geom(**case["geom"])
