"""Four AMOEBA waters and a Na+ in a uniform external field (Tinker9
test/extfield.cpp) from the committed fixture tests/golden/extfield.json."""
import importlib
import json
import os

import numpy as np

tg = importlib.import_module("tinker-gpu_gb300")
HERE = os.path.dirname(os.path.abspath(__file__))

# Tinker's default PME grid for an 18.643 A box (1.2 points per A, listed size)
NFFT = 24


def load():
    with open(os.path.join(HERE, "golden", "extfield.json")) as f:
        return json.load(f)


def wrap_molecules(xyz, box, bonds, masses):
    """Move each molecule (bonded component) so that its centre of mass lies
    in the primary cell [-L/2, L/2), as the reference's bounds() does before
    the external-field term (src/acc/atom.cpp:16-58, src/elec.cpp:823-833)."""
    n = len(xyz)
    parent = list(range(n))

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    for i, k in bonds:
        parent[find(i)] = find(k)
    out = np.array(xyz, dtype=np.float64)
    box = np.asarray(box, dtype=np.float64)
    roots = np.array([find(i) for i in range(n)])
    for r in np.unique(roots):
        idx = np.nonzero(roots == r)[0]
        c = (out[idx] * masses[idx, None]).sum(axis=0) / masses[idx].sum()
        out[idx] += -box * np.round(c / box)
    return out


def system(fx=None):
    fx = load() if fx is None else fx
    atoms = fx["atoms"]
    xyz = [a["xyz"] for a in atoms]
    types = [a["type"] for a in atoms]
    bonds = sorted({(min(a["index"], b) - 1, max(a["index"], b) - 1) for a in atoms for b in a["bonds"]})
    records = {
        int(t): [(r["axes"][0], r["axes"][1], r["axes"][2], r["values"]) for r in recs]
        for t, recs in fx["multipole"].items()
    }
    polar = {int(t): (p["alpha"], p["thole"], tuple(p["group"])) for t, p in fx["polarize"].items()}
    masses = np.array([fx["mass"][str(t)] for t in types])
    xyz = wrap_molecules(xyz, [fx["box"]] * 3, bonds, masses)
    s = tg.systems.build_system(xyz, types, bonds, records, polar, scales=fx["scales"], box=[fx["box"]] * 3,
                                name="extfield")
    s.exfld = np.array(fx["field_e_per_a2"])
    st = dict(tg.systems.DEFAULT_SETTINGS)
    cut = fx["ewald_cutoff"]
    st.update(use_ewald=1, ewald_cutoff=cut, nfft=(NFFT,) * 3, aewald=tg.systems.ewald_coefficient(cut))
    s.settings = st
    return s, fx
