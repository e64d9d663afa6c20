"""Na+/Cl- pair with a per-type-pair Thole coefficient (Tinker9
test/polpair.cpp) from the committed fixture tests/golden/polpair.json."""
import importlib
import json
import os

import numpy as np

tg = importlib.import_module("tinker-gpu_gb300")
HERE = os.path.dirname(os.path.abspath(__file__))

# Tinker's default PME grid for a 20 A box (1.2 points per A, listed FFT size)
NFFT = 24


def load():
    with open(os.path.join(HERE, "golden", "polpair.json")) as f:
        return json.load(f)


def thole_pairs(types, polar, pairs):
    """Polarization type per atom and the [t][t] table: min(thole_a, thole_b)
    overridden by each POLPAIR entry (both orders)."""
    kinds = sorted(set(types))
    idx = {t: j for j, t in enumerate(kinds)}
    tab = np.array([[min(polar[a][1], polar[b][1]) for b in kinds] for a in kinds])
    for a, b, v in pairs:
        tab[idx[a], idx[b]] = tab[idx[b], idx[a]] = v
    return np.array([idx[t] for t in types], dtype=np.int32), tab


def system(ewald, fx=None):
    fx = load() if fx is None else fx
    atoms = fx["atoms"]
    xyz = [a["xyz"] for a in atoms]
    types = [a["type"] for a in atoms]
    records = {
        int(t): [(r["axes"][0], r["axes"][1], r["axes"][2], r["values"]) for r in recs]
        for t, recs in fx["multipole"].items()
    }
    polar = {int(t): (p["alpha"], p["thole"], tuple(p["group"])) for t, p in fx["polarize"].items()}
    s = tg.systems.build_system(xyz, types, [], records, polar, scales=fx["scales"], box=[fx["box"]] * 3,
                                name="polpair")
    s.ptype, s.thole_table = thole_pairs(types, polar, fx["polpair"])
    st = dict(tg.systems.DEFAULT_SETTINGS)
    cut = fx["cutoff"]
    if ewald:
        st.update(use_ewald=1, ewald_cutoff=cut, nfft=(NFFT,) * 3, aewald=tg.systems.ewald_coefficient(cut))
    else:
        st.update(use_ewald=0, ewald_cutoff=cut, nfft=(0, 0, 0), aewald=0.0)
    s.settings = st
    return s, fx["expected"]["ewald" if ewald else "nonewald"], fx["eps"]
