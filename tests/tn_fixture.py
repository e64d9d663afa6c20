"""TinkerNIST water box (Tinker9 test/tinkernist.cpp): 892 AMOEBA waters and
four Na+/Cl- pairs in a 30 A cube, from the committed fixture
tests/golden/tinkernist.npz (coordinates and the reference's induced and
direct dipoles after MD steps 1 and 2)."""
import importlib
import json
import os

import numpy as np

tg = importlib.import_module("tinker-gpu_gb300")
HERE = os.path.dirname(os.path.abspath(__file__))

# Tinker's default PME grid for a 30 A box: the smallest listed FFT size
# (products of 2, 3, 5) at or above 1.2 points per A.
NFFT = 36
REFERENCE_EPS = 0.001  # Debye, test/tinkernist.cpp:232-239


def load():
    z = np.load(os.path.join(HERE, "golden", "tinkernist.npz"))
    meta = json.loads(str(z["meta"]))
    return {
        "meta": meta,
        "types": z["types"].tolist(),
        "bonds": [tuple(b) for b in z["bonds"].tolist()],
        "xyz": z["xyz_e6"] * 1e-6,
        "uind": z["uind_e6"] * 1e-6,
        "udir": z["udir_e6"] * 1e-6,
    }


def system(fx=None, frame=0):
    fx = load() if fx is None else fx
    m = fx["meta"]
    records = {
        int(t): [(r["axes"][0], r["axes"][1], r["axes"][2], r["values"]) for r in recs]
        for t, recs in m["multipole"].items()
    }
    polar = {int(t): (p["alpha"], p["thole"], tuple(p["group"])) for t, p in m["polarize"].items()}
    s = tg.systems.build_system(fx["xyz"][frame], fx["types"], fx["bonds"], records, polar, scales=m["scales"],
                                box=m["box"], name="tinkernist")
    st = dict(tg.systems.DEFAULT_SETTINGS)
    cut = m["ewald_cutoff"]
    st.update(use_ewald=1, ewald_cutoff=cut, nfft=(NFFT,) * 3, aewald=tg.systems.ewald_coefficient(cut))
    s.settings = st
    return s, fx
