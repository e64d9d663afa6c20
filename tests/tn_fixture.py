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
        "vel": z["vel_e6"] * 1e-6,
        "dyn_x": z["dyn_x"],
        "dyn_v": z["dyn_v"],
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


def md_system(fx=None):
    """The water30 restart (positions and velocities of test/file/tinkernist/
    water30.dyn) with the whole amoeba09 force field of the MD test: the
    electrostatics above, buffered 14-7 van der Waals (12 A cutoff, taper
    from 10.8 A) and the water bond / angle / Urey-Bradley terms.
    Returns (system, masses, velocities, fixture)."""
    fx = load() if fx is None else fx
    m = fx["meta"]
    md = m["md"]
    s, _ = system(fx, 0)
    s.xyz = np.array(fx["dyn_x"], dtype=np.float64)
    types = fx["types"]
    vrec = {int(t): tuple(v) + ((0.0,) if len(v) == 2 else ()) for t, v in md["vdw"].items()}
    # vdw-12 / -13 / -14 scales 0 / 0 / 1 (amoeba09.prm:31-34)
    s.vdw = tg.systems.hal_params(types, fx["bonds"], vrec, tg.systems.AMOEBA_VDW_SCALES, m["vdw_cutoff"])
    b, a, u = [], [], []
    adj = {}
    for i, k in fx["bonds"]:
        adj.setdefault(i, []).append(k)
        adj.setdefault(k, []).append(i)
    for o, hs in sorted(adj.items()):
        if types[o] == 36 and len(hs) == 2:
            h1, h2 = sorted(hs)
            b += [(o, h1) + tuple(md["bond"]), (o, h2) + tuple(md["bond"])]
            a.append((h1, o, h2) + tuple(md["angle"]))
            u.append((h1, o, h2) + tuple(md["urey"]))
    g = md["globals"]
    s.valence = tg.systems.ValenceParams(
        bonds=np.array(b), angles=np.array(a), ureys=np.array(u), bond_cubic=g["bond-cubic"],
        bond_quartic=g["bond-quartic"],
        angle_terms=(g["angle-cubic"], g["angle-quartic"], g["angle-pentic"], g["angle-sextic"]))
    mass = np.array([md["mass"][str(t)] for t in types])
    return s, mass, np.array(fx["dyn_v"], dtype=np.float64), fx
