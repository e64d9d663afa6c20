"""Local-frame test system (Tinker9 test/localframe.cpp) from the committed
fixture tests/golden/local_frame.json."""
import importlib
import json
import os

import numpy as np

tg = importlib.import_module("tinker-gpu_gb300")
HERE = os.path.dirname(os.path.abspath(__file__))


def load():
    with open(os.path.join(HERE, "golden", "local_frame.json")) as f:
        return json.load(f)


def system(ewald):
    fx = load()
    atoms = fx["atoms"]
    xyz = [a["xyz"] for a in atoms]
    types = [a["type"] for a in atoms]
    bonds = sorted({(min(a["index"], b) - 1, max(a["index"], b) - 1) for a in atoms for b in a["bonds"]})
    records = {
        int(t): [(r["axes"][0], r["axes"][1], r["axes"][2], r["values"]) for r in recs]
        for t, recs in fx["multipole"].items()
    }
    polar = {int(t): (p["alpha"], p["thole"], tuple(p["group"])) for t, p in fx["polarize"].items()}
    box = [fx["ewald"]["box"]] * 3 if ewald else None
    s = tg.systems.build_system(xyz, types, bonds, records, polar, scales=fx["scales"], box=box, name="local_frame")
    st = dict(tg.systems.DEFAULT_SETTINGS)
    st["usolve_cutoff"] = fx["usolve_cutoff"]
    if ewald:
        cut = fx["ewald"]["cutoff"]
        st.update(use_ewald=1, ewald_cutoff=cut, nfft=(24, 24, 24), pbuffer=fx["ewald"]["list_buffer"],
                  aewald=tg.systems.ewald_coefficient(cut))
    else:
        st.update(use_ewald=0, ewald_cutoff=1.0e9, nfft=(0, 0, 0), aewald=0.0, pbuffer=fx["ewald"]["list_buffer"])
    s.settings = st
    return s, fx


def expected(fx, ewald):
    case = fx["expected"]["Local-Frame-4" if ewald else "Local-Frame-3"]
    tag = "pme" if ewald else "non-ewald no cutoff"
    return {
        "dfield": case["dfield -- " + tag],
        "ufield": case["ufield -- " + tag],
        "induce": case["default induce routine -- " + tag],
        "epolar": case["various epolar versions -- " + tag],
    }


def synthetic_dipoles(n):
    """uind = 0.1(i+1) + 0.03(j+1), uinp = 0.1(i+1) - 0.03(j+1) (localframe.cpp:276-281)."""
    i = np.arange(n)[:, None] + 1
    j = np.arange(3)[None, :] + 1
    return 0.1 * i + 0.03 * j, 0.1 * i - 0.03 * j
