"""Two-ion known answers (Tinker9 test/nacl.cpp NaCl-2, NaCl-3) from the
committed fixture tests/golden/nacl.json."""
import importlib
import json
import os

tg = importlib.import_module("tinker-gpu_gb300")
HERE = os.path.dirname(os.path.abspath(__file__))


def load():
    with open(os.path.join(HERE, "golden", "nacl.json")) as f:
        return json.load(f)


def system(name, fx=None):
    c = (load() if fx is None else fx)[name]
    atoms = c["atoms"]
    xyz = [a["xyz"] for a in atoms]
    types = [a["type"] for a in atoms]
    bonds = sorted({(min(a["index"], b) - 1, max(a["index"], b) - 1) for a in atoms for b in a["bonds"]})
    records = {
        int(t): [(r["axes"][0], r["axes"][1], r["axes"][2], r["values"]) for r in recs]
        for t, recs in c["multipole"].items()
    }
    polar = {int(t): (p["alpha"], p["thole"], tuple(p["group"])) for t, p in c["polarize"].items()}
    s = tg.systems.build_system(xyz, types, bonds, records, polar, scales=c["scales"], box=[c["box"]] * 3, name=name)
    st = dict(tg.systems.DEFAULT_SETTINGS)
    if c["ewald"]:
        st.update(use_ewald=1, ewald_cutoff=c["cutoff"], nfft=tuple(c["nfft"]),
                  aewald=tg.systems.ewald_coefficient(c["cutoff"]))
    else:
        st.update(use_ewald=0, ewald_cutoff=c["cutoff"], nfft=(0, 0, 0), aewald=0.0)
    s.settings = st
    return s, c["expected"]


def hal_system(title, fx=None):
    """NaCl-1 (test/nacl.cpp:35-190): a Na+/Cl- pair in an 18.643 A box with
    only the buffered 14-7 term, vdw-cutoff 2.6 A."""
    c = (load() if fx is None else fx)["NaCl-1"]
    case = c["cases"][title]
    atoms = case["atoms"]
    xyz = [a["xyz"] for a in atoms]
    types = [a["type"] for a in atoms]
    # multipole / polarize records are not used by this term: a neutral,
    # non-polarizable placeholder keeps the context valid
    records = {t: [(0, 0, 0, [0.0] * 10)] for t in types}
    polar = {t: (0.0, 0.39, ()) for t in types}
    s = tg.systems.build_system(xyz, types, [], records, polar, box=[c["box"]] * 3, name="nacl-hal")
    vrec = {int(t): tuple(v) for t, v in c["vdw"].items()}
    s.vdw = tg.systems.hal_params(types, [], vrec, {}, c["vdw_cutoff"])
    st = dict(tg.systems.DEFAULT_SETTINGS)
    st.update(use_ewald=0, ewald_cutoff=c["vdw_cutoff"], nfft=(0, 0, 0), aewald=0.0)
    s.settings = st
    return s, case
