"""The FP64 oracle against the reference's own arithmetic: the harness
oracle/_ref/libt9ref.so runs Tinker9's pair_dfield / pair_ufield /
pair_mpole, damp_thole / damp_ewald, chkpole + rotpole, bsplgen and
image2General (include/seq/*.h, include/ff/image.h) compiled from the
reference's source in double precision, in loops with the structure of its
host path (a pass over every pair at scale 1, then the scaled pairs with
scale - 1 and the non-Ewald kernel).  On the same inputs the oracle's
real-space fields, multipole energy, rotated multipoles and B-splines agree
to FP64 rounding (1e-10 relative).  Skipped where the reference checkout
is absent (the harness is built from it)."""
import numpy as np
import pytest

from gpu_util import water_cluster

ref = pytest.importorskip("oracle.ref")
if not ref.available():
    pytest.skip("reference checkout absent: harness not built", allow_module_level=True)

RTOL = 1e-10


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def systems(tg):
    import lf_fixture as L

    out = {"water648": tg.systems.make_config("water648"), "cluster": water_cluster(tg)}
    out["localframe_pme"], _ = L.system(1)
    out["localframe_gas"], _ = L.system(0)
    return out


@pytest.mark.parametrize("name", ["water648", "cluster", "localframe_pme", "localframe_gas"])
def test_rotpole_matches_reference(oracle, systems, name):
    s = systems[name]
    assert _rel(oracle.rotpole(s), ref.rotpole(s)) < RTOL


@pytest.mark.parametrize("name", ["water648", "cluster", "localframe_pme", "localframe_gas"])
def test_real_space_fields_match_reference(oracle, systems, name):
    s = systems[name]
    if getattr(s, "ptype", None) is not None:
        pytest.skip("per-type-pair Thole table: the harness passes per-atom thole")
    o = oracle.OracleSystem(s, real_only=True)
    h = ref.RefHarness(s)
    f, fp = o.dfield()
    rf, rfp = h.dfield()
    print(name, "dfield", _rel(f, rf), _rel(fp, rfp))
    assert _rel(f, rf) < RTOL and _rel(fp, rfp) < RTOL
    rng = np.random.default_rng(4)
    ud = rng.normal(scale=0.05, size=(s.n, 3))
    up = rng.normal(scale=0.05, size=(s.n, 3))
    g, gp = o.ufield(ud, up)
    rg, rgp = h.ufield(ud, up)
    print(name, "ufield", _rel(g, rg), _rel(gp, rgp))
    assert _rel(g, rg) < RTOL and _rel(gp, rgp) < RTOL


@pytest.mark.parametrize("name", ["water648", "cluster", "localframe_pme", "localframe_gas"])
def test_real_space_multipole_energy_matches_reference(oracle, systems, name):
    s = systems[name]
    _, parts = oracle.OracleSystem(s).empole_energy()
    eo = parts[0] if s.settings.get("use_ewald", 1) else parts.sum()
    er = ref.RefHarness(s).empole()
    print(name, "empole real", eo, er)
    assert abs(eo - er) < RTOL * max(abs(er), 1.0) * 10


def test_bsplgen_matches_reference(oracle):
    for w in np.linspace(0.0, 0.999, 37):
        assert np.abs(oracle.bsplgen(w) - ref.bsplgen(w)).max() < 1e-14
