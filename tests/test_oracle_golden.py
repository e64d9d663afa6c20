"""The FP64 oracle against the reference's own known answers (Tinker9
test/localframe.cpp, Local-Frame-3 non-Ewald and Local-Frame-4 PME), margin
1e-4 as in the reference test (localframe.cpp:211, :382)."""
import numpy as np
import pytest

import lf_fixture as L

MARGIN = 1.0e-4


@pytest.mark.parametrize("ewald", [0, 1], ids=["nonewald", "pme"])
def test_dfield_golden(oracle, ewald):
    s, fx = L.system(ewald)
    ex = L.expected(fx, ewald)["dfield"]
    f, fp = oracle.OracleSystem(s).dfield()
    assert np.abs(f - ex["ref_dir_field_d"]).max() < MARGIN
    assert np.abs(fp - ex["ref_dir_field_p"]).max() < MARGIN


@pytest.mark.parametrize("ewald", [0, 1], ids=["nonewald", "pme"])
def test_ufield_golden(oracle, ewald):
    s, fx = L.system(ewald)
    ex = L.expected(fx, ewald)["ufield"]
    ud, up = L.synthetic_dipoles(s.n)
    f, fp = oracle.OracleSystem(s).ufield(ud, up)
    assert np.abs(f - ex["ref_ufield_d"]).max() < MARGIN
    assert np.abs(fp - ex["ref_ufield_p"]).max() < MARGIN


@pytest.mark.parametrize("ewald", [0, 1], ids=["nonewald", "pme"])
def test_induce_golden(oracle, tg, ewald):
    s, fx = L.system(ewald)
    ex = L.expected(fx, ewald)["induce"]
    u, p, _, _, it, eps = oracle.OracleSystem(s).induce()
    d = tg.units.DEBYE
    assert eps < s.settings["poleps"]
    assert 3 <= it < 100
    assert np.abs(u * d - ex["ref_ud_debye"]).max() < MARGIN
    assert np.abs(p * d - ex["ref_up_debye"]).max() < MARGIN


def test_fft_matches_numpy(oracle):
    """The oracle's mixed-radix FFT against numpy on a 24 x 18 x 10 grid."""
    import ctypes as C

    lib = oracle.lib()
    rng = np.random.default_rng(0)
    g = (rng.normal(size=(10, 18, 24)) + 1j * rng.normal(size=(10, 18, 24))).astype(np.complex128)
    ref = np.fft.fftn(g)
    h = np.ascontiguousarray(g.copy())
    lib.or_fft3d.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
    lib.or_fft3d(h.ctypes.data, 24, 18, 10, -1)
    assert np.abs(h - ref).max() < 1e-9 * np.abs(ref).max()


def test_bspline_partition_of_unity(oracle):
    for w in (0.0, 0.13, 0.5, 0.99):
        th = oracle.bsplgen(w, 5, 4)
        assert abs(th[:, 0].sum() - 1) < 1e-14
        assert abs(th[:, 1].sum()) < 1e-14  # derivative of a constant
        assert abs(th[:, 2].sum()) < 1e-13


def test_bsmod_positive(oracle):
    for n in (24, 64, 72, 128):
        m = oracle.bsmod(n)
        assert (m > 0).all() and abs(m[0] - 1) < 1e-12


def test_aspc_weights_sum_to_one(oracle):
    """ASPC extrapolation reproduces a constant history."""
    hist = np.ones((16, 6))
    for nualt in (16, 17, 31):
        assert np.allclose(oracle.aspc_sum(hist, nualt), 1.0, atol=1e-12)


def test_gear_extrapolates_a_quintic(oracle):
    """Gear's six weights continue any polynomial of degree <= 5; the ring
    slot of frame t is t mod 6 (ulspredSave, src/amoeba/induce.cpp:37)."""
    rng = np.random.default_rng(3)
    c = rng.normal(size=(6, 4))
    p = lambda t: sum(c[k] * t ** k for k in range(6))
    for nualt in (6, 7, 11):
        hist = np.zeros((6, 4))
        for t in range(nualt - 6, nualt):
            hist[t % 6] = p(t)
        assert np.allclose(oracle.gear_sum(hist, nualt), p(nualt), rtol=1e-9, atol=1e-6)


@pytest.mark.parametrize("ewald", [0, 1], ids=["nonewald", "pme"])
def test_epolar_energy_golden(oracle, ewald):
    """Polarization energy by the dot product (localframe.cpp:329-333, :500-505)."""
    s, fx = L.system(ewald)
    e = oracle.OracleSystem(s).epolar_energy()
    assert abs(e - L.expected(fx, ewald)["epolar"]["ref_eng"]) < MARGIN


def test_empole_energy_golden_nonewald(oracle):
    """Local-Frame-1: gas phase, no cutoff (localframe.cpp:22-74), eps 1e-5."""
    s, fx = L.system(0)
    e, _ = oracle.OracleSystem(s).empole_energy()
    assert abs(e - fx["expected"]["Local-Frame-1"]["empole -- gas phase, no cutoff"]["ref_eng"]) < 1e-4


def test_empole_energy_golden_pme_parts(oracle):
    """Local-Frame-2: PME real / recip / self parts (localframe.cpp:124-130), eps 1e-4."""
    s, fx = L.system(1)
    e, parts = oracle.OracleSystem(s).empole_energy()
    ex = fx["expected"]["Local-Frame-2"]["empole -- pme"]
    assert abs(parts[0] - ex["ref_ereal"]) < 1e-4
    assert abs(parts[1] - ex["ref_erecip"]) < 1e-4
    assert abs(parts[2] - ex["ref_eself"]) < 1e-4
    assert abs(e - (ex["ref_ereal"] + ex["ref_erecip"] + ex["ref_eself"])) < 1e-4


# The reference skips the last molecule (a planar NH3) in its gradient
# comparisons (test/localframe.cpp:12-21, do_ij); so do these tests.
GRAD_ATOMS = 18


@pytest.mark.parametrize("ewald", [0, 1], ids=["gas", "pme"])
def test_empole_gradient_golden(oracle, ewald):
    """Local-Frame-1/2 empole gradients (localframe.cpp:49-72, :133-151), eps 5e-4."""
    s, fx = L.system(ewald)
    case = fx["expected"]["Local-Frame-2" if ewald else "Local-Frame-1"]
    ex = case["empole -- pme" if ewald else "empole -- gas phase, no cutoff"]
    g = oracle.empole_gradient_fd(s, atoms=range(GRAD_ATOMS))
    ref = np.array(ex["ref_grad"])[:GRAD_ATOMS]
    assert np.abs(g - ref).max() < ex["eps_g"]


@pytest.mark.parametrize("ewald", [0, 1], ids=["nonewald", "pme"])
def test_epolar_gradient_golden(oracle, ewald):
    """Local-Frame-3/4 epolar gradients at the converged dipoles
    (localframe.cpp:344-366, :521-543), eps 5e-4."""
    s, fx = L.system(ewald)
    ud, up, *_ = oracle.OracleSystem(s).induce()
    g = oracle.epolar_gradient_fd(s, ud, up, atoms=range(GRAD_ATOMS))
    ref = np.array(L.expected(fx, ewald)["epolar"]["ref_grad"])[:GRAD_ATOMS]
    assert np.abs(g - ref).max() < 5e-4


def test_virial_fd_gas_symmetric(oracle, tg):
    """Without PBC the strain derivative of the energy is symmetric
    (rotational invariance): a check of the finite-difference virial that the
    GPU virial tests compare against."""
    from gpu_util import water_cluster

    s = water_cluster(tg, nmol=12)
    w = oracle.empole_virial_fd(s)
    assert np.abs(w - w.T).max() < 1e-5 * max(1.0, np.abs(w).max())


TN_MAX = 1e-4   # Debye, every atom (the reference test's own margin is 1e-3 on four atoms)
TN_RMS = 2e-5   # Debye: the files' 1e-6 rounding plus the reference run's 1e-5 RMS convergence


@pytest.mark.parametrize("frame", [0, 1])
def test_tinkernist_dipoles_golden(oracle, tg, frame):
    """2,684-atom water/ion box, PME 36^3 (test/tinkernist.cpp): the oracle's
    induced and direct dipoles against the reference's .uind / .udir files."""
    import tn_fixture as T

    s, fx = T.system(frame=frame)
    o = oracle.OracleSystem(s)
    ud, _, *_ = o.induce()
    fd, _ = o.dfield()
    D = tg.units.DEBYE
    for got, ref in ((ud * D, fx["uind"][frame]), (fd * s.polarity[:, None] * D, fx["udir"][frame])):
        d = got - ref
        assert np.abs(d).max() < TN_MAX and np.sqrt((d ** 2).mean()) < TN_RMS


@pytest.mark.parametrize("name", ["NaCl-2", "NaCl-3"])
def test_nacl_empole_golden(oracle, name):
    """Two ions (test/nacl.cpp): multipole energy, gradient (central
    differences) and virial (strain derivatives; the diagonal under PME)
    against the reference's known answers at its own margins."""
    import nacl_fixture as N

    s, ex = N.system(name)
    eps = ex["eps"]
    cut = s.settings["ewald_cutoff"]
    e, _ = oracle.OracleSystem(s).empole_energy()
    assert abs(e - ex["ref_eng"]) < eps + 5e-5  # known answers carry four decimals
    g = oracle.empole_gradient_fd(s, atoms=np.arange(2), cutoff=cut)
    assert np.abs(g - np.array(ex["ref_grad"])).max() < eps + 5e-5
    w = oracle.empole_virial_fd(s, diag_only=bool(s.settings["use_ewald"]), cutoff=cut)
    m = ~np.isnan(w)
    assert np.abs(w - np.array(ex["ref_v"]))[m].max() < eps + 5e-4  # three decimals


@pytest.mark.parametrize("ewald", [1, 0], ids=["ewald", "nonewald"])
def test_polpair_golden(oracle, ewald):
    """Na+/Cl- with a per-type-pair Thole coefficient (test/polpair.cpp):
    total energy, gradient and virial (diagonal under PME) of the multipole
    plus polarization terms against the reference's known answers."""
    import pp_fixture as P

    s, ex, eps = P.system(ewald)
    cut = s.settings["ewald_cutoff"]
    o = oracle.OracleSystem(s)
    ud, up, *_ = o.induce()
    e = o.empole_energy()[0] + o.epolar_energy()
    assert abs(e - ex["energy"]) < eps["energy"]
    g = oracle.empole_gradient_fd(s, atoms=np.arange(2), cutoff=cut) + oracle.epolar_gradient_fd(
        s, ud, up, atoms=np.arange(2), cutoff=cut)
    assert np.abs(g - np.array(ex["gradient"])).max() < eps["gradient"]
    w = oracle.empole_virial_fd(s, diag_only=bool(ewald), cutoff=cut) + oracle.epolar_virial_fd(
        s, ud, up, diag_only=bool(ewald), cutoff=cut)
    m = ~np.isnan(w)
    assert np.abs(w - np.array(ex["virial"]))[m].max() < eps["virial"]
    # the pair coefficient matters: min(thole) gives another answer
    s.ptype = None
    assert abs(oracle.OracleSystem(s).epolar_energy() - (ex["energy"] - o.empole_energy()[0])) > 1.0


def test_extfield_golden(oracle):
    """Four waters and a Na+ in a uniform external field (test/extfield.cpp,
    amoebabio18): multipole, polarization and total energies, gradients and
    virials (diagonal under PME) against the reference's known answers."""
    import ef_fixture as F

    s, fx = F.system()
    ex, eps = fx["expected"], fx["eps"]
    cut = s.settings["ewald_cutoff"]
    o = oracle.OracleSystem(s)
    em = o.empole_energy()[0]
    ud, up, *_ = o.induce()
    ep = o.epolar_energy()
    assert abs(em - ex["mpole"]["energy"]) < eps["energy"]
    assert abs(ep - ex["polar"]["energy"]) < eps["energy"]
    assert abs(em + ep - ex["mplar"]["energy"]) < eps["energy"]
    atoms = np.arange(s.n)
    gm = oracle.empole_gradient_fd(s, atoms=atoms, cutoff=cut)
    gp = oracle.epolar_gradient_fd(s, ud, up, atoms=atoms, cutoff=cut)
    for g, key in ((gm, "mpole"), (gp, "polar"), (gm + gp, "mplar")):
        assert np.abs(g - np.array(ex[key]["gradient"])).max() < eps["gradient"]
    wm = np.diag(oracle.empole_virial_fd(s, diag_only=True, cutoff=cut))
    wp = np.diag(oracle.epolar_virial_fd(s, ud, up, diag_only=True, cutoff=cut))
    for w, key in ((wm, "mpole"), (wp, "polar"), (wm + wp, "mplar")):
        assert np.abs(w - np.diag(np.array(ex[key]["virial"]))).max() < eps["virial"]


HAL_TITLES = ["- ehal -- no switch", "- ehal -- switch, near cut", "- ehal -- switch, near off"]


@pytest.mark.parametrize("title", HAL_TITLES)
def test_hal_golden(oracle, title):
    """Buffered 14-7 energy, gradient and virial of the NaCl-1 pair at 2.2,
    2.38 and 2.5 A (no taper, taper near its start, near the cutoff)."""
    import dataclasses

    import nacl_fixture as N
    from oracle import mm_oracle

    s, ex = N.hal_system(title)
    e = mm_oracle.hal_energy(s)
    assert abs(e - ex["ref_eng"]) < ex["eps"]
    g = oracle._fd(lambda x: mm_oracle.hal_energy(s, x), np.asarray(s.xyz, dtype=np.float64), [0, 1], 1e-6)
    assert np.abs(g - np.array(ex["ref_grad"])).max() < ex["eps"]
    w = oracle._strain_fd(s, lambda s2: mm_oracle.hal_energy(s2), False, 1e-6)
    assert np.abs(w - np.array(ex["ref_v"])).max() < ex["eps"] * 10  # known answers with three decimals


def _valence_golden():
    import json
    import os

    with open(os.path.join(os.path.dirname(__file__), "golden", "valence.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("term", ["bond", "urey"])
def test_valence_golden(oracle, term):
    """Anharmonic bonds of a 304-atom protein (test/bond.cpp) and the
    Urey-Bradley term of ten waters (test/urey.cpp): energy, gradient,
    virial of the oracle against the reference's known answers."""
    from oracle import mm_oracle

    d = _valence_golden()[term]
    x = np.asarray(d["xyz"], dtype=np.float64)
    if term == "bond":
        f = lambda y: mm_oracle.bond_energy(y, d["bonds"], d["cubic"], d["quartic"])
    else:
        f = lambda y: mm_oracle.urey_energy(y, d["ureys"], d["cubic"], d["quartic"])
    ex, eps = d["expected"], d["eps"]
    assert abs(f(x) - ex["energy"]) < eps["energy"]
    g = oracle._fd(f, x, list(range(len(x))), 1e-6)
    assert np.abs(g - np.array(ex["gradient"])).max() < eps["gradient"]
    # virial: dE/d(eps_ab) = sum_i g_ia x_ib (a translation-invariant sum)
    w = g.T @ x
    assert np.abs(0.5 * (w + w.T) - np.array(ex["virial"])).max() < eps["virial"]
