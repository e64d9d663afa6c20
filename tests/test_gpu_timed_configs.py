"""The configurations the benchmark times, against the FP64 oracle.

* water12288 (PME 64^3, the default path: the fused three-kernel transform
  with the convolution, 8 lanes per atom in the field kernels): fields,
  induced dipoles from the alpha E start and from the ASPC start after a
  16-frame history, energies per component, multipole + polarization
  gradients of a subset of atoms.
* The 4-lane field kernels (the default above 32,768 atoms) on nacl23142
  and water12288.
* water98304 (PME 128^3 through cuFFT, 4 lanes): fields and the induced
  dipoles of one frame.
* The diagonal preconditioner (pcgprec = 0, Tinker9 src/cu/diagprecond.cu:5-35)
  and the zero start (pcgguess = 0, src/cu/amoeba/pcg.cu:41-48).

Tolerances: fields, max error over the largest component 5e-5; dipoles RMS
2e-5 D, max 2e-4 D; energy components 1e-6 relative each (the multipole
total is a near-cancellation of its three components and is held to 1e-6 of
the sum of their magnitudes); gradients 1e-4 kcal/mol/A RMS, 1e-3 max."""
import numpy as np
import pytest

from gpu_util import cpu, engine_for, rel_err, rms_err

pytestmark = pytest.mark.gpu

FIELD_RTOL = 5.0e-5
DIPOLE_RMS_DEBYE = 2.0e-5
DIPOLE_MAX_DEBYE = 2.0e-4
REL_E = 1.0e-6
RMS_FORCE = 1.0e-4
MAX_FORCE = 1.0e-3


@pytest.fixture(scope="module")
def w12(tg, oracle):
    s = tg.systems.make_config("water12288")
    o = oracle.OracleSystem(s)
    return s, o, o.induce()


def _check_fields(e, o, s, seed=5):
    f, fp = e.dfield()
    of, ofp = o.dfield()
    ef, efp = rel_err(cpu(f), of), rel_err(cpu(fp), ofp)
    rng = np.random.default_rng(seed)
    ud = rng.normal(scale=0.05, size=(s.n, 3))
    up = rng.normal(scale=0.05, size=(s.n, 3))
    g, gp = e.ufield(ud, up)
    og, ogp = o.ufield(ud, up)
    eg, egp = rel_err(cpu(g), og), rel_err(cpu(gp), ogp)
    print(f"{s.name}: dfield {ef:.2e} / {efp:.2e}, ufield {eg:.2e} / {egp:.2e} (max err / max |field|)")
    assert max(ef, efp, eg, egp) < FIELD_RTOL


def _check_dipoles(tg, ud, up, ou, op):
    D = tg.units.DEBYE
    ud, up = np.asarray(ud, dtype=np.float64), np.asarray(up, dtype=np.float64)
    r_d, r_p = rms_err(ud * D, ou * D), rms_err(up * D, op * D)
    m = max(np.abs(ud - ou).max(), np.abs(up - op).max()) * D
    print(f"dipoles vs FP64 oracle: RMS {r_d:.2e} / {r_p:.2e} D, max {m:.2e} D")
    assert r_d < DIPOLE_RMS_DEBYE and r_p < DIPOLE_RMS_DEBYE and m < DIPOLE_MAX_DEBYE


def test_water12288_default_path_fields(gpu_lib, tg, w12):
    s, o, _ = w12
    assert s.settings["nfft"] == (64, 64, 64)
    _check_fields(engine_for(s), o, s)


def test_water12288_default_path_induce(gpu_lib, tg, w12):
    s, o, (ou, op, _, _, oit, _) = w12
    e = engine_for(s)
    ud, up, rc = e.induce()
    it, eps, st = e.stats()
    print(f"water12288: {it} iterations (oracle {oit}), eps {eps:.2e} D")
    assert rc == 0 and st == 0 and eps < 1e-6 and abs(it - oit) <= 2
    _check_dipoles(tg, cpu(ud), cpu(up), ou, op)


def test_water12288_aspc_start_matches_oracle(gpu_lib, tg, oracle, w12):
    """The benchmark's step: a graph-captured solve from the ASPC
    extrapolation of a 16-frame history on a 1 fs trajectory."""
    s, _, _ = w12
    tr = tg.systems.Trajectory(s)
    e = engine_for(s, predictor=1)
    its = []
    for k in range(20):
        x = tr.frame(k)
        ud, up, rc = e.induce_host(x)
        assert rc == 0
        its.append(e.stats()[0])
    ou, op, *_ = oracle.OracleSystem(s, x).induce()
    print("iterations", its)
    assert np.mean(its[17:]) < np.mean(its[:16])
    _check_dipoles(tg, ud, up, ou, op)


def test_water12288_energies(gpu_lib, tg, w12):
    s, o, (ou, op, _, udirp, _, _) = w12
    e = engine_for(s)
    em, parts = e.empole_energy()
    oem, oparts = o.empole_energy()
    rel = np.abs(parts - oparts) / np.abs(oparts)
    print("water12288 empole parts", parts, "oracle", oparts, "relative", rel)
    assert np.all(rel < REL_E)
    assert abs(em - oem) < REL_E * np.abs(oparts).sum()
    e.induce()
    ep = e.epolar_energy()
    oep = o.epolar_energy(ou, udirp)
    print(f"water12288 epolar {ep:.8f} oracle {oep:.8f} relative {abs(ep - oep) / abs(oep):.2e}")
    assert abs(ep - oep) < REL_E * abs(oep)


def test_water12288_gradient_subset(gpu_lib, tg, oracle, w12):
    """emplar (the MD path: multipoles + polarization in one real-space
    pass) against central differences of the oracle energies."""
    s, _, (ou, op, *_) = w12
    e = engine_for(s)
    en, g = e.emplar()
    atoms = np.array([0, 1, 2, 4097, 8190, 12287])
    go = oracle.empole_gradient_fd(s, atoms=atoms) + oracle.epolar_gradient_fd(s, ou, op, atoms=atoms)
    d = cpu(g)[atoms] - go
    rms = float(np.sqrt((d ** 2).mean()))
    print(f"water12288 emplar gradient: RMS err {rms:.2e}, max {np.abs(d).max():.2e}, max |g| {np.abs(go).max():.2f}")
    assert rms < RMS_FORCE and np.abs(d).max() < MAX_FORCE


@pytest.mark.parametrize("name", ["nacl23142", "water12288"])
def test_four_lane_field_kernels(gpu_lib, tg, oracle, name):
    """The 4-lane field and preconditioner kernels (the default above
    32,768 atoms) on smaller boxes where the oracle solve is quick."""
    s = tg.systems.make_config(name)
    e = engine_for(s)
    e.pair_lanes(4)
    o = oracle.OracleSystem(s)
    _check_fields(e, o, s, seed=9)
    ud, up, rc = e.induce()
    assert rc == 0 and e.stats()[1] < 1e-6
    ou, op, *_ = o.induce()
    _check_dipoles(tg, cpu(ud), cpu(up), ou, op)
    rng = np.random.default_rng(7)
    r = rng.normal(size=(s.n, 3))
    rp = rng.normal(size=(s.n, 3))
    z, zp = e.sparse_precond(r, rp)
    oz, ozp = o.sparse_precond(r, rp)
    assert rel_err(cpu(z), oz) < FIELD_RTOL and rel_err(cpu(zp), ozp) < FIELD_RTOL


def test_water98304_fields_and_dipoles(gpu_lib, tg, oracle):
    """The large box: 128^3 grid through cuFFT, 4 lanes per atom."""
    s = tg.systems.make_config("water98304")
    o = oracle.OracleSystem(s)
    e = engine_for(s)
    _check_fields(e, o, s, seed=11)
    ud, up, rc = e.induce()
    it, eps, _ = e.stats()
    assert rc == 0 and eps < 1e-6
    ou, op, _, udirp, oit, _ = o.induce()
    print(f"water98304: {it} iterations (oracle {oit})")
    _check_dipoles(tg, cpu(ud), cpu(up), ou, op)
    ep = e.epolar_energy()
    oep = o.epolar_energy(ou, udirp)
    print(f"water98304 epolar {ep:.6f} oracle {oep:.6f} relative {abs(ep - oep) / abs(oep):.2e}")
    assert abs(ep - oep) < REL_E * abs(oep)


@pytest.mark.parametrize("pcgprec,pcgguess", [(0, 1), (1, 0), (0, 0)],
                         ids=["diagonal", "zero-start", "diagonal-zero-start"])
def test_pcg_variants_vs_oracle(gpu_lib, tg, oracle, pcgprec, pcgguess):
    """The diagonal preconditioner and the zero start, solved by the graph
    and by the host-driven loop (bit-identical), against the oracle run with
    the same options."""
    s = tg.systems.make_config("water648")
    e = engine_for(s, pcgprec=pcgprec, pcgguess=pcgguess)
    f = engine_for(s, pcgprec=pcgprec, pcgguess=pcgguess)
    f.use_graph(False)
    ud, up, rc = e.induce()
    it, eps, _ = e.stats()
    vd, vp, _ = f.induce()
    assert rc == 0 and eps < 1e-6 and f.stats()[0] == it
    assert np.array_equal(cpu(ud), cpu(vd)) and np.array_equal(cpu(up), cpu(vp))
    ou, op, _, _, oit, _ = oracle.OracleSystem(s).induce(guess=pcgguess, pcgprec=pcgprec)
    print(f"pcgprec {pcgprec} pcgguess {pcgguess}: {it} iterations (oracle {oit})")
    assert abs(it - oit) <= 2
    _check_dipoles(tg, cpu(ud), cpu(up), ou, op)
    # the sparse preconditioner takes fewer iterations than the diagonal one
    if pcgprec == 0:
        g = engine_for(s, pcgprec=1, pcgguess=pcgguess)
        g.induce()
        assert g.stats()[0] < it
