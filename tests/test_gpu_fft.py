"""The fused power-of-two PME FFT against the FP64 oracle and against cuFFT
on the same system."""
import numpy as np
import pytest

from gpu_util import cpu, engine_for, rel_err, rms_err

pytestmark = pytest.mark.gpu
FIELD_RTOL = 5e-5
SAME_RTOL = 2e-6  # own FFT vs cuFFT, both FP32


def test_fields_32cubed_vs_oracle(gpu_lib, oracle, tg):
    s = tg.systems.make_config("water648", nfft=32)
    e = engine_for(s)
    e.pme_own_fft(True)
    f, fp = e.dfield()
    o = oracle.OracleSystem(s)
    of, ofp = o.dfield()
    assert rel_err(cpu(f), of) < FIELD_RTOL and rel_err(cpu(fp), ofp) < FIELD_RTOL
    rng = np.random.default_rng(3)
    u, up = rng.normal(size=(s.n, 3)) * 0.05, rng.normal(size=(s.n, 3)) * 0.05
    g, gp = e.ufield(u, up)
    og, ogp = o.ufield(u, up)
    assert rel_err(cpu(g), og) < FIELD_RTOL and rel_err(cpu(gp), ogp) < FIELD_RTOL


def test_own_fft_matches_cufft_64cubed(gpu_lib, tg):
    s = tg.systems.make_config("water12288")
    a = engine_for(s)
    a.pme_own_fft(True)
    b = engine_for(s)
    b.pme_own_fft(False)
    fa, fpa = a.dfield()
    fb, fpb = b.dfield()
    assert rel_err(cpu(fa), cpu(fb)) < SAME_RTOL and rel_err(cpu(fpa), cpu(fpb)) < SAME_RTOL
    ua, pa, _ = a.induce()
    ub, pb, _ = b.induce()
    D = tg.units.DEBYE
    assert rms_err(cpu(ua) * D, cpu(ub) * D) < 1e-6 and rms_err(cpu(pa) * D, cpu(pb) * D) < 1e-6
    assert a.stats()[0] == b.stats()[0]


def test_forces_and_virial_32cubed_vs_oracle(gpu_lib, oracle, tg):
    """The split transform around the k-space virial pass."""
    s = tg.systems.make_config("water648", nfft=32)
    e = engine_for(s)
    e.pme_own_fft(True)
    _, g, w = e.empole(0x070)
    atoms = np.arange(0, s.n, 40)
    go = oracle.empole_gradient_fd(s, atoms=atoms, cutoff=9.0)
    d = cpu(g)[atoms] - go
    assert float(np.sqrt((d ** 2).mean())) < 1e-4
    wo = oracle.empole_virial_fd(s, diag_only=True, cutoff=9.0)
    assert np.abs(np.diag(w) - np.diag(wo)).max() < 2e-3 + 2e-5 * np.abs(np.diag(wo)).max()
    _, _, w2 = e.epolar(0x070)
    ud, up, *_ = oracle.OracleSystem(s).induce()
    wo2 = oracle.epolar_virial_fd(s, ud, up, diag_only=True, cutoff=9.0)
    assert np.abs(np.diag(w2) - np.diag(wo2)).max() < 2e-3 + 2e-5 * np.abs(np.diag(wo2)).max()


@pytest.mark.parametrize("name,nfft", [("water648", 32), ("water12288", 64)])
@pytest.mark.parametrize("ctas", [2, 4, 8])
def test_cluster_plane_passes_bit_identical(gpu_lib, tg, name, nfft, ctas):
    """Plane passes spread over a thread-block cluster per z plane (bulk
    copies of the row slabs, rows exchanged for columns through distributed
    shared memory) give the same bits as one CTA per plane: fields of both
    grids, a whole graph-captured solve, and the k-space virial split."""
    if ctas == 8 and nfft < 64:
        pytest.skip("8-CTA clusters need 64 points per edge")
    s = tg.systems.make_config(name, nfft=nfft)
    a = engine_for(s)
    a.pme_own_fft(True)
    a.fft_cluster(0)
    b = engine_for(s)
    b.pme_own_fft(True)
    b.fft_cluster(ctas)
    for x, y in zip(a.dfield(), b.dfield()):
        assert np.array_equal(cpu(x), cpu(y))
    rng = np.random.default_rng(8)
    u, up = rng.normal(size=(s.n, 3)) * 0.05, rng.normal(size=(s.n, 3)) * 0.05
    for x, y in zip(a.ufield(u, up), b.ufield(u, up)):
        assert np.array_equal(cpu(x), cpu(y))
    ua, pa, _ = a.induce()
    ub, pb, _ = b.induce()
    assert a.stats()[0] == b.stats()[0]
    assert np.array_equal(cpu(ua), cpu(ub)) and np.array_equal(cpu(pa), cpu(pb))
    ea, ga, wa = a.emplar(0x070)
    eb, gb, wb = b.emplar(0x070)
    assert ea == eb and np.array_equal(cpu(ga), cpu(gb)) and np.array_equal(wa, wb)
    assert b.copy_error() == 0
