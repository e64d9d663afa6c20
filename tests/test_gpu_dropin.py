"""The C++ drop-in layer on the GPU: a g++-compiled Tinker9-style caller
(tests/dropin/dropin_driver.cpp) sets the reference's module globals and
calls tinker::induce / dfield / ufield / diagPrecond / sparsePrecondApply /
empole / epolar / emplar with the reference's signatures.  Its results equal
the C-ABI calls on the same inputs bit for bit, gradients arrive in the
reference's fixed-point grad_prec form (2^32 per kcal/mol/A), and the
iteration cap raises tinker::FatalError like src/cu/amoeba/pcg.cu:180-184."""
import importlib
import os
import subprocess

import numpy as np
import pytest

from gpu_util import cpu, engine_for

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER_SRC = os.path.join(ROOT, "tests", "dropin", "dropin_driver.cpp")
DRIVER = os.path.join(ROOT, "tests", "dropin", "_build", "dropin_driver")
CALC_V1 = 0x070


def _write_input(path, s, probe):
    abi = importlib.import_module("tinker-gpu_gb300.abi")
    cfg = abi.make_config(s)
    eik = np.ascontiguousarray(s.excl_ik, dtype=np.int32).reshape(-1)
    with open(path, "wb") as f:
        f.write(bytes(cfg))
        f.write(np.int32(len(eik) // 2).tobytes())
        f.write(np.ascontiguousarray(s.frames, dtype=np.int32).tobytes())
        for a in (s.pole, s.polarity, s.thole, s.pdamp):
            f.write(np.ascontiguousarray(a, dtype=np.float64).tobytes())
        f.write(eik.tobytes())
        f.write(np.ascontiguousarray(s.excl_scale, dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(s.xyz, dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(probe, dtype=np.float64).tobytes())


class _Reader:
    def __init__(self, path, n):
        self.b = open(path, "rb").read()
        self.o = 0
        self.n = n

    def take(self, dtype, count):
        a = np.frombuffer(self.b, dtype=dtype, count=count, offset=self.o)
        self.o += a.nbytes
        return a

    def vec3(self):
        return self.take(np.float32, 3 * self.n).reshape(self.n, 3)


def _fixed(g):
    """The reference's floatTo<fixed>: x * 2^32, truncated toward zero."""
    return np.trunc(np.asarray(g, dtype=np.float64) * 2.0 ** 32).astype(np.int64)


@pytest.fixture(scope="module")
def dropin(gpu_lib, tg, tmp_path_factory):
    b = importlib.import_module("tinker-gpu_gb300.build")
    exe = b.build_cxx_program(DRIVER_SRC, DRIVER)
    s = tg.systems.make_config("water648")
    probe = np.random.default_rng(21).normal(scale=0.05, size=(s.n, 3))
    d = tmp_path_factory.mktemp("dropin")
    fin, fout = str(d / "in.bin"), str(d / "out.bin")
    _write_input(fin, s, probe)
    r = subprocess.run([exe, fin, fout], capture_output=True, text=True, timeout=300)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stderr
    rd = _Reader(fout, s.n)
    out = {k: rd.vec3() for k in ("uind", "uinp", "udir", "udirp", "dfield", "dfieldp", "ufield", "ufieldp",
                                  "diag", "diagp", "sparse", "sparsep")}
    for term in ("empole", "epolar", "emplar"):
        em, ep = rd.take(np.float64, 2)
        vir = rd.take(np.float64, 9).reshape(3, 3)
        g = np.stack([rd.take(np.int64, s.n) for _ in range(3)], axis=1)
        out[term] = (em, ep, vir, g)
    out["threw"] = int(rd.take(np.int32, 1)[0])
    return s, probe, out, r.stdout


def test_dropin_induce_and_fields_equal_c_abi(dropin):
    s, probe, out, _ = dropin
    e = engine_for(s)
    ud, up, rc = e.induce()
    assert rc == 0
    assert np.array_equal(out["uind"], cpu(ud).astype(np.float32))
    assert np.array_equal(out["uinp"], cpu(up).astype(np.float32))
    dd, dp = e.udir()
    assert np.array_equal(out["udir"], cpu(dd).astype(np.float32))
    assert np.array_equal(out["udirp"], cpu(dp).astype(np.float32))
    f, fp = e.dfield()
    assert np.array_equal(out["dfield"], cpu(f).astype(np.float32))
    assert np.array_equal(out["dfieldp"], cpu(fp).astype(np.float32))
    g, gp = e.ufield(probe, -probe)
    assert np.array_equal(out["ufield"], cpu(g).astype(np.float32))
    assert np.array_equal(out["ufieldp"], cpu(gp).astype(np.float32))
    z, zp = e.sparse_precond(probe, -probe)
    assert np.array_equal(out["sparse"], cpu(z).astype(np.float32))
    assert np.array_equal(out["sparsep"], cpu(zp).astype(np.float32))
    # diagPrecond: z = alpha r (src/cu/diagprecond.cu:5-28), in FP32
    pf = probe.astype(np.float32)
    alpha = s.polarity.astype(np.float32)[:, None]
    assert np.array_equal(out["diag"], alpha * pf)
    assert np.array_equal(out["diagp"], alpha * -pf)
    zd, zdp = e.diag_precond(probe, -probe)
    assert np.array_equal(out["diag"], cpu(zd).astype(np.float32))


@pytest.mark.parametrize("term", ["empole", "epolar", "emplar"])
def test_dropin_terms_equal_c_abi(dropin, term):
    s, _, out, _ = dropin
    em, ep, vir, gfix = out[term]
    e = engine_for(s)
    energy, g, w = getattr(e, term)(CALC_V1)
    gf = _fixed(cpu(g))
    print(term, "energy", energy, "drop-in", em, ep)
    assert np.array_equal(gfix, gf)
    assert np.array_equal(vir, w)
    if term == "empole":
        assert em == energy and ep == 0.0
    elif term == "epolar":
        assert ep == energy
    else:
        assert abs((em + ep) - energy) <= 1e-9 * abs(energy)
        parts = e.energy_components()
        assert em == parts[0] + parts[1] + parts[2] and ep == parts[3]
    # the fixed-point conversion through the C ABI gives the same words
    words = [t.cpu().numpy() for t in e.gradient_fixed(g)]
    assert np.array_equal(np.stack(words, axis=1), gf)


def test_dropin_non_convergence_throws(dropin):
    _, _, out, stdout = dropin
    assert out["threw"] == 1
    assert "not converged" in stdout
