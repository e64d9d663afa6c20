"""CUDA dfield / ufield / sparse preconditioner against the FP64 oracle and
the reference's known answers.  FP32 kernels: max error relative to the
largest field component below FIELD_RTOL."""
import numpy as np
import pytest

import lf_fixture as L
from gpu_util import cpu, engine_for, rel_err

pytestmark = pytest.mark.gpu
FIELD_RTOL = 5.0e-5
GOLDEN_MARGIN = 1.0e-4


@pytest.mark.parametrize("ewald", [0, 1], ids=["nonewald", "pme"])
def test_localframe_dfield(gpu_lib, oracle, ewald):
    s, fx = L.system(ewald)
    e = engine_for(s)
    f, fp = e.dfield()
    of, ofp = oracle.OracleSystem(s).dfield()
    assert rel_err(cpu(f), of) < FIELD_RTOL
    assert rel_err(cpu(fp), ofp) < FIELD_RTOL
    ex = L.expected(fx, ewald)["dfield"]
    assert np.abs(cpu(f) - ex["ref_dir_field_d"]).max() < GOLDEN_MARGIN
    assert np.abs(cpu(fp) - ex["ref_dir_field_p"]).max() < GOLDEN_MARGIN


@pytest.mark.parametrize("ewald", [0, 1], ids=["nonewald", "pme"])
def test_localframe_ufield(gpu_lib, oracle, ewald):
    s, fx = L.system(ewald)
    e = engine_for(s)
    ud, up = L.synthetic_dipoles(s.n)
    f, fp = e.ufield(ud, up)
    of, ofp = oracle.OracleSystem(s).ufield(ud, up)
    assert rel_err(cpu(f), of) < FIELD_RTOL
    assert rel_err(cpu(fp), ofp) < FIELD_RTOL
    ex = L.expected(fx, ewald)["ufield"]
    assert np.abs(cpu(f) - ex["ref_ufield_d"]).max() < GOLDEN_MARGIN
    assert np.abs(cpu(fp) - ex["ref_ufield_p"]).max() < GOLDEN_MARGIN


@pytest.mark.parametrize("name", ["water648", "nacl23142"])
def test_water_fields(gpu_lib, oracle, tg, name):
    s = tg.systems.make_config(name)
    e = engine_for(s)
    o = oracle.OracleSystem(s)
    f, fp = e.dfield()
    of, ofp = o.dfield()
    assert rel_err(cpu(f), of) < FIELD_RTOL
    assert rel_err(cpu(fp), ofp) < FIELD_RTOL
    rng = np.random.default_rng(5)
    ud = rng.normal(scale=0.05, size=(s.n, 3))
    up = rng.normal(scale=0.05, size=(s.n, 3))
    g, gp = e.ufield(ud, up)
    og, ogp = o.ufield(ud, up)
    assert rel_err(cpu(g), og) < FIELD_RTOL
    assert rel_err(cpu(gp), ogp) < FIELD_RTOL


def test_sparse_precond(gpu_lib, oracle, tg):
    s = tg.systems.make_config("water648")
    e = engine_for(s)
    rng = np.random.default_rng(7)
    r = rng.normal(size=(s.n, 3))
    rp = rng.normal(size=(s.n, 3))
    z, zp = e.sparse_precond(r, rp)
    oz, ozp = oracle.OracleSystem(s).sparse_precond(r, rp)
    assert rel_err(cpu(z), oz) < FIELD_RTOL
    assert rel_err(cpu(zp), ozp) < FIELD_RTOL


def test_fields_bit_reproducible(gpu_lib, tg):
    """Fixed-point accumulation: two evaluations are bit-identical."""
    s = tg.systems.make_config("water648")
    e = engine_for(s)
    a = cpu(e.dfield()[0])
    b = cpu(e.dfield()[0])
    print("dfield repeat max diff", np.abs(a - b).max(), "entries differing", int((a != b).sum()))
    assert np.array_equal(a, b)
    rng = np.random.default_rng(1)
    u = rng.normal(scale=0.05, size=(s.n, 3))
    c = cpu(e.ufield(u, u)[0])
    d = cpu(e.ufield(u, u)[0])
    assert np.array_equal(c, d)
