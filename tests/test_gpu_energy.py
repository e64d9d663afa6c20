"""CUDA multipole and polarization energies against the FP64 oracle and the
reference's known answers.  Tolerances: relative 1e-6 of the magnitude (FP32
pair and spline arithmetic, FP64 accumulation) and the reference tests'
absolute margins for the golden values."""
import numpy as np
import pytest

import lf_fixture as L
from gpu_util import engine_for

pytestmark = pytest.mark.gpu
REL_E = 1.0e-6


def test_localframe_empole_nonewald(gpu_lib):
    s, fx = L.system(0)
    e, _ = engine_for(s).empole_energy()
    assert abs(e - fx["expected"]["Local-Frame-1"]["empole -- gas phase, no cutoff"]["ref_eng"]) < 1e-4


def test_localframe_empole_pme_parts(gpu_lib):
    s, fx = L.system(1)
    e, parts = engine_for(s).empole_energy()
    ex = fx["expected"]["Local-Frame-2"]["empole -- pme"]
    print("gpu parts", parts, "reference", ex["ref_ereal"], ex["ref_erecip"], ex["ref_eself"])
    assert abs(parts[0] - ex["ref_ereal"]) < 1e-3
    assert abs(parts[1] - ex["ref_erecip"]) < 1e-3
    assert abs(parts[2] - ex["ref_eself"]) < 1e-3
    assert abs(e - (ex["ref_ereal"] + ex["ref_erecip"] + ex["ref_eself"])) < 1e-3


@pytest.mark.parametrize("ewald", [0, 1], ids=["nonewald", "pme"])
def test_localframe_epolar(gpu_lib, ewald):
    s, fx = L.system(ewald)
    e = engine_for(s)
    e.induce()
    assert abs(e.epolar_energy() - L.expected(fx, ewald)["epolar"]["ref_eng"]) < 1e-4


@pytest.mark.parametrize("name", ["water648", "nacl23142"])
def test_water_energies(gpu_lib, oracle, name, tg):
    s = tg.systems.make_config(name)
    e = engine_for(s)
    o = oracle.OracleSystem(s)
    em, parts = e.empole_energy()
    oem, oparts = o.empole_energy()
    print(name, "empole gpu", em, parts, "oracle", oem, oparts, "rel", abs(em - oem) / abs(oem))
    assert abs(em - oem) < REL_E * max(abs(oparts).max(), abs(oem))
    e.induce()
    ep = e.epolar_energy()
    oep = o.epolar_energy()
    print(name, "epolar gpu", ep, "oracle", oep, "rel", abs(ep - oep) / abs(oep))
    assert abs(ep - oep) < REL_E * abs(oep)
