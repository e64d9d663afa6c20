"""Molecular dynamics from Tinker files: the job of Tinker's `dynamic`
program for the force field this library carries (AMOEBA multipoles and
polarization, buffered 14-7 van der Waals, bond / angle / Urey-Bradley),
on the GPU through the C ABI.

    out = run("water30.xyz", nsteps=1000, dt_fs=1.0, save_every=100,
              kelvin=298.0, tau_ps=0.1, arc="water30.arc", dyn_out="water30.dyn")

The .key beside the .xyz and the parameter file it names supply the force
field and settings (tinkerio.system_from_tinker).  Each saved frame appends
to the .arc trajectory and, when asked, the induced dipoles of the frame's
solve to .uind (Debye); the restart (.dyn) is written at the end.  A restart
given as dyn_in supplies the starting positions and velocities, as Tinker
reads water30.dyn in its TinkerNIST test (test/tinkernist.cpp:195-365); else
kelvin seeds Maxwell-Boltzmann velocities.  The reference's driver is
src/xdynamic.cpp around src/md/integrator.cpp:70-190.
"""
import importlib

import numpy as np

from . import tinkerio as tio
from . import units

GASCONST = 1.987204259e-3  # kcal/mol/K
EKCAL = 418.4  # (g/mol) (A/ps)^2 -> kcal/mol


def maxwell_velocities(mass, kelvin, seed=1):
    """Seeded Maxwell-Boltzmann velocities (A/ps) at the given temperature."""
    rng = np.random.default_rng(seed)
    return rng.normal(size=(len(mass), 3)) * np.sqrt(GASCONST * kelvin * EKCAL / np.asarray(mass))[:, None]


def run(xyz, key=None, prm=None, nsteps=1000, dt_fs=1.0, save_every=0, kelvin=None, tau_ps=0.1, seed=1,
        dyn_in=None, arc=None, dyn_out=None, uind_out=None, predictor=None, extrapolation=0, stream=None):
    """Integrate nsteps velocity-Verlet steps of dt_fs: Bussi thermostat at
    kelvin with coupling tau_ps when kelvin is given, else NVE.  predictor:
    0 none, 1 ASPC, 2 Gear; None takes the keyword file's POLAR-PREDICT
    (tinkerio.predictor_from_keys).  extrapolation: frames of the learned
    extrapolation of the predictor ring (t9gb_learn_extrapolation, 2-8 with
    ASPC, 2-5 with Gear), 0 off.
    Returns the steps done, the final kinetic energy (kcal/mol), temperature
    (K), positions (A) and velocities (A/ps)."""
    abi = importlib.import_module(__package__ + ".abi")
    key, prm = tio.resolve_files(xyz, key, prm)
    s = tio.system_from_tinker(xyz, key, prm)
    fr = tio.read_xyz(xyz)[0]
    mass = tio.masses(s.types, tio.read_prm(prm))
    x0, v0 = s.xyz, None
    if dyn_in is not None:
        x0, v0, _, _, _ = tio.read_dyn(dyn_in)
    elif kelvin is not None:
        v0 = maxwell_velocities(mass, kelvin, seed)
    if predictor is None:
        predictor = s.settings.get("predictor", 0)
    eng = abi.Engine(s, predictor=predictor, stream=stream)
    eng.prepare(x0)
    if extrapolation:
        eng.learn_extrapolation(extrapolation)
    eng.md_init(x0, mass, v0)
    dt = dt_fs * 1e-3
    thermo = 1 if kelvin is not None else 0
    T = 298.0 if kelvin is None else float(kelvin)
    chunk = save_every if save_every > 0 else nsteps
    done, ek, temp = 0, 0.0, 0.0
    while done < nsteps:
        k = min(chunk, nsteps - done)
        ek, temp, rc = eng.md_run(k, dt, thermostat=thermo, kelvin=T, tau_ps=tau_ps, seed=seed)
        if rc != 0:
            eng.close()
            raise RuntimeError(f"the dipole solve failed (status {rc}) within steps {done + 1}-{done + k}")
        if save_every > 0:
            x, _, _ = eng.md_state()
            frame = tio.Frame(fr.title, fr.names, x, fr.types, fr.bonds, fr.box)
            if arc:
                tio.write_xyz(arc, frame, append=done > 0)
            if uind_out:
                ud, _ = eng.uind()
                tio.write_dipoles(uind_out, frame, ud.double().cpu().numpy() * units.DEBYE, append=done > 0)
        done += k
    x, v, _ = eng.md_state()
    if dyn_out:
        tio.write_dyn(dyn_out, fr.title, x, v, box=None if s.box is None else tuple(s.box))
    eng.close()
    return {"steps": done, "kinetic_kcal": ek, "temperature_k": temp, "xyz": x, "vel": v}
