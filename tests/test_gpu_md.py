"""Molecular dynamics on the GPU (t9gb_md_*): two velocity-Verlet steps of
the TinkerNIST water/ion box from the reference's own restart file against
the positions and velocities it saved (Tinker9 test/tinkernist.cpp, every
atom), energy conservation without a thermostat, and the Bussi thermostat
pulling a cold box to its temperature."""
import numpy as np
import pytest

import tn_fixture as T
from gpu_util import engine_for

pytestmark = pytest.mark.gpu


def test_tinkernist_two_md_steps(gpu_lib):
    s, mass, v0, fx = T.md_system()
    m = fx["meta"]
    e = engine_for(s)
    e.md_init(s.xyz, mass, v0)
    box = np.asarray(m["box"])
    for frame in (0, 1):
        e.md_run(1, m["dt_ps"])
        x, v, _ = e.md_state()
        dx = x - fx["xyz"][frame]
        dx -= box * np.round(dx / box)  # the reference wraps molecules before saving
        dv = v - fx["vel"][frame]
        print(f"step {frame + 1}: positions max {np.abs(dx).max():.2e} A, velocities max {np.abs(dv).max():.2e} A/ps")
        assert np.abs(dx).max() < m["md_eps"]["xyz"]
        assert np.abs(dv).max() < m["md_eps"]["vel"]


def _potential(e):
    em = e.emplar(0x010)[0]
    return em + e.ehal(0x010)[0] + e.evalence(0x010)[0]


def test_nve_energy_conservation(gpu_lib, tg):
    s = tg.systems.make_config("water648", vdw=True, valence=True)
    mass = np.where(s.types == tg.systems.WATER_O, 15.999, 1.008)
    rng = np.random.default_rng(5)
    v0 = rng.normal(size=(s.n, 3)) * np.sqrt(0.0019872 * 298.0 * 418.4 / mass)[:, None]
    e = engine_for(s, predictor=1)
    e.md_init(s.xyz, mass, v0)
    ek0, _, _ = e.md_run(0, 0.0005)
    e0 = ek0 + _potential(e)
    ek, t, _ = e.md_run(200, 0.0005)
    e1 = ek + _potential(e)
    print(f"E0 {e0:.3f} E1 {e1:.3f} kinetic {ek:.3f} T {t:.1f} K")
    assert abs(e1 - e0) < 2e-3 * abs(ek)


def test_bussi_thermostat_heats_a_cold_box(gpu_lib, tg):
    s = tg.systems.make_config("water648", vdw=True, valence=True)
    mass = np.where(s.types == tg.systems.WATER_O, 15.999, 1.008)
    e = engine_for(s, predictor=1)
    e.md_init(s.xyz, mass, None)
    temps = [e.md_run(40, 0.001, thermostat=1, kelvin=298.0, tau_ps=0.01, seed=7)[1] for _ in range(5)]
    print("temperatures", [round(t, 1) for t in temps])
    assert 200.0 < np.mean(temps[2:]) < 400.0


def test_trajectory_recording_and_iteration_counts(gpu_lib, tg):
    """Frames copied on the device match the host state, and the step and
    PCG-iteration counters add up the solves of the steps."""
    import torch

    s = tg.systems.make_config("water648", vdw=True, valence=True)
    mass = np.where(s.types == tg.systems.WATER_O, 15.999, 1.008)
    e = engine_for(s, predictor=1)
    e.md_init(s.xyz, mass, None)
    frames = torch.zeros((3, s.n, 3), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()  # the engine copies on its own stream
    iters = 0
    for k in range(3):
        e.md_run(1, 0.001, thermostat=1, kelvin=298.0, tau_ps=0.1, seed=2)
        iters += e.stats()[0]
        e.md_positions_device(frames[k])
    x, _, _ = e.md_state()
    torch.cuda.synchronize()
    assert np.array_equal(frames[2].cpu().numpy(), x.astype(np.float32))
    assert not np.array_equal(frames[0].cpu().numpy(), frames[2].cpu().numpy())
    steps, its = e.md_stats()
    assert steps == 3 and its == iters and its > 0
