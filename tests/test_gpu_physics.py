"""Known answers of the wave physics through the CUDA path (FP32): body-wave travel times
in a homogeneous box, energy conservation with traction-free boundaries and energy
absorption by the PML, each also compared with the FP64 oracle's energy history."""
import numpy as np
import pytest

from ses3d_gb300 import synth

pytestmark = pytest.mark.gpu

ENERGY_BOX = dict(n_el=(6, 6, 4), colat=(44.0, 46.0), lon=(9.0, 11.0), r=(6171000.0, 6371000.0), nt=800, dt=0.05,
                  source_type=10, depth_m=60000.0, t0=3.0, sigma=1.0)


@pytest.mark.parametrize("source_type,comp,speed", [(1, 0, 4000.0), (2, 1, 4000.0), (3, 2, 7000.0)])
def test_body_wave_travel_times(native, source_type, comp, speed):
    """A force 150 km below a surface receiver (Gaussian in time, peak at 8 s): S arrival on
    the transverse component for a horizontal force, P arrival on the vertical one for a
    vertical force, within 1.5 s of 8 s + 150 km / speed."""
    from ses3d_gb300.solver import Simulation
    p = synth.homogeneous_problem(source_type=source_type)
    with Simulation.from_problem(p) as sim:
        sim.run()
        s = sim.seismograms(0)
    dt = float(p.events[0].event.dt)
    u = np.cumsum(s[comp][0].astype(np.float64)) * dt
    t_peak = np.argmax(np.abs(u)) * dt
    assert abs(t_peak - (8.0 + 150e3 / speed)) < 1.5, t_peak


@pytest.mark.parametrize("lean", [False, True])
def test_energy_conserved_without_pml_and_absorbed_with_pml(native, oracle_mod, wave_energy, lean):
    """Explosion at 60 km depth ending by 6 s: constant total energy with traction-free
    boundaries, non-increasing and mostly absorbed with PML; every sample within 1e-4 of
    the FP64 oracle's energy."""
    from ses3d_gb300.solver import Simulation
    series = {}
    for pml in (0, 2):
        p = synth.homogeneous_problem(pml=pml, **ENERGY_BOX)
        o = oracle_mod.Oracle(p, fp64=True)
        g, r = [], []
        with Simulation.from_problem(p) as sim:
            sim.set_lean(lean)
            for _ in range(20):                 # t = 2, 4, ..., 40 s
                sim.step(40)
                o.run(40)
                g.append(wave_energy(sim.field, sim.setup_real, p))
                r.append(wave_energy(o.get, o.get, p))
        g, r = np.array(g), np.array(r)
        assert np.all(np.abs(g - r) <= 1e-4 * r), (pml, np.max(np.abs(g - r) / r))
        series[pml] = g
    free, absorbed = series[0][3:], series[2][4:]
    assert free.max() - free.min() < 0.03 * free.mean(), free
    assert np.all(absorbed[1:] <= 1.005 * absorbed[:-1]), absorbed
    assert absorbed[-1] < 0.35 * series[2][3]
