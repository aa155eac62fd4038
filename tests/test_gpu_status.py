"""The device status word (the reference's Validation, Validation.cpp:40-72: exit(1) on non-finite
values, a throw on a lost particle) bit by bit, each failure made on the host -- no kernel is made to
fault: a state or parameter set that forces the condition. Each bit makes tds_step return
TDS_ERR_STATE, tds_clear_status clears it, and the handle keeps working afterwards."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WRAP, LOCATE, CELL = 2, 4, 16


def _sim(tg, mesh, n=300, precision=32, **kw):
    sim = tg.Simulation(mesh, tg.Params(**kw), n, seed=3, precision=precision)
    sim.start()
    sim.step(2)
    return sim


def _still_usable(tg, sim, good):
    """After the status is cleared and a valid state is loaded, steps run clean."""
    sim.clear_status()
    assert sim.status() == 0
    sim.set_state(good["uv"], good["theta"], good["face"])
    sim.step(3)
    assert sim.status() == 0


@pytest.mark.parametrize("precision", [32, 64])
def test_wrap_limit(tg, mesh_l4, precision):
    """v0 dt of ~200 chart diameters: the advance crosses the square's border far more than the
    8 wraps a step allows; the position is clamped and bit 2 is set."""
    sim = _sim(tg, mesh_l4, precision=precision)
    good = sim.get_state()
    sim.set_params(tg.Params(v0=1e4))
    with pytest.raises(tg.TdsError) as e:
        sim.step(1)
    assert e.value.code == 4 and "wrap" in str(e.value)
    assert sim.status() & WRAP
    s = sim.get_state()
    assert np.isfinite(s["uv"]).all()
    sim.clear_status()  # a set status is reported by every synchronising call until cleared
    sim.set_params(tg.Params())
    _still_usable(tg, sim, good)


@pytest.mark.parametrize("precision", [32, 64])
def test_locate_fallback(tg, mesh_l4, precision):
    """A chart point outside the unit square, loaded without a face: no face contains it, the
    nearest face is taken and bit 4 is set by the load; the next step reports it."""
    sim = _sim(tg, mesh_l4, precision=precision)
    s = good = sim.get_state()
    uv = s["uv"].copy()
    uv[5] = (1.25, 0.5)
    sim.set_state(uv, s["theta"])  # faces located on the device
    assert sim.status() & LOCATE
    with pytest.raises(tg.TdsError) as e:
        sim.step(1)
    assert e.value.code == 4
    _still_usable(tg, sim, good)


@pytest.mark.parametrize("precision", [32, 64])
def test_particle_outside_the_surface_cells(tg, mesh_l4, precision):
    """A 3D position given far off the surface: the particle is in no surface cell (the reference's
    lost particle); bit 16 is set by the load and the next step reports it. The step maps the
    particle back onto its face, so after a clear the system steps clean."""
    sim = _sim(tg, mesh_l4, precision=precision)
    s = good = sim.get_state()
    r3 = s["r3d"].copy()
    r3[11] = (40.0, -40.0, 40.0)
    sim.set_state(s["uv"], s["theta"], s["face"], r3)
    assert sim.status() & CELL
    with pytest.raises(tg.TdsError) as e:
        sim.step(1)
    assert e.value.code == 4 and "surface cells" in str(e.value)
    sim.clear_status()
    sim.step(2)
    assert sim.status() == 0
    after = sim.get_state()
    assert np.abs(after["r3d"][11]).max() < 3.0
    _still_usable(tg, sim, good)


def test_status_bits_of_an_ensemble(tg, mesh_l4):
    """The word is per handle: a lost particle in one replica of an ensemble is reported."""
    sim = tg.Simulation(mesh_l4, [tg.Params(), tg.Params(v0=0.5)], [120, 80], seed=2)
    sim.start()
    s = good = sim.get_state()
    r3 = s["r3d"].copy()
    r3[150] = (30.0, 30.0, 30.0)
    sim.set_state(s["uv"], s["theta"], s["face"], r3)
    with pytest.raises(tg.TdsError):
        sim.step(1)
    assert sim.status() & CELL
    _still_usable(tg, sim, good)
