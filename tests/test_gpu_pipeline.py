"""Pipelined state transfer (tds_set_state_async / tds_get_state_async / tds_sync): the same
states as the synchronous calls, step by step, with the upload of step k+1 in flight while step k
downloads."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _out(n):
    return dict(uv=np.zeros((n, 2)), theta=np.zeros(n), face=np.zeros(n, np.int32), r3d=np.zeros((n, 3)),
                vel_uv=np.zeros((n, 2)), nbr=np.zeros(n, np.int32))


def _inputs(tg, mesh, n, precision, k):
    a = tg.Simulation(mesh, tg.Params(), n, seed=11, precision=precision)
    a.start()
    ins = []
    for _ in range(k):
        a.step(1)
        s = a.get_state()
        ins.append({key: s[key].copy() for key in ("uv", "theta", "face", "r3d")})
    a.close()
    return ins


@pytest.mark.parametrize("precision", [32, 64])
def test_pipelined_transfers_match_synchronous(tg, mesh_l4, precision):
    n = 2000
    ins = _inputs(tg, mesh_l4, n, precision, 4)
    ref = tg.Simulation(mesh_l4, tg.Params(), n, seed=3, precision=precision)
    expect = []
    for x in ins:
        ref.set_state(**x)
        ref.step(1)
        expect.append(ref.get_state())
    sim = tg.Simulation(mesh_l4, tg.Params(), n, seed=3, precision=precision)
    outs = [_out(n) for _ in ins]
    for x, o in zip(ins, outs):
        sim.set_state_async(**x)
        sim.step_async(1)
        sim.get_state_async(o)
    sim.sync()
    for e, o in zip(expect, outs):
        for key in e:
            np.testing.assert_array_equal(e[key], o[key])
    # a synchronous read after the pipelined calls sees the last state
    last = sim.get_state()
    for key in last:
        np.testing.assert_array_equal(last[key], outs[-1][key])


@pytest.mark.parametrize("kind", ["single", "ensemble"])
@pytest.mark.parametrize("use_async", [False, True])
def test_a_load_with_bad_faces_is_refused_and_changes_nothing(tg, mesh_l4, use_async, kind):
    """Face indices are checked on the device: a load with an index >= F is refused as a whole,
    reported by tds_set_state itself or by the next tds_sync, and leaves the state, the cell lists
    and the steps after it exactly as if the load had not been asked for -- on a plain system and
    on a 3-replica ensemble, after an odd number of steps (the per-tile counts and the step counter
    have advanced past their initial parity)."""
    if kind == "single":
        n, ps = 500, tg.Params()
    else:
        n, ps = [200, 137, 163], [tg.Params(eta=0.2), tg.Params(v0=1.3), tg.Params(eta=1.0, v0=0.7)]
    total = int(np.sum(n))
    (x,) = _inputs(tg, mesh_l4, total, 32, 1)
    sim = tg.Simulation(mesh_l4, ps, n, seed=1)
    ref = tg.Simulation(mesh_l4, ps, n, seed=1)
    sim.set_state(**x)
    ref.set_state(**x)
    sim.step(3)
    ref.step(3)
    before = sim.get_state()
    bad = dict(x)
    bad["face"] = x["face"].copy()
    bad["face"][7] = mesh_l4.F
    bad["uv"] = x["uv"][::-1].copy()
    if use_async:
        sim.set_state_async(**bad)  # enqueued; refused on the device
        with pytest.raises(tg.TdsError) as e:
            sim.sync()
    else:
        with pytest.raises(tg.TdsError) as e:
            sim.set_state(**bad)
    assert e.value.code == 1 and "face index out of range" in str(e.value)
    sim.sync()  # reported once
    after = sim.get_state()
    for key in before:
        np.testing.assert_array_equal(before[key], after[key])
    sim.step(3)
    ref.step(3)
    a, b = sim.get_state(), ref.get_state()
    for key in a:
        np.testing.assert_array_equal(a[key], b[key])
    np.testing.assert_array_equal(sim.order_parameter()[0], ref.order_parameter()[0])


def test_get_state_async_checks_output_arrays(tg, mesh_l4):
    sim = tg.Simulation(mesh_l4, tg.Params(), 100, seed=1)
    sim.start()
    o = _out(100)
    o["uv"] = np.zeros((100, 2), np.float32)
    with pytest.raises(ValueError):
        sim.get_state_async(o)


@pytest.mark.parametrize("precision", [32, 64])
def test_state_without_r3d_is_the_same_state(tg, mesh_l4, precision):
    """The 3D position is the face's chart map of the chart position: a state given as (uv, theta,
    face) alone loads to the same device state, bit for bit, as one given with r3d, and the next
    steps agree exactly (the end-to-end bench uploads the state that way)."""
    n = 1500
    (x,) = _inputs(tg, mesh_l4, n, precision, 1)
    a = tg.Simulation(mesh_l4, tg.Params(), n, seed=5, precision=precision)
    b = tg.Simulation(mesh_l4, tg.Params(), n, seed=5, precision=precision)
    a.set_state(**x)
    b.set_state(x["uv"], x["theta"], x["face"])
    sa, sb = a.get_state(), b.get_state()
    np.testing.assert_array_equal(sa["r3d"], sb["r3d"])
    a.step(3)
    b.step(3)
    sa, sb = a.get_state(), b.get_state()
    for key in sa:
        np.testing.assert_array_equal(sa[key], sb[key])


@pytest.mark.parametrize("precision", [32, 64])
def test_particle_records_match_the_state(tg, mesh_l4, precision):
    """tds_get_particles packs the reference's Particle records on the device: the same values as
    the state arrays, the angle in degrees as (theta * 180) / pi, the compass fields 0."""
    sim = tg.Simulation(mesh_l4, tg.Params(), 700, seed=9, precision=precision)
    sim.start()
    sim.step(4)
    st = sim.get_state()
    pk = sim.get_particles()
    assert pk.dtype.itemsize == 88
    np.testing.assert_array_equal(pk["x_UV"], st["uv"][:, 0])
    np.testing.assert_array_equal(pk["y_UV"], st["uv"][:, 1])
    np.testing.assert_array_equal(pk["x_velocity_UV"], st["vel_uv"][:, 0])
    np.testing.assert_array_equal(pk["y_velocity_UV"], st["vel_uv"][:, 1])
    np.testing.assert_array_equal(pk["alignment_UV"], st["theta"] * 180.0 / np.pi)
    np.testing.assert_array_equal(pk["x_3D"], st["r3d"][:, 0])
    np.testing.assert_array_equal(pk["z_3D"], st["r3d"][:, 2])
    np.testing.assert_array_equal(pk["neighbor_count"], st["nbr"])
    assert not pk["compass_north_pole_UV"].any() and not pk["compass_south_pole_UV"].any()


def _out32(n):
    return dict(uv=np.zeros((n, 2), np.float32), theta=np.zeros(n, np.float32), face=np.zeros(n, np.int32),
                r3d=np.zeros((n, 3), np.float32), vel_uv=np.zeros((n, 2), np.float32), nbr=np.zeros(n, np.int32))


def test_fp32_views_are_the_device_state(tg, mesh_l4):
    """tds_get_state_f32 returns an FP32 handle's state as it is on the device: the double view's
    values are exactly these, widened. A state set through tds_set_state_f32 is the state set from
    the same values as doubles, and the steps after it agree bit for bit."""
    n = 1500
    (x,) = _inputs(tg, mesh_l4, n, 32, 1)
    a = tg.Simulation(mesh_l4, tg.Params(), n, seed=4, precision=32)
    a.set_state(**x)
    a.step(2)
    d, f = a.get_state(), a.get_state(dtype=np.float32)
    for key in ("uv", "theta", "r3d", "vel_uv"):
        assert f[key].dtype == np.float32
        np.testing.assert_array_equal(f[key].astype(np.float64), d[key])
    for key in ("face", "nbr"):
        np.testing.assert_array_equal(f[key], d[key])
    b = tg.Simulation(mesh_l4, tg.Params(), n, seed=4, precision=32)
    c = tg.Simulation(mesh_l4, tg.Params(), n, seed=4, precision=32)
    b.set_state(f["uv"], f["theta"], f["face"])
    c.set_state(f["uv"].astype(np.float64), f["theta"].astype(np.float64), f["face"])
    for _ in range(2):
        sb, sc = b.get_state(), c.get_state()
        for key in sb:
            np.testing.assert_array_equal(sb[key], sc[key])
        b.step(3)
        c.step(3)


def test_fp32_views_pipelined_match_synchronous(tg, mesh_l4):
    n = 2000
    ins = _inputs(tg, mesh_l4, n, 32, 4)
    ins32 = [dict(uv=x["uv"].astype(np.float32), theta=x["theta"].astype(np.float32), face=x["face"]) for x in ins]
    ref = tg.Simulation(mesh_l4, tg.Params(), n, seed=3, precision=32)
    expect = []
    for x in ins32:
        ref.set_state(x["uv"].astype(np.float64), x["theta"].astype(np.float64), x["face"])
        ref.step(1)
        expect.append(ref.get_state())
    sim = tg.Simulation(mesh_l4, tg.Params(), n, seed=3, precision=32)
    outs = [_out32(n) for _ in ins32]
    for x, o in zip(ins32, outs):
        sim.set_state_async(**x)
        sim.step_async(1)
        sim.get_state_async(o)
    sim.sync()
    for e, o in zip(expect, outs):
        for key in e:
            np.testing.assert_array_equal(e[key], o[key].astype(e[key].dtype))


def test_fp32_views_need_an_fp32_handle(tg, mesh_l4):
    n = 200
    sim = tg.Simulation(mesh_l4, tg.Params(), n, seed=1, precision=64)
    sim.start()
    with pytest.raises(tg.TdsError) as e:
        sim.get_state(dtype=np.float32)
    assert e.value.code == 1
    with pytest.raises(tg.TdsError) as e:
        sim.set_state(np.full((n, 2), 0.5, np.float32), np.zeros(n, np.float32))
    assert e.value.code == 1
    with pytest.raises(tg.TdsError):
        sim.get_state_async(_out32(n))
    # mixed float types in one output set are refused before anything is enqueued
    o = _out32(n)
    o["theta"] = np.zeros(n)
    with pytest.raises(ValueError):
        sim.get_state_async(o)
    sim.sync()


@pytest.mark.parametrize("kind", ["single", "ensemble"])
def test_a_load_gives_the_same_steps_whatever_the_current_order(tg, mesh_l4, kind):
    """A state load fills each slot with the particle it holds in the handle's current order; the
    next step's counting sort orders the particles by cell and id, so the steps after a load are the
    same, bit for bit, on a fresh handle (identity order) and on one whose order many steps have
    scrambled. (No noise: the two handles' step counters differ, and the noise follows the counter.)"""
    if kind == "single":
        n, ps = 700, tg.Params(eta=0.0)
    else:
        n, ps = [300, 250, 150], [tg.Params(eta=0.0), tg.Params(eta=0.0, v0=1.2), tg.Params(eta=0.0, v0=0.8)]
    total = int(np.sum(n))
    (x,) = _inputs(tg, mesh_l4, total, 32, 1)
    fresh = tg.Simulation(mesh_l4, ps, n, seed=2)
    used = tg.Simulation(mesh_l4, ps, n, seed=2)
    used.start()
    used.step(23)
    fresh.set_state(**x)
    used.set_state(**x)
    a0, b0 = fresh.get_state(), used.get_state()
    for key in a0:
        np.testing.assert_array_equal(a0[key], b0[key])
    fresh.step(5)
    used.step(5)
    a, b = fresh.get_state(), used.get_state()
    for key in a:
        np.testing.assert_array_equal(a[key], b[key])
