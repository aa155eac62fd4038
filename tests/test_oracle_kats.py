"""Pins the oracle to the reference's own known-answer tests (tests/golden/reference_kats.json,
extracted from the reference's tests/simulation/*.cpp by tests/golden/make_reference_kats.py)."""
import json
import os

import numpy as np
import pytest

KATS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))


def test_angles_to_unit_vectors(orc):
    k = KATS["angles_to_unit_vectors"]
    out = orc.ref_angles_to_unit_vectors(k["deg"])
    np.testing.assert_allclose(out, np.array(k["expected"]), atol=k["tol"], rtol=0)


@pytest.mark.parametrize("case", range(2))
def test_repulsive_adhesion(orc, case):
    k = KATS["repulsive_adhesion"]
    c = k["cases"][case]
    out = orc.ref_repulsive_adhesion(k["k"], k["sigma"], c["dist"], k["r_adh"], k["k_adh"], c["dist_v"])
    np.testing.assert_allclose(out, c["expected"], atol=k["tol"], rtol=0)


def test_mean_angle(orc):
    k = KATS["mean_angle"]
    for c in k["cases"]:
        assert abs(orc.ref_mean_angle_deg(c["angles"]) - c["expected"]) < k["tol"]
    with pytest.raises(ValueError):
        orc.ref_mean_angle_deg([])


def test_symmetrize_min(orc):
    for c in KATS["symmetrize_min"]["cases"]:
        out = orc.ref_symmetrize_min(np.array(c["mat"]).reshape(3, 3))
        np.testing.assert_allclose(out.ravel(), c["expected"], rtol=1e-12, atol=0)


def test_dist_vect(orc):
    k = KATS["dist_vect"]
    for c in k["cases"]:
        r = np.array(c["r"]).reshape(-1, 2)
        n = len(r)
        dx, dy = orc.ref_dist_vect(r)
        np.testing.assert_allclose(dx.ravel(), c["dx"], atol=k["tol"], rtol=0)
        np.testing.assert_allclose(dy.ravel(), c["dy"], atol=k["tol"], rtol=0)
        assert dx.shape == (n, n)


def test_average_n(orc):
    """Fragile reference KAT: particles 2 and 4 carry 290 and 110 degrees, which cancel exactly,
    so the expected 21 rests on floating-point residue; the reference allows 2 degrees."""
    k = KATS["average_n"]
    out = orc.ref_average_n(np.array(k["dist_length"]).reshape(10, 10), k["n"], k["sigma"])
    assert np.all(np.abs(out - np.array(k["expected"])) <= k["tol"])


def test_seam_wrap_ref_form(orc):
    k = KATS["seam_wrap"]
    uo = np.array(k["uv_old"]).reshape(-1, 2)
    u = np.array(k["uv"]).reshape(-1, 2)
    out, n, _ = orc.ref_seam_wrap(uo, u, k["n"])
    np.testing.assert_allclose(out.ravel(), k["expected"], atol=k["tol"], rtol=0)
    # rotations: right then down = -90 - 270; right then right = -180; left = -90
    assert list(n) == [80 - 360, 120 - 180, 42 - 90]


def test_seam_wrap_model_form(orc):
    """The model wrap (first side crossed along the segment) reproduces the reference KAT."""
    k = KATS["seam_wrap"]
    uo = np.array(k["uv_old"]).reshape(-1, 2)
    u = np.array(k["uv"]).reshape(-1, 2)
    exp = np.array(k["expected"]).reshape(-1, 2)
    for i in range(3):
        e, th, v, nw, rc = orc.model_wrap(uo[i], u[i], np.deg2rad(k["n"][i]), (1.0, 0.0))
        assert rc == 0
        np.testing.assert_allclose(e, exp[i], atol=k["tol"])
        assert nw == [2, 2, 1][i]


def test_philox_published_vectors(orc):
    """Philox4x32-10 known answers (Random123 distribution, kat_vectors)."""
    assert [hex(x) for x in orc.philox4x32_10([0, 0, 0, 0], [0, 0])] == [
        "0x6627e8d5", "0xe169c58d", "0xbc57ac4c", "0x9b00dbd8"]
    assert [hex(x) for x in orc.philox4x32_10([0xffffffff] * 4, [0xffffffff] * 2)] == [
        "0x408f276d", "0x41c83b0e", "0xa20bc7c6", "0x6d5451fd"]
    assert [hex(x) for x in orc.philox4x32_10([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                                              [0xa4093822, 0x299f31d0])] == [
        "0xd16cfe09", "0x94fdcceb", "0x5001e420", "0x24126ea1"]


def test_model_force_is_negated_reference_force(orc):
    """The model's pair force magnitude is the reference's piecewise-linear formula with the
    physical sign (ForceHelper.cpp:84-104 pulls overlapping particles together)."""
    k = KATS["repulsive_adhesion"]
    c = k["cases"][0]
    ref = orc.ref_repulsive_adhesion(k["k"], k["sigma"], c["dist"], k["r_adh"], k["k_adh"], c["dist_v"])
    twoR = 2 * k["sigma"]
    model_mag = k["k"] * (twoR - c["dist"]) / twoR
    dv = np.array(c["dist_v"])
    np.testing.assert_allclose(-ref, model_mag * dv / c["dist"], rtol=1e-12)
