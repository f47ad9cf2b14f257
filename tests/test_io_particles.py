"""Formats around the shower path and PETITE's Particle utilities, on the CPU:
a shower file written by PETITE read without PETITE, beam files, bulk
conversion, and boost / two- and three-body decays / the meson decay chain /
energy loss / detector_cut against the reference's own outputs on the same
seeded numpy generator (tests/golden/make_golden.py, ``files`` and
``particles`` modes)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from petite_gb300 import io as pio
from petite_gb300.particle import Particle
from petite_gb300.shower import detector_cut

P = np.load(os.path.join(GOLDEN, "particles.npz"))
FILE = os.path.join(GOLDEN, "petite_shower_file.npy")
CONTENT = np.load(os.path.join(GOLDEN, "petite_shower_file_content.npz"))
KEYS = ("PID", "ID", "parent_PID", "parent_ID", "generation_number", "weight", "mass")


def test_reads_petite_shower_file_without_petite():
    parts = pio.read_particle_file(FILE)
    assert len(parts) == len(CONTENT["p0"]) > 100
    assert all(isinstance(p, Particle) for p in parts)
    a = pio.particles_to_arrays(parts)
    for k in ("p0", "r0", "pf", "rf"):
        np.testing.assert_array_equal(a[k], CONTENT[k])
    np.testing.assert_array_equal(np.c_[[a[k] for k in KEYS]].T.astype(float), CONTENT["ids"])
    assert list(a["generation_process"]) == list(CONTENT["process"])
    np.testing.assert_array_equal(a["ended"], CONTENT["ended"])


def test_particle_file_round_trip(tmp_path):
    parts = pio.read_particle_file(FILE)
    path = tmp_path / "again.npy"
    pio.save_particle_file(path, parts)
    back = pio.read_particle_file(path)
    a, b = pio.particles_to_arrays(parts), pio.particles_to_arrays(back)
    for k in a:
        assert np.array_equal(a[k], b[k]) if a[k].dtype != object else list(a[k]) == list(b[k])


def test_arrays_round_trip():
    parts = pio.read_particle_file(FILE)
    a = pio.particles_to_arrays(parts)
    b = pio.particles_to_arrays(pio.arrays_to_particles(a))
    for k in a:
        assert np.array_equal(a[k], b[k]) if a[k].dtype != object else list(a[k]) == list(b[k])


def test_load_beam():
    p4 = np.array([[0.6, 0.1, 0.2, 0.5], [2.0, 0.0, 0.0, 1.9952]])
    parts = pio.load_beam(p4, pid=111)
    assert [p.get_ids()["ID"] for p in parts] == [1, 2]
    assert [p.get_ids()["weight"] for p in parts] == [0.5, 0.5]
    m = parts[0].get_ids()["mass"]
    assert m == round(np.sqrt(round(0.36 - 0.01 - 0.04 - 0.25, 12)), 6)
    with pytest.raises(ValueError):
        pio.load_beam(np.zeros((3, 3)), pid=111)


def _particle(row):
    pid, m = int(row[0]), row[1]
    return Particle(list(row[4:8]), [0.0, 0.0, 0.0], {"PID": pid, "mass": m})


def test_two_body_decay_and_boost_match_reference():
    for case, row in enumerate(P["decays"]):
        pid, m, seed, mv = int(row[0]), row[1], int(row[2]), row[3]
        par = Particle(list(row[4:8]), [0.0, 0.0, 0.1 * case], {"PID": pid, "mass": m, "ID": 3 + case})
        np.random.seed(seed)
        a, b = par.two_body_decay({"mass": 0, "PID": 22}, {"mass": mv, "PID": 4900022})
        scale = row[4]
        np.testing.assert_allclose(a.get_p0(), row[8:12], rtol=0, atol=1e-13 * scale)
        np.testing.assert_allclose(b.get_p0(), row[12:16], rtol=0, atol=1e-13 * scale)
        np.testing.assert_allclose(np.array(par.boost_matrix()).ravel(), row[16:32], rtol=1e-14, atol=1e-14)
        assert list(b.get_r0()) == [0.0, 0.0, 0.1 * case]


def test_three_body_decay_matches_reference():
    n = 0
    for row in P["decays"]:
        pid, m, seed = int(row[0]), row[1], int(row[2])
        if not m > 3 * 0.1349768:
            continue
        par = _particle(row)
        par.set_ids({"PID": pid, "mass": m})
        np.random.seed(seed + 1)
        x = par.three_body_decay({"PID": 22, "mass": 0.0}, {"PID": 22, "mass": 0.0}, {"PID": 111})
        got = np.concatenate([q.get_p0() for q in x])
        np.testing.assert_allclose(got, row[32:44], rtol=0, atol=1e-12 * row[4])
        n += 1
    assert n >= 10


def test_meson_decay_chain_matches_reference():
    n = 0
    for row in P["decays"]:
        pid, m, seed = int(row[0]), row[1], int(row[2])
        want = row[44:56]
        st = "short-lived" if pid in (111, 221, 331, 223) else "long-lived"
        q = Particle(list(row[4:8]), [0.0, 0.0, 0.0], {"PID": pid, "mass": m, "ID": 5, "stability": st,
                                                        "weight": 0.5})
        np.random.seed(seed + 2)
        if np.isnan(want).all():
            with pytest.raises(ValueError):            # a three-body mode drawn, or no decay listed
                q.decay_particle()
            continue
        dd = q.decay_particle()
        got = np.concatenate([dd[0].get_p0(), dd[1].get_p0(), [dd[0].get_ids()["weight"], dd[1].get_ids()["weight"],
                              dd[0].get_ids()["PID"], dd[1].get_ids()["PID"]]])
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-13 * row[4])
        np.testing.assert_allclose(q.get_rf(), row[56:59], rtol=1e-13, atol=0)
        assert [d.get_ids()["ID"] for d in dd] == [10, 11] and q.get_ended()
        n += 1
    assert n >= 20


def test_stable_particle_has_no_decay():
    q = Particle([1.0, 0.0, 0.0, 0.99], [0, 0, 0], {"PID": 111, "mass": 0.1349768})
    with pytest.raises(UnboundLocalError):
        q.decay_particle()


def test_lose_energy_matches_reference():
    for m, E, dE, dx, dy, dz, *pf in P["lose"]:
        par = Particle([E, *(np.sqrt(E * E - m * m) * np.array([dx, dy, dz]))], [0, 0, 0], {"PID": 11, "mass": m})
        par.lose_energy(dE)
        np.testing.assert_allclose(par.get_pf(), pf, rtol=1e-14, atol=1e-15)


def test_detector_cut_matches_reference():
    parts = [Particle(list(p4), list(r0), {"PID": 4900022, "weight": w, "mass": 0.01})
             for p4, r0, w in zip(P["det/p0"], P["det/r0"], P["det/w"])]
    zs, R = [5.0, 50.0, 100.0], 1.0
    np.testing.assert_array_equal(detector_cut(parts, zs, R, method="SampleW"), P["det/sampleW"])
    np.testing.assert_allclose(detector_cut(parts, zs, R, method="Efficiency", energy_cut=(1.0, 20.0),
                                            detector_inner_radius=0.05), P["det/eff"], rtol=1e-12)
    np.testing.assert_allclose(detector_cut(parts, zs, R, method="TotalWeight"), P["det/total"], rtol=1e-12)
    s = detector_cut(parts, zs, R, method="Sample")
    assert [len(x) for x in s] == list(P["det/sampleW"].sum(axis=1))
    assert detector_cut([], zs, R, method="Efficiency") == [0.0, 0.0, 0.0]
