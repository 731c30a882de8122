"""Seeded synthetic workloads are deterministic and have the stated shapes."""
import numpy as np

from gauxc_gb300 import workloads as W


def test_config0_single_water():
    c = W.config(0)
    s = c["systems"][0]
    assert s["nbf"] == 60 and s["n_water"] == 1 and s["functional"] == "SVWN5"
    assert s["P"].shape == (60, 60) and np.allclose(s["P"], s["P"].T)
    assert np.linalg.matrix_rank(s["P"]) == 5


def test_configs_deterministic_and_placement_rule():
    a = W.config(1)["systems"][0]
    b = W.config(1)["systems"][0]
    assert a["atoms"] == b["atoms"] and np.array_equal(a["P"], b["P"])
    assert a["nbf"] == 1920
    O = np.array([x[1:] for x in a["atoms"] if x[0] == 8]) / W.BOHR_PER_ANG
    d = np.linalg.norm(O[:, None] - O[None], axis=-1) + np.eye(len(O)) * 99
    assert d.min() >= 2.6
    assert O.min() >= 0.0 and O.max() <= 10.0


def test_config3_batched_mix():
    c = W.config(3)
    assert len(c["systems"]) == 64
    funcs = [s["functional"] for s in c["systems"]]
    assert funcs.count("SVWN5") == 32 and funcs.count("PBE") == 32
    assert all(1 <= s["n_water"] <= 40 for s in c["systems"])
    assert all(s["batch_size"] in (128, 256, 512, 1024) for s in c["systems"])


def test_water_geometry():
    at = W.water_cluster(1, 0.0, np.random.default_rng(0))
    O, H1, H2 = (np.array(a[1:]) / W.BOHR_PER_ANG for a in at)
    assert np.isclose(np.linalg.norm(H1 - O), np.hypot(0.757, 0.587))
    assert np.isclose(np.linalg.norm(H2 - O), np.hypot(0.757, 0.587))
