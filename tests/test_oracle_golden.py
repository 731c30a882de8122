"""The oracle against the reference's own golden vectors (no GPU needed).

Goldens: tests/ref_data/benzene_weights_ssf.hdf5 (SSF), water_cc-pVDZ_collocation.hdf5
(collocation), benzene_{svwn5,pbe0}_cc-pvdz_ufg_ssf*.hdf5 (EXC / VXC), the
cc-pVDZ G94 file (normalization); extracted by tests/golden/make_fixtures.py.
Tolerances are tighter than the reference's own tests (tests/xc_integrator.cxx:
EXC rel 1.2e-5, ||dVXC||_F / nbf < 1e-10).
"""
import numpy as np
import pytest

import oracle
from conftest import golden
from helpers import benzene_system, oracle_exc_vxc


def water_basis_raw():
    """Water cc-pVDZ as tests/standards.cxx builds it: s and p shells cartesian."""
    raw = golden("ccpvdz_raw.npz")
    c = golden("water_collocation.npz")
    ls, pures, nps, al, co, org = [], [], [], [], [], []
    for Z, x in zip(c["Z"], c["xyz"]):
        sym = {1: "H", 8: "O"}[int(Z)]
        for k in range(len(raw[sym + "_l"])):
            n = int(raw[sym + "_nprim"][k])
            l = int(raw[sym + "_l"][k])
            ls.append(l)
            pures.append(1 if l > 1 else 0)
            nps.append(n)
            a = np.zeros(32)
            a[:n] = raw[sym + "_alpha"][k, :n]
            cc = np.zeros(32)
            cc[:n] = oracle.normalize_shell(l, raw[sym + "_alpha"][k, :n], raw[sym + "_coeff"][k, :n])
            al.append(a)
            co.append(cc)
            org.append(x)
    return oracle.Basis(ls, pures, nps, np.array(al), np.array(co), np.array(org)), c


def test_ssf_weights_oracle_matches_golden():
    d = golden("benzene_weights_ssf.npz")
    w = oracle.ssf_weights(d["points"], d["iparent"], d["dist_nearest"], d["xyz"], d["w_unm"])
    np.testing.assert_allclose(w, d["w_mod"], rtol=1e-13, atol=0)


def test_normalization_oracle_matches_golden():
    raw = golden("ccpvdz_raw.npz")
    b = golden("benzene_svwn5.npz")
    # benzene basis: C atoms first (6 shells each), then H (3 shells each)
    for k in range(6):
        n = raw["C_nprim"][k]
        c = oracle.normalize_shell(int(raw["C_l"][k]), raw["C_alpha"][k, :n], raw["C_coeff"][k, :n])
        np.testing.assert_allclose(c, b["sh_coeff"][k, :n], rtol=1e-14)
    for k in range(3):
        n = raw["H_nprim"][k]
        c = oracle.normalize_shell(int(raw["H_l"][k]), raw["H_alpha"][k, :n], raw["H_coeff"][k, :n])
        np.testing.assert_allclose(c, b["sh_coeff"][36 + k, :n], rtol=1e-14)


def test_collocation_oracle_matches_golden():
    B, c = water_basis_raw()
    for i in range(int(c["nentries"][0])):
        f, fx, fy, fz = oracle.collocation(B, c[f"pts_{i}"], c[f"mask_{i}"], grad=True)
        for got, key in ((f, "eval"), (fx, "deval_x"), (fy, "deval_y"), (fz, "deval_z")):
            ref = c[f"{key}_{i}"].reshape(got.shape)
            assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("fname,func,prune", [
    ("benzene_svwn5.npz", "SVWN5", "Unpruned"),
    ("benzene_svwn5_treutler.npz", "SVWN5", "Treutler"),
    ("benzene_pbe0.npz", "PBE0", "Unpruned"),
])
def test_exc_vxc_oracle_matches_golden(g, fname, func, prune):
    d, mol, basis, mg, lb = benzene_system(g, fname, prune=prune, device=False)
    exc, V, nel = oracle_exc_vxc(basis, mol, lb, d["P"], func)
    nbf = V.shape[0]
    assert abs(exc - d["EXC"][0]) <= 1e-10
    assert np.linalg.norm(V - d["VXC"]) / nbf <= 1e-12
    # benzene has 42 electrons; P is the alpha density, rho = 2 phi^T P phi
    assert abs(nel - 42.0) < 1e-4


def test_functional_derivatives_finite_difference():
    rho = np.array([1e-6, 1e-3, 0.05, 0.3, 2.0, 40.0])
    sig = np.array([1e-12, 1e-6, 1e-3, 0.2, 3.0, 900.0])
    for name in ("SVWN5", "PBE"):
        e0, vr, vs = oracle.functional(name, rho, sig)
        h = 1e-6 * rho
        ep, _, _ = oracle.functional(name, rho + h, sig)
        em, _, _ = oracle.functional(name, rho - h, sig)
        dr = ((rho + h) * ep - (rho - h) * em) / (2 * h)
        np.testing.assert_allclose(vr, dr, rtol=1e-6)
        if name == "PBE":
            hs = 1e-6 * sig
            ep, _, _ = oracle.functional(name, rho, sig + hs)
            em, _, _ = oracle.functional(name, rho, sig - hs)
            ds = rho * (ep - em) / (2 * hs)
            np.testing.assert_allclose(vs, ds, rtol=1e-4, atol=1e-14)


def test_uks_svwn5_matches_golden():
    """UKS (cytosine doublet, SVWN5, cc-pVDZ, UltraFine, Robust pruning, tol = eps;
    tests/xc_integrator.cxx:455-458): oracle with its own SSF weights.  The
    reference's tolerance: EXC rel 1.2e-5, ||dVXC||_F / nbf < 1e-10."""
    import gauxc_gb300 as g
    from helpers import oracle_basis, oracle_ssf_tasks
    d, mol, basis, mg, lb = benzene_system(g, "cytosine_svwn5_uks.npz", prune="Robust",
                                           device=False)
    tasks = oracle_ssf_tasks(lb.get_tasks(), mol.coords())
    e, Vs, Vz, n = oracle.eval_exc_vxc_uks(oracle_basis(basis), tasks, d["Ps"], d["Pz"], "SVWN5")
    nbf = len(Vs)
    assert abs(e - d["EXC"][0]) <= 5e-9
    assert np.linalg.norm(Vs - d["VXCs"]) / nbf <= 2e-11
    assert np.linalg.norm(Vz - d["VXCz"]) / nbf <= 1e-12
    assert abs(n - 57.0) < 1e-4  # cytosine C4H5N3O: 58 electrons minus one (doublet cation)


@pytest.mark.parametrize("func", ["SVWN5", "PBE", "PBE0", "REVPBE"])
def test_polarized_functional_unpolarized_limit(func):
    """rho_a = rho_b = rho / 2, sigma_ss = sigma / 4: the polarized functional
    equals the unpolarized one (energy, d/drho, d/dsigma)."""
    rng = np.random.default_rng(11)
    rho = 10.0 ** rng.uniform(-8, 2, 400)
    sigma = rho ** (8 / 3) * 10.0 ** rng.uniform(-3, 2, 400)
    e0, vr0, vs0 = oracle.functional(func, rho, sigma)
    e1, vr1, vs1 = oracle.functional_pol(func, np.stack([rho / 2, rho / 2], 1),
                                         np.stack([sigma / 4] * 3, 1))
    assert np.allclose(e1, e0, rtol=1e-10, atol=1e-300)
    assert np.allclose(vr1[:, 0], vr0, rtol=1e-9, atol=1e-300)
    assert np.allclose(vr1[:, 1], vr0, rtol=1e-9, atol=1e-300)
    if func != "SVWN5":
        # the three partials cancel in their sum: compare on their own scale
        assert np.all(np.abs(vs1.sum(1) / 4 - vs0) <= 1e-13 * np.abs(vs1).sum(1))


def test_uks_closed_shell_equals_rks():
    """Ps = 2 P, Pz = 0: UKS gives the RKS EXC and VXC_s = VXC, VXC_z = 0."""
    import gauxc_gb300 as g
    from gauxc_gb300 import workloads as W
    from helpers import oracle_basis, oracle_ssf_tasks
    s = W.config(5)["systems"][0]
    mol, basis, mg, lb = W.build_system(s, device=False)
    tasks = oracle_ssf_tasks(lb.get_tasks(), mol.coords())[::7]
    ob = oracle_basis(basis)
    e, V, n = oracle.eval_exc_vxc(ob, tasks, s["P"], "PBE")
    eu, Vs, Vz, nu = oracle.eval_exc_vxc_uks(ob, tasks, 2 * s["P"], np.zeros_like(s["P"]), "PBE")
    assert abs(eu - e) <= 1e-10 * abs(e)
    assert np.abs(Vs - V).max() <= 1e-10 * np.abs(V).max()
    assert np.abs(Vz).max() == 0.0
    assert abs(nu - n) <= 1e-12 * n
