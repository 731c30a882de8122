"""Host setup layer: quadrature grids, shells, screening and task lists (no GPU).

The task list is compared bit-for-bit with the Python restatement in
oracle/screening.py on the same atomic grids.  Grid points and weights are
pinned to the reference's golden (tests/ref_data/benzene_weights_ssf.hdf5
stores the unmodified points/weights of 15 tasks of a 75 x 302 grid).
"""
import math

import numpy as np
import pytest

from conftest import golden
from helpers import benzene_system
from oracle import screening


def test_lebedev_rules_integrate_polynomials(g):
    mol = g.Molecule([(1, 0.0, 0.0, 0.0)])
    for grid, nang in (("FineGrid", 302), ("UltraFineGrid", 590)):
        mg = g.MolGridFactory.create_default_molgrid(mol, g.PruningScheme.Unpruned, 512,
                                                     g.RadialQuad.MuraKnowles,
                                                     g.AtomicGridSizeDefault[grid])
        pts, w, br = mg.atomic_grid(1)
        r = np.linalg.norm(pts, axis=1)
        shell = np.isclose(r, r.min())
        u = pts[shell] / r[shell, None]
        assert shell.sum() == nang
        # radial x angular weights integrate exp(-r^2) over R^3 to pi^(3/2)
        assert abs(np.sum(w * np.exp(-r ** 2)) - math.pi ** 1.5) < 1e-10
        # batches tile the grid exactly, each within the batch size
        assert br[0, 0] == 0 and br[-1, 1] == len(w)
        assert np.all(br[1:, 0] == br[:-1, 1]) and np.all(br[:, 1] - br[:, 0] <= 512)
        assert np.allclose(np.linalg.norm(u, axis=1), 1.0)


def test_grid_sizes_with_pruning(g):
    mol = g.Molecule([(8, 0.0, 0.0, 0.0)])
    expect = {("FineGrid", "Unpruned"): 75 * 302, ("FineGrid", "Treutler"): 12450,
              ("UltraFineGrid", "Treutler"): 30594, ("UltraFineGrid", "Unpruned"): 99 * 590,
              ("FineGrid", "Robust"): 19 * 26 + 19 * 194 + 37 * 302}
    for (grid, prune), n in expect.items():
        mg = g.MolGridFactory.create_default_molgrid(mol, g.PruningScheme[prune], 512,
                                                     g.RadialQuad.MuraKnowles,
                                                     g.AtomicGridSizeDefault[grid])
        assert len(mg.atomic_grid(8)[1]) == n, (grid, prune)


def test_grid_matches_golden_points_and_weights(g):
    """Every golden (unmodified) point/weight exists in our 75 x 302 carbon grid."""
    d = golden("benzene_weights_ssf.npz")
    mol = g.Molecule([(int(Z), *x) for Z, x in zip(d["Z"], d["xyz"])])
    mg = g.MolGridFactory.create_default_molgrid(mol, g.PruningScheme.Unpruned, 512,
                                                 g.RadialQuad.MuraKnowles,
                                                 g.AtomicGridSizeDefault.FineGrid)
    grids = {Z: mg.atomic_grid(Z) for Z in (1, 6)}
    for Z in (1, 6):
        pts, w, _ = grids[Z]
        key = {tuple(np.round(p, 9)): wi for p, wi in zip(pts, w)}
        sel = np.array([int(d["Z"][i]) == Z for i in d["iparent"]])
        if not sel.any():
            continue
        rel = d["points"][sel] - d["xyz"][d["iparent"][sel]]
        for p, wg in zip(rel, d["w_unm"][sel]):
            wi = key[tuple(np.round(p, 9))]
            assert abs(wi - wg) <= 4e-15 * abs(wg)


def test_shell_normalization_matches_golden(g):
    raw = golden("ccpvdz_raw.npz")
    b = golden("benzene_svwn5.npz")
    shells = []
    for k in range(len(raw["C_l"])):
        n = raw["C_nprim"][k]
        shells.append(g.Shell(int(raw["C_l"][k]), raw["C_alpha"][k, :n], raw["C_coeff"][k, :n],
                              b["sh_origin"][0], pure=int(raw["C_l"][k]) > 1))
    basis = g.BasisSet(shells, normalize=True)
    for k in range(len(shells)):
        c = basis.shell(k)[3]
        np.testing.assert_allclose(c, b["sh_coeff"][k, :len(c)], rtol=1e-14)


def test_cutoff_radii_bitexact(g):
    d = golden("benzene_svwn5.npz")
    for tol in (1e-6, 1e-10, 1e-12, np.finfo(float).eps):
        _, _, basis, _, _ = benzene_system(g, "benzene_svwn5.npz", tol=tol, grid="FineGrid",
                                           device=False)
        for i in range(basis.nshells()):
            l, pure, a, c, o, t, r = basis.shell(i)
            assert r == screening.cutoff_radius(l, list(a), list(c), tol)


@pytest.mark.parametrize("tol", [1e-6, 1e-10])
def test_task_list_bitexact_vs_restatement(g, tol):
    d, mol, basis, mg, lb = benzene_system(g, "benzene_svwn5.npz", tol=tol, grid="FineGrid",
                                           device=False)
    l, pure, nprim, alpha, coeff, origin, radii = basis.arrays()
    sizes = np.where(pure != 0, 2 * l + 1, (l + 1) * (l + 2) // 2)
    atoms = mol.atoms
    grids = {Z: mg.atomic_grid(Z) for Z in set(a[0] for a in atoms)}
    ref = screening.make_tasks(atoms, grids, [tuple(o) for o in origin], list(radii),
                               list(sizes), screening.dist_nearest(atoms))
    got = lb.get_tasks()
    assert len(got) == len(ref)
    for a, b in zip(got, ref):
        assert a["iParent"] == b["iParent"]
        assert a["npts"] == b["npts"]
        assert list(a["shell_list"]) == b["shell_list"]
        assert a["nbe"] == b["nbe"]
        assert a["dist_nearest"] == b["dist_nearest"]
        assert np.array_equal(a["points"], np.array(b["points"]))
        assert np.array_equal(a["weights"], np.array(b["weights"]))


def test_task_list_invariants_and_golden_metadata(g):
    """Invariants shared with the reference task list of the same system
    (benzene cc-pVDZ, UltraFine unpruned, tol = eps): points per atom, nbe as the
    sum of shell sizes, dist_nearest per parent atom."""
    gt = golden("benzene_tasks.npz")
    d, mol, basis, mg, lb = benzene_system(g, "benzene_svwn5.npz", device=False)
    l, pure, *_ = basis.arrays()
    sizes = np.where(pure != 0, 2 * l + 1, (l + 1) * (l + 2) // 2)
    tasks = lb.get_tasks()
    for i in range(len(gt["npts"])):
        sl = gt["shell_list"][gt["shell_off"][i]:gt["shell_off"][i + 1]]
        assert sizes[sl].sum() == gt["nbe"][i]
    for at in range(12):
        ours = sum(t["npts"] for t in tasks if t["iParent"] == at)
        theirs = int(gt["npts"][gt["iparent"] == at].sum())
        assert ours == theirs == 99 * 590
        dn = {t["dist_nearest"] for t in tasks if t["iParent"] == at}
        assert dn == {float(gt["dist_nearest"][gt["iparent"] == at][0])}
    for t in tasks:
        assert t["nbe"] == sizes[t["shell_list"]].sum()
        assert np.all(np.diff(t["shell_list"]) > 0)
    keys = [(t["iParent"], tuple(t["shell_list"])) for t in tasks]
    assert keys == sorted(keys) and len(set(keys)) == len(keys)


def test_task_list_keyed_against_golden(g):
    """Keyed comparison with the reference task list of the same system: the
    (iParent, shell_list) keys both lists hold, and the points under them.
    The batcher here is this project's own (IntegratorXX's is not in the
    reference tree), so batch boundaries, and with them the per-key point
    counts, differ; the shared keys hold most of the reference's points.
    Measured: 253 of the reference's 664 keys are shared, holding 89.3 % of
    its points (88.6 % of ours); no shared key has the same point count."""
    gt = golden("benzene_tasks.npz")
    d, mol, basis, mg, lb = benzene_system(g, "benzene_svwn5.npz", device=False)
    ours = {(t["iParent"], tuple(int(x) for x in t["shell_list"])): t["npts"]
            for t in lb.get_tasks()}
    theirs = {}
    for i in range(len(gt["npts"])):
        sl = gt["shell_list"][gt["shell_off"][i]:gt["shell_off"][i + 1]]
        theirs[(int(gt["iparent"][i]), tuple(int(x) for x in sl))] = int(gt["npts"][i])
    common = set(ours) & set(theirs)
    frac_keys = len(common) / len(theirs)
    frac_pts = sum(theirs[k] for k in common) / sum(theirs.values())
    assert len(theirs) == 664 and sum(theirs.values()) == 12 * 99 * 590
    assert frac_keys >= 0.38 and frac_pts >= 0.89


def test_empty_and_far_batches_are_dropped(g):
    """A shell far from the atom screens out every batch: no tasks at all."""
    mol = g.Molecule([(1, 0.0, 0.0, 0.0)])
    basis = g.BasisSet([g.Shell(0, [1.0], [1.0], (500.0, 0.0, 0.0))])
    mg = g.MolGridFactory.create_default_molgrid(mol, g.PruningScheme.Unpruned, 512,
                                                 g.RadialQuad.MuraKnowles,
                                                 g.AtomicGridSizeDefault.FineGrid)
    lb = g.LoadBalancerFactory(g.ExecutionSpace.Host, "Default").get_instance(
        g.RuntimeEnvironment(), mol, mg, basis)
    assert lb.ntasks() == 0
