"""Shared test helpers: systems from the golden fixtures, oracle adapters."""
import numpy as np

import oracle
from conftest import golden

EPS = np.finfo(float).eps


def benzene_system(g, fname, tol=EPS, prune="Unpruned", grid="UltraFineGrid", device=True):
    d = golden(fname)
    mol = g.Molecule([(int(Z), *x) for Z, x in zip(d["Z"], d["xyz"])])
    shells = [g.Shell(int(d["sh_l"][i]), d["sh_alpha"][i, :d["sh_nprim"][i]],
                      d["sh_coeff"][i, :d["sh_nprim"][i]], d["sh_origin"][i],
                      bool(d["sh_pure"][i]), tolerance=tol) for i in range(len(d["sh_l"]))]
    basis = g.BasisSet(shells, normalize=False)
    mg = g.MolGridFactory.create_default_molgrid(mol, g.PruningScheme[prune], 512,
                                                 g.RadialQuad.MuraKnowles,
                                                 g.AtomicGridSizeDefault[grid])
    rt = g.DeviceRuntimeEnvironment(0.9) if device else g.RuntimeEnvironment()
    ex = g.ExecutionSpace.Device if device else g.ExecutionSpace.Host
    lb = g.LoadBalancerFactory(ex, "Default").get_instance(rt, mol, mg, basis)
    return d, mol, basis, mg, lb


def oracle_basis(basis):
    l, pure, nprim, alpha, coeff, origin, _ = basis.arrays()
    return oracle.Basis(l, pure, nprim, alpha, coeff, origin)


def flat_points(tasks):
    pts = np.concatenate([t["points"] for t in tasks])
    w = np.concatenate([t["weights"] for t in tasks])
    ip = np.concatenate([np.full(t["npts"], t["iParent"], np.int32) for t in tasks])
    dn = np.concatenate([np.full(t["npts"], t["dist_nearest"]) for t in tasks])
    return pts, w, ip, dn


def oracle_ssf_tasks(tasks, coords):
    """Tasks with SSF weights applied by the oracle (host algorithm)."""
    pts, w, ip, dn = flat_points(tasks)
    wm = oracle.ssf_weights(pts, ip, dn, coords, w)
    out, o = [], 0
    for t in tasks:
        out.append((t["points"], wm[o:o + t["npts"]], t["shell_list"]))
        o += t["npts"]
    return out


def oracle_exc_vxc(basis, mol, lb, P, func, weighted=False):
    tasks = lb.get_tasks()
    if weighted:
        otasks = [(t["points"], t["weights"], t["shell_list"]) for t in tasks]
    else:
        otasks = oracle_ssf_tasks(tasks, mol.coords())
    return oracle.eval_exc_vxc(oracle_basis(basis), otasks, P, func)
