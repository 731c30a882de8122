"""Extract small ``.npz`` fixtures from the reference's HDF5 golden files.

Run where the reference checkout (read-only) is available, with its root in
``$GAUXC_REF``::

    GAUXC_REF=<reference checkout> python tests/golden/make_fixtures.py

The GPU test machines never see the reference tree; they only read the
committed ``.npz`` files this script writes next to itself.

Sources (reference paths):
  tests/ref_data/benzene_svwn5_cc-pvdz_ufg_ssf.hdf5            -> benzene_svwn5.npz
  tests/ref_data/benzene_svwn5_cc-pvdz_ufg_ssf_treutler_prune.hdf5 -> benzene_svwn5_treutler.npz
  tests/ref_data/benzene_pbe0_cc-pvdz_ufg_ssf.hdf5             -> benzene_pbe0.npz
      (molecule, normalized basis, alpha density P, VXC, EXC; read as in
       tests/xc_integrator.cxx:47-106)
  tests/ref_data/cytosine_svwn5_cc-pvdz_ufg_ssf_robust_uks.hdf5 -> cytosine_svwn5_uks.npz
      (UKS: scalar and z densities, VXC_SCALAR / VXC_Z, EXC;
       tests/xc_integrator.cxx:218-236)
  tests/ref_data/benzene_weights_ssf.hdf5                      -> benzene_weights_ssf.npz
      (points, unmodified and SSF-modified weights per task; every
       ``POINT_STRIDE``-th point is kept: SSF acts point by point)
  tests/ref_data/water_cc-pVDZ_collocation.hdf5                -> water_collocation.npz
      (shell mask, points, phi and grad phi per task, host layout
       eval[ipt*nbe + ibf]; tests/collocation.cxx)
  tests/ref_data/benzene_cc-pvdz_ufg_tasks_1mpi_rank0_pv1.hdf5 -> benzene_tasks.npz
      (iParent, npts, nbe, shell_list, dist_nearest per task;
       tests/load_balancer_test.cxx)
  tests/basis/old/cc-pvdz.g94                                  -> ccpvdz_raw.npz
      (unnormalized H, C, O shells, parsed like tests/basis/parse_basis.cxx)
"""
import os
import sys
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from h5lite import H5File  # noqa: E402

REF = os.environ.get("GAUXC_REF")
DATA = os.path.join(REF, "tests", "ref_data") if REF else None
POINT_STRIDE = 7


def mol_arrays(f, path="/MOLECULE"):
    m = f.read(path)
    Z = m["Atomic Number"].astype(np.int64)
    xyz = np.stack([m["X Coordinate"], m["Y Coordinate"], m["Z Coordinate"]], 1)
    return Z, xyz


def basis_arrays(f, path="/BASIS"):
    b = f.read(path)
    nsh = len(b)
    nprim = b["NPRIM"].astype(np.int32)
    l = b["L"].astype(np.int32)
    pure = b["PURE"].astype(np.int32)
    alpha = np.zeros((nsh, 32))
    coeff = np.zeros((nsh, 32))
    for i in range(nsh):
        n = nprim[i]
        alpha[i, :n] = b["ALPHA"][i][:n]
        coeff[i, :n] = b["COEFF"][i][:n]
    origin = np.array([b["ORIGIN"][i] for i in range(nsh)])
    return dict(sh_nprim=nprim, sh_l=l, sh_pure=pure, sh_alpha=alpha,
                sh_coeff=coeff, sh_origin=origin)


def xc_case(fname, out):
    f = H5File(os.path.join(DATA, fname))
    Z, xyz = mol_arrays(f)
    d = dict(Z=Z, xyz=xyz, **basis_arrays(f))
    # HighFive writes Eigen column-major data as-is; the matrices are
    # symmetric so the orientation does not matter.
    d["P"] = f.read("/DENSITY")
    d["VXC"] = f.read("/VXC")
    d["EXC"] = np.array(f.read("/EXC")).reshape(-1)[:1]
    np.savez_compressed(os.path.join(HERE, out), **d)


def uks_case(fname, out):
    """UKS golden: scalar / z densities (Ps = Pa + Pb, Pz = Pa - Pb) and the
    two VXC matrices (tests/xc_integrator.cxx:218-236)."""
    f = H5File(os.path.join(DATA, fname))
    Z, xyz = mol_arrays(f)
    d = dict(Z=Z, xyz=xyz, **basis_arrays(f))
    d["Ps"] = f.read("/DENSITY_SCALAR")
    d["Pz"] = f.read("/DENSITY_Z")
    d["VXCs"] = f.read("/VXC_SCALAR")
    d["VXCz"] = f.read("/VXC_Z")
    d["EXC"] = np.array(f.read("/EXC")).reshape(-1)[:1]
    np.savez_compressed(os.path.join(HERE, out), **d)


def tasks_group(f, group):
    n = int(f.read(group + "/ntasks")[0])
    rows = []
    for i in range(n):
        g = f"{group}/task_{i}/"
        rows.append(dict(
            iParent=int(f.read(g + "iParent")[0]),
            npts=int(f.read(g + "npts")[0]),
            nbe=int(f.read(g + "bfn_screening_nbe")[0]),
            dist_nearest=float(f.read(g + "dist_nearest")[0]),
            shell_list=f.read(g + "shell_list").astype(np.int32),
            points=f.read(g + "points") if f.exists(g + "points") else None,
            weights=f.read(g + "weights"),
        ))
    return rows


def weights_case():
    f = H5File(os.path.join(DATA, "benzene_weights_ssf.hdf5"))
    Z, xyz = mol_arrays(f)
    unm = tasks_group(f, "/tasks_unm")
    mod = tasks_group(f, "/tasks_mod")
    pts, w0, w1, ipar, dn, tid = [], [], [], [], [], []
    for it, (a, b) in enumerate(zip(unm, mod)):
        sel = np.arange(0, len(a["weights"]), POINT_STRIDE)
        pts.append(a["points"][sel])
        w0.append(a["weights"][sel])
        w1.append(b["weights"][sel])
        ipar.append(np.full(len(sel), a["iParent"], np.int32))
        dn.append(np.full(len(sel), a["dist_nearest"]))
        tid.append(np.full(len(sel), it, np.int32))
    np.savez_compressed(os.path.join(HERE, "benzene_weights_ssf.npz"),
                        Z=Z, xyz=xyz, points=np.concatenate(pts),
                        w_unm=np.concatenate(w0), w_mod=np.concatenate(w1),
                        iparent=np.concatenate(ipar),
                        dist_nearest=np.concatenate(dn),
                        task=np.concatenate(tid))


def collocation_case():
    f = H5File(os.path.join(DATA, "water_cc-pVDZ_collocation.hdf5"))
    n = int(f.read("/nentries")[0])
    d = {"nentries": np.array([n])}
    for i in range(n):
        g = f"/entry_{i}/"
        d[f"mask_{i}"] = f.read(g + "mask").astype(np.int32)
        d[f"pts_{i}"] = f.read(g + "pts")
        for k in ("eval", "deval_x", "deval_y", "deval_z"):
            d[f"{k}_{i}"] = f.read(g + k)
    # Water geometry from tests/standards.cxx (make_water), bohr.
    d["Z"] = np.array([1, 8, 1])
    d["xyz"] = np.array([[0.0, 1.579252144093028, 2.174611055780858],
                         [0.0, 0.0, 0.0],
                         [0.0, 1.579252144093028, -2.174611055780858]])
    np.savez_compressed(os.path.join(HERE, "water_collocation.npz"), **d)


def tasks_case():
    f = H5File(os.path.join(DATA, "benzene_cc-pvdz_ufg_tasks_1mpi_rank0_pv1.hdf5"))
    rows = tasks_group(f, "/tasks")
    sl = [r["shell_list"] for r in rows]
    off = np.cumsum([0] + [len(s) for s in sl])
    np.savez_compressed(
        os.path.join(HERE, "benzene_tasks.npz"),
        iparent=np.array([r["iParent"] for r in rows], np.int32),
        npts=np.array([r["npts"] for r in rows], np.int32),
        nbe=np.array([r["nbe"] for r in rows], np.int32),
        dist_nearest=np.array([r["dist_nearest"] for r in rows]),
        shell_list=np.concatenate(sl).astype(np.int32),
        shell_off=off.astype(np.int64))


AM = {"S": 0, "P": 1, "D": 2, "F": 3, "G": 4}


def g94_case():
    """Parse the G94 cc-pVDZ file for H, C, O (unnormalized primitives)."""
    path = os.path.join(REF, "tests", "basis", "old", "cc-pvdz.g94")
    recs, cur = [], None
    with open(path) as fh:
        for line in fh:
            if "!" in line or not line.strip():
                continue
            if "****" in line:
                cur = []
                recs.append(cur)
                continue
            cur.append(line.rstrip("\n"))
    out = {}
    for rec in recs:
        if not rec:
            continue
        sym = rec[0].split()[0].upper()
        if sym not in ("H", "C", "O"):
            continue
        shells = []
        i = 1
        while i < len(rec):
            tok = rec[i].split()
            l = AM[tok[0]]
            n = int(tok[1])
            prims = [[float(v.replace("D", "e").replace("d", "e")) for v in rec[i + 1 + k].split()]
                     for k in range(n)]
            shells.append((l, [p[0] for p in prims], [p[1] for p in prims]))
            i += 1 + n
        out[sym + "_l"] = np.array([s[0] for s in shells], np.int32)
        out[sym + "_nprim"] = np.array([len(s[1]) for s in shells], np.int32)
        a = np.zeros((len(shells), 32))
        c = np.zeros((len(shells), 32))
        for k, s in enumerate(shells):
            a[k, :len(s[1])] = s[1]
            c[k, :len(s[2])] = s[2]
        out[sym + "_alpha"] = a
        out[sym + "_coeff"] = c
    np.savez_compressed(os.path.join(HERE, "ccpvdz_raw.npz"), **out)


if __name__ == "__main__":
    if not REF or not os.path.isdir(DATA):
        sys.exit("set GAUXC_REF to the reference checkout (its tests/ref_data holds the HDF5 files)")
    xc_case("benzene_svwn5_cc-pvdz_ufg_ssf.hdf5", "benzene_svwn5.npz")
    xc_case("benzene_svwn5_cc-pvdz_ufg_ssf_treutler_prune.hdf5", "benzene_svwn5_treutler.npz")
    xc_case("benzene_pbe0_cc-pvdz_ufg_ssf.hdf5", "benzene_pbe0.npz")
    uks_case("cytosine_svwn5_cc-pvdz_ufg_ssf_robust_uks.hdf5", "cytosine_svwn5_uks.npz")
    weights_case()
    collocation_case()
    tasks_case()
    g94_case()
    print("fixtures written to", HERE)
