"""Seeded synthetic workloads: water clusters in an even-tempered basis.

The five workloads (index 0-4) are:
  0  one water, SVWN5, Mura-Knowles 75 x Lebedev 302 unpruned, 60 bf, nocc 5
  1  32 waters in a 10 A cube, PBE, MK 99 x 590 Treutler-pruned, 1920 bf, nocc 160
  2  96 waters in a 14 A cube, PBE, MK 75 x 302 Treutler, 5760 bf, nocc 480
  3  64 clusters of 1-40 waters (4-13 A cubes), half SVWN5 / half PBE,
     MK 75 x 302 Treutler, batch sizes 128-1024, nocc = 5 n_water
  4  256 waters in a 20 A cube, PBE, MK 75 x 302 Treutler, shell tol 1e-12,
     15360 bf, nocc 1280
  5  profiling case: 4 waters in a 6 A cube, PBE, MK 99 x 590 Treutler, 240 bf
     (same kernels as 1 with a few GB of device memory)
Water geometry: O at (0,0,0) A, H at (+-0.757, 0.587, 0) A; clusters apply
uniform random rotations (Shoemake quaternions) and uniform random centres
in the cube, rejecting placements with an O-O distance below 2.6 A.
Basis: uncontracted spherical Gaussians, O: 10 s (0.08*3^k), 6 p (0.1*3^k),
2 d (0.5*3^k); H: 5 s (0.08*3^k), 2 p (0.1*3^k).  Density P = C C^T with
C[nbf, nocc] ~ N(0,1)/sqrt(nbf).  All randomness uses numpy's PCG64 with the
fixed seeds below, so every machine builds identical inputs.
"""
import numpy as np

BOHR_PER_ANG = 1.0 / 0.529177210903
WATER_ANG = np.array([[0.0, 0.0, 0.0], [0.757, 0.587, 0.0], [-0.757, 0.587, 0.0]])
WATER_Z = [8, 1, 1]

SEEDS = {0: 1000, 1: 1001, 2: 1002, 3: 1003, 4: 1004, 5: 1005}


def _rotation(u):
    u1, u2, u3 = u
    q = np.array([np.sqrt(1 - u1) * np.sin(2 * np.pi * u2), np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
                  np.sqrt(u1) * np.sin(2 * np.pi * u3), np.sqrt(u1) * np.cos(2 * np.pi * u3)])
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def water_cluster(n, cube_ang, rng, min_oo_ang=2.6, max_tries=100000):
    """Atoms (Z, x, y, z) in bohr for n rotated waters placed in a cube."""
    if n == 1:
        centres = [np.zeros(3)]
        rots = [np.eye(3)]
    else:
        centres, rots = [], []
        tries = 0
        while len(centres) < n:
            tries += 1
            if tries > max_tries:
                raise RuntimeError("could not place waters; cube too small")
            c = rng.uniform(0.0, cube_ang, size=3)
            R = _rotation(rng.uniform(size=3))
            if all(np.linalg.norm(c - o) >= min_oo_ang for o in centres):
                centres.append(c)
                rots.append(R)
    atoms = []
    for c, R in zip(centres, rots):
        for Z, x in zip(WATER_Z, WATER_ANG):
            p = (R @ x + c) * BOHR_PER_ANG
            atoms.append((Z, p[0], p[1], p[2]))
    return atoms


def even_tempered_shells(atoms, tolerance=1e-10):
    """Shell tuples (l, [alpha], [coeff], origin) for the even-tempered basis."""
    spec = {8: [(0, 0.08, 10), (1, 0.1, 6), (2, 0.5, 2)], 1: [(0, 0.08, 5), (1, 0.1, 2)]}
    shells = []
    for Z, x, y, z in atoms:
        for l, a0, n in spec[Z]:
            for k in range(n):
                shells.append((l, [a0 * 3.0 ** k], [1.0], (x, y, z), tolerance))
    return shells


def density(nbf, nocc, rng):
    C = rng.standard_normal((nbf, nocc)) / np.sqrt(nbf)
    return np.asfortranarray(C @ C.T)


def config(idx):
    """Description of one workload: dict(systems=[...]) with per-system
    atoms, shells, P, functional, grid options and batch size."""
    rng = np.random.default_rng(SEEDS[idx])
    if idx == 0:
        specs = [(1, 0.0, "SVWN5", "Unpruned", "FineGrid", 512, 1e-10)]
    elif idx == 1:
        specs = [(32, 10.0, "PBE", "Treutler", "UltraFineGrid", 512, 1e-10)]
    elif idx == 2:
        specs = [(96, 14.0, "PBE", "Treutler", "FineGrid", 512, 1e-10)]
    elif idx == 3:
        specs = []
        for i in range(64):
            n = int(rng.integers(1, 41))
            cube = 4.0 + 9.0 * (n - 1) / 39.0
            bs = int(rng.choice([128, 256, 512, 1024]))
            specs.append((n, cube, "SVWN5" if i % 2 == 0 else "PBE", "Treutler", "FineGrid", bs, 1e-10))
    elif idx == 4:
        specs = [(256, 20.0, "PBE", "Treutler", "FineGrid", 512, 1e-12)]
    elif idx == 5:
        specs = [(4, 6.0, "PBE", "Treutler", "UltraFineGrid", 512, 1e-10)]
    else:
        raise ValueError(idx)
    systems = []
    for n, cube, func, prune, grid, bs, tol in specs:
        atoms = water_cluster(n, cube, rng)
        shells = even_tempered_shells(atoms, tol)
        nbf = sum(2 * s[0] + 1 for s in shells)
        P = density(nbf, 5 * n, rng)
        systems.append(dict(n_water=n, atoms=atoms, shells=shells, P=P, functional=func,
                            pruning=prune, grid=grid, batch_size=bs, tolerance=tol, nbf=nbf))
    return dict(index=idx, systems=systems)


def build_system(sysd, device=True):
    """Molecule, basis, grid and load balancer for one system (no weights yet)."""
    import gauxc_gb300 as g
    mol = g.Molecule(sysd["atoms"])
    basis = g.BasisSet([g.Shell(l, a, c, o, pure=True, tolerance=t) for l, a, c, o, t in sysd["shells"]])
    mg = g.MolGridFactory.create_default_molgrid(
        mol, g.PruningScheme[sysd["pruning"]], sysd["batch_size"], g.RadialQuad.MuraKnowles,
        g.AtomicGridSizeDefault[sysd["grid"]])
    rt = g.DeviceRuntimeEnvironment(0.9) if device else g.RuntimeEnvironment()
    # the Device load balancer screens on the GPU; the Host one on the host
    ex = g.ExecutionSpace.Device if device else g.ExecutionSpace.Host
    lb = g.LoadBalancerFactory(ex, "Default").get_instance(rt, mol, mg, basis)
    return mol, basis, mg, lb
