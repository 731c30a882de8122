"""Compiled clients of the library: a C program that walks the C API
(tests/native/c_api_walk.c, after the reference's tests/c_api_test.cxx) and a
C++ program on the header-only front end (tests/native/front_end.cxx).

Without a GPU both run their host parts (status handling, handles, factories,
error strings, the null-status exception).  The GPU tests run the device walk
and compare EXC, VXC and N_el with the oracle on the same system (one water,
PBE, the programs' fixed density).
"""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

import oracle
from helpers import oracle_basis, oracle_ssf_tasks

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NATIVE = os.path.join(ROOT, "tests", "native")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "gauxc_gb300", "lib")

WATER = [(1, 0.0, 1.579252144093028, 2.174611055780858), (8, 0.0, 0.0, 0.0),
         (1, 0.0, 1.579252144093028, -2.174611055780858)]


@pytest.fixture(scope="module")
def programs(g):
    g.lib()  # the library is built
    out = tempfile.mkdtemp(prefix="gauxc_gb300_native_")
    link = ["-L" + LIBDIR, "-lgauxc_gb300", "-Wl,-rpath," + LIBDIR]
    c = os.path.join(out, "c_api_walk")
    cxx = os.path.join(out, "front_end")
    subprocess.run(["gcc", "-std=c11", "-O1", "-Wall", "-I", INCLUDE,
                    os.path.join(NATIVE, "c_api_walk.c"), "-o", c] + link + ["-lm"], check=True)
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I", INCLUDE,
                    os.path.join(NATIVE, "front_end.cxx"), "-o", cxx] + link, check=True)
    yield {"c": c, "cxx": cxx, "dir": out}
    shutil.rmtree(out, ignore_errors=True)


def _run(exe, *args):
    r = subprocess.run([exe, *args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_c_api_walk_host(programs):
    assert "host walk ok" in _run(programs["c"])


def test_cxx_front_end_host(programs):
    assert "host front end ok" in _run(programs["cxx"])


def _oracle_water(g, P):
    from gauxc_gb300 import workloads as W
    shells = W.even_tempered_shells(WATER, 1e-10)
    mol = g.Molecule(WATER)
    basis = g.BasisSet([g.Shell(l, a, c, o, pure=True, tolerance=t) for l, a, c, o, t in shells])
    mg = g.MolGridFactory.create_default_molgrid(mol, g.PruningScheme.Unpruned, 512,
                                                 g.RadialQuad.MuraKnowles,
                                                 g.AtomicGridSizeDefault.FineGrid)
    lb = g.LoadBalancerFactory(g.ExecutionSpace.Host, "Default").get_instance(
        g.RuntimeEnvironment(), mol, mg, basis)
    return oracle.eval_exc_vxc(oracle_basis(basis), oracle_ssf_tasks(lb.get_tasks(), mol.coords()),
                               P, "PBE")


@pytest.mark.gpu
@pytest.mark.parametrize("prog", ["c", "cxx"])
def test_device_walk_matches_oracle(g, programs, prog):
    path = os.path.join(programs["dir"], prog + ".bin")
    _run(programs[prog], "gpu", path)
    raw = np.fromfile(path, dtype=np.float64)
    nbf = int(raw[:1].view(np.int64)[0])
    P = raw[1:1 + nbf * nbf].reshape(nbf, nbf, order="F")
    V = raw[1 + nbf * nbf:1 + 2 * nbf * nbf].reshape(nbf, nbf, order="F")
    exc, exc_only, den = raw[1 + 2 * nbf * nbf:]
    eo, Vo, no = _oracle_water(g, P)
    assert abs(exc - eo) <= 1e-10
    assert np.abs(V - Vo).max() <= 1e-10
    assert abs(exc_only - exc) <= 1e-12
    assert abs(den - 0.5 * no) <= 1e-10
