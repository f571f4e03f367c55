"""Recombination sampling along a thread (sample_recombinations, recomb.cpp:151-235): the
device routine's logic, compiled for the host, against the reference's recombinations on
the fixtures' own sampled paths (same draws: rand() after srand(seed))."""

import ctypes as C
import glob
import os
import subprocess

import numpy as np
import pytest

from argweaver_gb300 import api, build, capi
from argweaver_gb300.problem import Problem
from conftest import GOLDEN, load_golden

RMAX = 2147483647.0  # glibc RAND_MAX
NAMES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "recomb", "*.npz")))


def draws(seed: int, n: int) -> np.ndarray:
    """rand() / RAND_MAX after srand(seed), in draw order."""
    libc = C.CDLL(None)
    libc.srand(C.c_uint(seed))
    return np.array([libc.rand() / RMAX for _ in range(n)], dtype=np.float64)


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("rs") / "librs.so")
    here = os.path.dirname(os.path.abspath(__file__))
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread",
           "-ffp-contract=off", "-I" + build.INCLUDE, "-I" + build.CSRC,
           "-I/usr/local/cuda/include", "-o", out, os.path.join(here, "recomb_host_shim.cpp"),
           os.path.join(build.CSRC, "host_plan.cpp")]
    subprocess.run(cmd, check=True)
    lib = C.CDLL(out)
    lib.rs_host.restype = C.c_int
    V = C.c_void_p
    lib.rs_host.argtypes = [C.POINTER(capi.AwgProblem), V, V, C.c_int, V, V, V, C.c_int,
                            C.POINTER(C.c_int)]
    return lib


def run_host(lib, prob, path, u):
    b = api._Bound(prob)
    L = prob.seqlen
    pos, node, time = (np.zeros(L, dtype=np.int32) for _ in range(3))
    used = C.c_int(0)
    path = np.ascontiguousarray(path, dtype=np.int32)
    n = lib.rs_host(C.byref(b.c), path.ctypes.data, u.ctypes.data, len(u), pos.ctypes.data,
                    node.ctypes.data, time.ctypes.data, L, C.byref(used))
    return n, pos[:max(n, 0)], node[:max(n, 0)], time[:max(n, 0)], used.value


def case(name):
    """(problem, path, fixture): the golden problem and its sampled path, or a larger
    problem stored with the fixture (names extra_*)."""
    rec = np.load(os.path.join(GOLDEN, "recomb", name + ".npz"))
    if name.startswith("extra_"):
        return Problem.load(os.path.join(GOLDEN, "recomb", name + ".prob")), rec["path"], rec
    prob, gold = load_golden(name)
    return prob, gold["path"], rec


@pytest.mark.parametrize("name", NAMES)
def test_host_routine_matches_reference(shim, name):
    prob, path, rec = case(name)
    u = draws(int(rec["seed"]), 2 * prob.seqlen + 2)
    n, pos, node, time, used = run_host(shim, prob, path, u)
    assert n == len(rec["pos"])
    np.testing.assert_array_equal(pos, rec["pos"])
    np.testing.assert_array_equal(node, rec["node"])
    np.testing.assert_array_equal(time, rec["time"])
    assert u[used] == int(rec["next_rand"]) / RMAX  # the same number of draws


def test_host_routine_edges(shim):
    prob, path, rec = case("extra_k8_T20")
    u = draws(int(rec["seed"]), 2 * prob.seqlen + 2)
    n = len(rec["pos"])
    # too few uniforms, too small an output, a path entry that is no state: refused
    assert run_host(shim, prob, path, u[:5])[0] == -2
    assert run_host(shim, prob, path, u)[0] == n
    b = api._Bound(prob)
    small = np.zeros(n - 1, dtype=np.int32)
    used = C.c_int(0)
    p32 = np.ascontiguousarray(path, dtype=np.int32)
    assert shim.rs_host(C.byref(b.c), p32.ctypes.data, u.ctypes.data, len(u), small.ctypes.data,
                        small.ctypes.data, small.ctypes.data, n - 1, C.byref(used)) == -3
    bad = p32.copy()
    bad[rec["pos"][0]] = 10 ** 6
    assert run_host(shim, prob, bad, u)[0] == -1


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference(name):
    import pyoracle
    prob, path, rec = case(name)
    u = draws(int(rec["seed"]), 2 * prob.seqlen + 2)
    pos, node, time, used = pyoracle.sample_recombinations(prob, path, u)
    np.testing.assert_array_equal(pos, rec["pos"])
    np.testing.assert_array_equal(node, rec["node"])
    np.testing.assert_array_equal(time, rec["time"])
    assert u[used] == int(rec["next_rand"]) / RMAX


def stress_path(prob, path, seed):
    """The path with extra state changes inside blocks (each a valid state of its tree):
    every recombination branch of the sampler runs many times."""
    import pyoracle
    ns = pyoracle.nstates(prob)
    rng = np.random.default_rng(seed)
    out = np.array(path, dtype=np.int32)
    flip = rng.random(prob.seqlen) < 0.05
    for i in np.nonzero(flip)[0]:
        if ns[i] > 0:
            out[i] = rng.integers(0, ns[i])
    # a state holds until the next change, so the new state stays valid within its block
    starts = np.concatenate([[0], np.cumsum(prob.blocklens)[:-1]])
    block = np.searchsorted(starts, np.arange(prob.seqlen), side="right") - 1
    for i in range(1, prob.seqlen):
        if not flip[i] and block[i] == block[i - 1]:
            out[i] = out[i - 1]
    return out


@pytest.mark.parametrize("k,L,T,missing,internal,seed", [
    (10, 4000, 20, 0.0, False, 1), (25, 3000, 16, 0.02, False, 2), (6, 6000, 32, 0.0, False, 3),
    (15, 3000, 20, 0.01, True, 4), (30, 2000, 20, 0.0, True, 5)])
def test_device_routine_matches_oracle(shim, k, L, T, missing, internal, seed):
    # random problems, traceback paths with extra state changes: the routine the device
    # runs equals the oracle's restatement on thousands of draws
    import pyoracle
    from argweaver_gb300.sim import leaf_cut, simulate
    prob = simulate(k, L, seed, ntimes=T, missing=missing, rho=1.6e-7)
    if internal:
        prob = leaf_cut(prob)
    fw, _ = pyoracle.forward(prob)
    path = pyoracle.traceback(prob, fw, pyoracle.rand_uniforms(seed, prob.seqlen))
    path = stress_path(prob, path, seed)
    u = np.random.default_rng(seed).random(2 * prob.seqlen + 2)
    o = pyoracle.sample_recombinations(prob, path, u)
    n, pos, node, time, used = run_host(shim, prob, path, u)
    assert n == len(o[0]) > 20
    np.testing.assert_array_equal(pos, o[0])
    np.testing.assert_array_equal(node, o[1])
    np.testing.assert_array_equal(time, o[2])
    assert used == o[3]
