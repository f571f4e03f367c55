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
