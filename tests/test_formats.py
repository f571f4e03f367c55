"""arg-sample's input formats on the host (formats.cpp): sites and SMC files read and
compressed as the reference reads them (its own reader's output on the same files is the
fixture), written so that the reference reads them back, and malformed files rejected."""

import gzip
import os

import numpy as np
import pytest

from argweaver_gb300 import formats as fm
from argweaver_gb300.problem import Problem
from argweaver_gb300.sim import simulate
from conftest import GOLDEN

FIX = os.path.join(GOLDEN, "formats")
CASES = [("k8", "", 1), ("k8", "", 10), ("k16_missing", ".gz", 1), ("k16_missing", ".gz", 4)]


@pytest.mark.parametrize("name,ext,c", CASES)
def test_reader_matches_reference(name, ext, c):
    ref = Problem.load(os.path.join(FIX, f"{name}_c{c}.prob"))
    prob, names = fm.read_arg(os.path.join(FIX, name + ".sites" + ext),
                              os.path.join(FIX, name + ".smc" + ext), c, times=ref.times)
    for k in ("ptrees", "ages", "sprs", "blocklens", "seqs"):
        np.testing.assert_array_equal(getattr(prob, k), getattr(ref, k), err_msg=k)
    assert prob.start_coord == ref.start_coord
    assert prob.rho == ref.rho and prob.mu == ref.mu
    np.testing.assert_array_equal(prob.popsizes, ref.popsizes)
    assert names == [f"n{i}" for i in range(prob.nseqs)]


def test_sites_only():
    names, seqs = fm.read_sites(os.path.join(FIX, "k8.sites"), compress=10)
    ref = Problem.load(os.path.join(FIX, "k8_c10.prob"))
    np.testing.assert_array_equal(seqs, ref.seqs)
    assert len(names) == seqs.shape[0]


def test_compression_refused_like_the_reference():
    # the reference's find_compress_cols gives up when variant sites leave no room
    with pytest.raises(ValueError, match="compress"):
        fm.read_arg(os.path.join(FIX, "k16_missing.sites.gz"),
                    os.path.join(FIX, "k16_missing.smc.gz"), 10)


def test_round_trip(tmp_path):
    prob = simulate(12, 6000, 99, compress=1, add_thread=False)
    names = [f"s{i}" for i in range(prob.nseqs)]
    fm.write_sites(str(tmp_path / "a.sites.gz"), names, prob.seqs)
    fm.write_smc(str(tmp_path / "a.smc"), prob, names)
    with gzip.open(tmp_path / "a.sites.gz", "rt") as f:
        assert f.readline().startswith("NAMES\ts0\ts1")
    back, names2 = fm.read_arg(str(tmp_path / "a.sites.gz"), str(tmp_path / "a.smc"), 1,
                               times=prob.times)
    assert names2 == names
    for k in ("ptrees", "ages", "sprs", "blocklens"):
        np.testing.assert_array_equal(getattr(back, k), getattr(prob, k), err_msg=k)
    var = (prob.seqs != prob.seqs[:1]).any(axis=0)
    np.testing.assert_array_equal(back.seqs[:, var], prob.seqs[:, var])
    assert (back.seqs[:, ~var] == ord("A")).all()


def test_leaf_order_follows_the_sites_file(tmp_path):
    # SMC leaves named in another order than the sites file: leaf i becomes sequence i
    prob = simulate(6, 3000, 5, compress=1, add_thread=False)
    names = [f"s{i}" for i in range(prob.nseqs)]
    order = [3, 0, 5, 1, 4, 2]
    fm.write_sites(str(tmp_path / "b.sites"), [names[i] for i in order], prob.seqs[order])
    fm.write_smc(str(tmp_path / "b.smc"), prob, names)
    back, names2 = fm.read_arg(str(tmp_path / "b.sites"), str(tmp_path / "b.smc"), 1,
                               times=prob.times)
    assert names2 == [names[i] for i in order]
    # the tree read back, relabelled to the file's leaf order, is the original tree
    inv = np.argsort(order)
    n = prob.nnodes
    perm = np.concatenate([inv, np.arange(len(order), n)])
    pt0 = back.ptrees[0]
    orig = prob.ptrees[0]
    for j in range(n):
        p = orig[j]
        assert pt0[perm[j]] == (-1 if p == -1 else perm[p])


@pytest.mark.parametrize("text,match", [
    ("NAMES\ta\tb\nREGION\tchr\t1\n", "REGION"),
    ("NAMES\ta\tb\nREGION\tchr\t1\t100\n5\tAC\n3\tAG\n", "sorted"),
    ("NAMES\ta\tb\nREGION\tchr\t1\t100\n5\tAX\n", "invalid"),
    ("NAMES\ta\tb\nREGION\tchr\t1\t100\n5\tACG\n", "number of bases"),
    ("NAMES\ta\tb\nRANGE\tchr\t1\t100\n", "RANGE"),
])
def test_malformed_sites(tmp_path, text, match):
    path = tmp_path / "bad.sites"
    path.write_text(text)
    with pytest.raises(ValueError, match=match):
        fm.read_sites(str(path))


def test_malformed_smc(tmp_path):
    prob = simulate(4, 500, 1, compress=1, add_thread=False)
    names = [f"s{i}" for i in range(prob.nseqs)]
    fm.write_sites(str(tmp_path / "c.sites"), names, prob.seqs)
    (tmp_path / "c.smc").write_text("NAMES\ts0\ts1\ts2\ts3\nREGION\tchr\t1\t500\n"
                                    "TREE\t1\t500\t((0:1,1:1)4,(2:1,3:1)5;\n")
    with pytest.raises(ValueError, match="newick"):
        fm.read_arg(str(tmp_path / "c.sites"), str(tmp_path / "c.smc"), 1, times=prob.times)
    with pytest.raises(ValueError, match="cannot read"):
        fm.read_arg(str(tmp_path / "c.sites"), str(tmp_path / "missing.smc"), 1, times=prob.times)
