"""The C ABI library builds, loads without a GPU and exports every declared entry point;
its host-side planning agrees with the oracle and rejects malformed problems."""

import os
import re

import numpy as np
import pytest

import pyoracle
from argweaver_gb300 import api, capi
from argweaver_gb300.problem import Problem
from conftest import GOLDEN, ROOT, golden_names

HEADER = os.path.join(ROOT, "include", "argweaver_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    text = re.sub(r"^\s*#[^\n]*", "", text, flags=re.M)  # preprocessor lines
    names = []
    for decl in text.split(";"):
        decl = " ".join(decl.split())
        if "typedef" in decl or "(" not in decl or decl.startswith("#"):
            continue
        m = re.search(r"([A-Za-z_][A-Za-z0-9_]*)\s*\(", decl)
        if m:
            names.append(m.group(1))
    return names


def test_header_declares_the_reference_abi():
    names = set(declared_functions())
    for ref in ["arghmm_forward_alg", "arghmm_sample_posterior", "arghmm_new_trees",
                "arghmm_sample_arg_thread_internal", "arghmm_get_nstates",
                "delete_forward_matrix", "delete_path", "delete_double_matrix",
                "delete_local_trees", "arghmm_backward_alg"]:
        assert ref in names


def test_library_exports_every_declared_symbol():
    lib = capi.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert {n for n, _, _ in capi.PROTOTYPES} == set(declared_functions())


@pytest.mark.parametrize("name", golden_names())
def test_host_plan_cells_match_oracle(name):
    prob = Problem.load(os.path.join(GOLDEN, name + ".prob"))
    fw, _ = pyoracle.forward(prob)
    assert api.cells(prob) == fw.shape[0] == prob.cells()


def _bad(prob, **kw):
    d = dict(prob.__dict__)
    d.update(kw)
    return Problem(**d)


def test_invalid_problems_are_rejected():
    prob = Problem.load(os.path.join(GOLDEN, "dsmc_k8_s11.prob"))
    bad = []
    par = prob.ptrees.copy(); par[0, 0] = 99
    bad.append(_bad(prob, ptrees=par))                                    # parent out of range
    bl = prob.blocklens.copy(); bl[0] += 1
    bad.append(_bad(prob, blocklens=bl))                                  # lengths != seqlen
    seqs = prob.seqs.copy(); seqs[0, 0] = ord("X")
    bad.append(_bad(prob, seqs=seqs))                                     # bad base
    bad.append(_bad(prob, times=np.linspace(0, 1, 40), popsizes=np.ones(40)))  # ntimes > 32
    bad.append(_bad(prob, seqs=prob.seqs[:-1]))                           # missing sequence
    ages = prob.ages.copy(); ages[0, 0] = prob.ntimes
    bad.append(_bad(prob, ages=ages))                                     # age out of range
    for b in bad:
        with pytest.raises(ValueError):
            api.cells(b)
    assert api.cells(prob) > 0


def test_batch_sizing_checks_sequence_bytes():
    # the batch path checks sequence bytes while it packs them (plan_fill); a dry sizing
    # run goes through the same packing and must refuse a bad byte, in any problem
    from argweaver_gb300 import capi
    prob = Problem.load(os.path.join(GOLDEN, "dsmc_k8_s11.prob"))
    lib = capi.load()
    probs, _, _, keep = api._bind_batch([prob, prob], "fp32", False, True, False, None)
    assert lib.awg_batch_device_bytes(probs, 2, capi.AWG_FP32, 1, 0) > 0
    for row, col in ((0, 0), (prob.nseqs - 1, prob.seqlen - 1)):
        seqs = prob.seqs.copy()
        seqs[row, col] = ord("x")
        probs, _, _, keep2 = api._bind_batch([prob, _bad(prob, seqs=seqs)], "fp32", False, True,
                                             False, None)
        assert lib.awg_batch_device_bytes(probs, 2, capi.AWG_FP32, 1, 0) < 0
        assert "problem 1: sequence byte" in capi.last_error()
