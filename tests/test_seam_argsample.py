"""The in-process C++ seam (argweaver_gb300/seam/sample_thread_gpu.cpp) under the reference's
own arg-sample.

oracle/Makefile target `seam` compiles arg-sample from the reference's sources twice: as the
reference builds it, and with sample_thread.o replaced by the seam, whose forward pass and
traceback go through this library's C ABI. Here that C ABI is served by the oracle on the CPU
(oracle/seam_backend.cpp), so the run needs no GPU; it checks that the seam hands the
reference's objects (trees, SPRs, node mappings, sequences by leaf, the model, the conditioned
samplers' first column and last state) to the C ABI as the reference means them and draws
rand() in the reference's order. The same seam linked to libargweaver_gb300.so (target
arg-sample-gpu) runs the CUDA path, which the GPU parity tests hold to the oracle.

Runs only where the reference checkout exists ($AWG_REFERENCE, by default the checkout the
fixture script uses); it is skipped elsewhere.
"""

import gzip
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("AWG_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))
SEAM = os.path.join(ROOT, "oracle", "_ref", "seam")
SITES = os.path.join(REF, "examples", "sim1", "sim1.sites")

pytestmark = pytest.mark.skipif(not os.path.exists(SITES),
                                reason="the reference checkout is not present")


@pytest.fixture(scope="module")
def binaries():
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), "ref", "seam",
                    f"REF={REF}"], check=True)
    return os.path.join(SEAM, "arg-sample-ref"), os.path.join(SEAM, "arg-sample-oracle")


def run(binary, out, seed, iters):
    os.makedirs(os.path.dirname(out), exist_ok=True)
    subprocess.run([binary, "-s", SITES, "--ntimes", "20", "--maxtime", "200e3", "-c", "10",
                    "-x", str(seed), "-n", str(iters), "-o", out], check=True,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)


@pytest.mark.parametrize("seed", [3, 11])
def test_arg_sample_through_the_seam_writes_the_reference_args(binaries, tmp_path, seed):
    """Sequential threading of the 8 haplotypes (sample_arg_thread), then 20 MCMC iterations
    of subtree re-threading (cond_sample_arg_thread_internal): every sampled ARG and the
    statistics file equal the unmodified arg-sample's under the same seed."""
    ref_bin, seam_bin = binaries
    iters = 20
    run(ref_bin, str(tmp_path / "ref" / "out"), seed, iters)
    run(seam_bin, str(tmp_path / "seam" / "out"), seed, iters)
    for i in range(0, iters + 1, 10):
        a = gzip.open(tmp_path / "ref" / f"out.{i}.smc.gz").read()
        b = gzip.open(tmp_path / "seam" / f"out.{i}.smc.gz").read()
        assert a == b, f"ARG of iteration {i} differs"
    assert (tmp_path / "ref" / "out.stats").read_bytes() == \
        (tmp_path / "seam" / "out.stats").read_bytes()


def test_gpu_build_of_the_seam_links(binaries):
    """arg-sample over the CUDA library links (it runs on a GPU machine that also holds the
    reference's sources)."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"),
                    "_ref/seam/arg-sample-gpu", f"REF={REF}"], check=True)
    assert os.path.exists(os.path.join(SEAM, "arg-sample-gpu"))
