"""The FP32 path's decomposed traceback draw, checked on the CPU (oracle restatement).

The decomposed draw maps the uniform to states in another order than the reference's scan
(sample(), common.h:272-290) but must give every state the same probability. Both draws
are monotone pieces of [0, 1) (the reference's one interval per state, the decomposed draw
at most two: same-branch and background), so on a grid of N uniforms the counts per state
agree to within a few grid points. The tables are random positive columns spread over six
decades, so the draws leave the current state often and reach tens of states.
"""

import numpy as np
import pytest

import pyoracle
from argweaver_gb300.sim import simulate


@pytest.mark.parametrize("k,L,seed", [(6, 60, 3), (10, 60, 4)])
def test_decomposed_draw_has_the_reference_distribution(k, L, seed):
    p = simulate(k, L, seed=seed, missing=0.01)
    fw, _ = pyoracle.forward(p)
    rng = np.random.default_rng(seed)
    table = np.exp(-rng.random(fw.size) * 14.0)
    u = rng.random(p.seqlen)
    N = 400
    reached = 0
    for i in range(0, p.seqlen - 1, 4):
        ref, dec = {}, {}
        for q in range(N):
            uu = u.copy()
            uu[i] = (q + 0.5) / N
            pr = pyoracle.traceback(p, table, uu)
            a = int(pr[i])
            # conditioned on the reference's own draw at i + 1
            b = int(pyoracle.traceback_split(p, table, uu, given=pr)[i])
            ref[a] = ref.get(a, 0) + 1
            dec[b] = dec.get(b, 0) + 1
        keys = set(ref) | set(dec)
        reached = max(reached, len(keys))
        assert max(abs(ref.get(x, 0) - dec.get(x, 0)) for x in keys) <= 3, i
    assert reached >= 10


def test_decomposed_draw_path_is_a_valid_path_on_real_tables():
    # on the real forward table both samplers give paths of positive posterior weight
    p = simulate(8, 400, seed=5, missing=0.005)
    fw, _ = pyoracle.forward(p)
    bw = pyoracle.backward(p)
    post = pyoracle.posterior(p, fw, bw)
    off = pyoracle.offsets(pyoracle.nstates(p))
    u = np.random.default_rng(2).random(p.seqlen)
    path = pyoracle.traceback_split(p, fw, u)
    assert all(post[off[i] + path[i]] > 0 for i in range(p.seqlen))


def test_leaf_cut_is_the_external_problem_in_internal_form():
    # a single-leaf subtree cut: the internal-branch HMM over the main tree equals the
    # external threading HMM of that leaf (same states, same likelihood)
    from argweaver_gb300.sim import leaf_cut

    p = simulate(12, 800, seed=9, missing=0.01)
    q = leaf_cut(p)
    assert q.internal and q.nnodes == p.nnodes + 2
    fe, le = pyoracle.forward(p)
    fi, li = pyoracle.forward(q)
    assert fi.shape == fe.shape
    assert abs(li - le) <= 1e-12 * abs(le)
    np.testing.assert_allclose(fi, fe, rtol=1e-12, atol=0)
