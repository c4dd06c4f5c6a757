"""The network oracle (oracle/mpnn.py) against itself: its hand-derived backward
pass agrees with finite differences of its forward pass (plain float64), and the
BF16-rounded variant stays close to the plain one."""
import numpy as np
import pytest

from oracle import mpnn as M
from senk_gb300 import problems as P


def _case(seed=0):
    A = P.vardiff3d(8, 1.0, 3.0, seed)
    g = M.Graph(A.val, A.cind, A.rptr)
    rng = np.random.default_rng(seed + 1)
    r = rng.standard_normal(A.n)
    ilu = rng.standard_normal(A.n) * 0.1
    e = ilu + rng.standard_normal(A.n) * 0.05
    params = M.init_params(seed).astype(np.float64)
    params[M.OFF_WOUT:M.OFF_BOUT] = rng.normal(0, 0.1, M.HID)  # let gradients reach every layer
    params[M.OFF_BOUT] = 0.01
    return g, r, ilu, e, params


@pytest.mark.parametrize("mode", [0, 1])
def test_backward_matches_finite_differences(mode):
    g, r, ilu, e, params = _case()
    loss, G = M.loss_grad(params, g, r, ilu, e, rounding=False, mode=mode)
    rng = np.random.default_rng(7)
    eps = 1e-6
    for _ in range(4):
        v = rng.standard_normal(M.NPARAMS)
        v /= np.linalg.norm(v)
        lp, _ = M.loss_grad(params + eps * v, g, r, ilu, e, rounding=False, mode=mode)
        lm, _ = M.loss_grad(params - eps * v, g, r, ilu, e, rounding=False, mode=mode)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - G @ v) <= 1e-5 * max(1.0, abs(fd))
    # every parameter block receives gradient
    for lo, hi in [(M.OFF_WIN, M.OFF_BIN), (M.OFF_LAYER, M.OFF_LAYER + M.LAYER_SIZE),
                   (M.OFF_LAYER + 3 * M.LAYER_SIZE, M.OFF_WOUT), (M.OFF_WOUT, M.OFF_BOUT)]:
        assert np.linalg.norm(G[lo:hi]) > 0


def test_rounded_network_stays_close():
    g, r, ilu, e, params = _case(1)
    a, _ = M.forward(params, g, r, rounding=False)
    b, _ = M.forward(params, g, r, rounding=True)
    assert np.linalg.norm(a - b) <= 2e-2 * np.linalg.norm(a)
    la, Ga = M.loss_grad(params, g, r, ilu, e, rounding=False)
    lb, Gb = M.loss_grad(params, g, r, ilu, e, rounding=True)
    assert abs(la - lb) <= 2e-2 * la
    assert np.linalg.norm(Ga - Gb) <= 5e-2 * np.linalg.norm(Ga)


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2**-8, 1.0 + 3 * 2**-8, -2.5, 3.0e-3], np.float64)
    y = M.bf16(x)
    assert y[0] == 1.0 and y[1] == 1.0 and y[2] == 1.0 + 2**-6 and y[3] == -2.5
    assert abs(y[4] - 3.0e-3) <= 3.0e-3 * 2**-8


def test_learned_gcr_history_is_iluGcrm_between_restarts():
    """oracle/learned_gcr.py's per-iteration GCR with K = ILU(0) is the oracle's
    IluGcrm (senk_gcr.hpp:93-161) observed every iteration: its first iteration
    below eps, rounded up to a restart, is IluGcrm's count; within a cycle the
    residual never grows (GCR minimises it over the directions of the cycle)."""
    import oracle
    from oracle import learned_gcr as LG
    from senk_gb300.learned import family_member

    mb = family_member(8, 1234)
    pt = oracle.port()
    m, eps = 5, 1e-8
    ilu = lambda r: pt.ilu_apply(mb.L, mb.U, r, mb.cptr, mb.cnum, 16)
    h = LG.gcr_history(mb.A, mb.b, ilu, m, 80)
    k = LG.first_below(h, eps)
    assert k > 0
    nb = float(np.linalg.norm(mb.b))
    _, it, _, conv = pt.solve("gcr", mb.A, mb.b, L=mb.L, U=mb.U, pc=oracle.PC_ILU_ABMC, cptr=mb.cptr, cnum=mb.cnum,
                              bsize=16, outer=80 // m, m=m, eps=eps, nrm_b=nb)
    assert conv and it == -(-k // m) * m
    for c in range(0, 80, m):
        assert np.all(np.diff(h[c:c + m + 1]) <= 1e-12 * h[c])


def test_least_squares_step_never_worsens_one_application():
    """|r - A K(r)| with K = ILU + alpha c (alpha the least-squares step) is at
    most |r - A ILU(r)|, whatever the network's output; the fixed step has no
    such bound."""
    g, r, ilu, e, params = _case(3)
    params[M.OFF_WOUT:M.OFF_BOUT] = 50.0  # a large, useless correction
    base = np.linalg.norm(r - g.A @ ilu)
    ks = M.apply_step(params, g, r, ilu, rounding=False)
    kf = M.apply(params, g, r, ilu, rounding=False)
    assert np.linalg.norm(r - g.A @ ks) <= base * (1 + 1e-12)
    assert np.linalg.norm(r - g.A @ kf) > base


@pytest.mark.parametrize("step", [0, 1])
def test_untrained_network_leaves_gcr_as_plain_ilu(step):
    """The initial parameters have a zero output layer, so K = ILU exactly under
    either step and the GCR residual histories coincide."""
    from oracle import learned_gcr as LG
    from senk_gb300.learned import family_member

    c = LG.compare(M.init_params(0).astype(np.float64), family_member(8, 4321), m=5, iters=40, step=step)
    assert c["plain_iters"] == c["learned_iters"] > 0
    assert np.allclose(c["plain_res"], c["learned_res"], rtol=1e-12, atol=0)
