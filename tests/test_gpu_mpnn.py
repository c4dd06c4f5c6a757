"""The learned preconditioner on the GPU: the tcgen05 BF16 GEMMs against a plain
PyTorch FP32 product of the same BF16 inputs, the network's output, loss and
gradient against the CPU oracle (oracle/mpnn.py, BF16 rounding points
reproduced), training, and flexible GCR with K = ILU + net."""
import numpy as np
import pytest

from oracle import mpnn as M
from senk_gb300 import learned as LN
from senk_gb300 import lib as L
from senk_gb300 import problems as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("n,K,NO", [(1000, 128, 64), (4096, 128, 64), (1000, 64, 128), (257, 64, 128)])
def test_tc_gemm_matches_fp32_product(torch, n, K, NO):
    g = torch.Generator(device="cuda").manual_seed(n + K)
    A = torch.randn(n, K, device="cuda", generator=g).to(torch.bfloat16).contiguous()
    Bt = torch.randn(NO, K, device="cuda", generator=g).to(torch.bfloat16).contiguous()
    C = torch.full((n, NO), float("nan"), device="cuda", dtype=torch.float32)
    L.check("gemm", L.lib().senk_dev_gemm_bf16(A.data_ptr(), Bt.data_ptr(), C.data_ptr(), n, K, NO, None))
    want = A.float() @ Bt.float().T
    torch.cuda.synchronize()
    err = (C - want).abs().max().item() / want.abs().max().item()
    assert err <= 1e-5, err


@pytest.mark.parametrize("n", [64, 1000, 70000])
def test_tc_gemm_tn_matches_fp32_product(torch, n):
    g = torch.Generator(device="cuda").manual_seed(n)
    X = torch.randn(n, 128, device="cuda", generator=g).to(torch.bfloat16).contiguous()
    dZ = torch.randn(n, 64, device="cuda", generator=g).to(torch.bfloat16).contiguous()
    out = torch.full((128, 64), float("nan"), device="cuda", dtype=torch.float32)
    L.check("gemm_tn", L.lib().senk_dev_gemm_tn_bf16(X.data_ptr(), dZ.data_ptr(), out.data_ptr(), n, None))
    want = X.float().T @ dZ.float()
    torch.cuda.synchronize()
    err = (out - want).abs().max().item() / want.abs().max().item()
    assert err <= 1e-5, err


@pytest.fixture(scope="module")
def small_member():
    return LN.family_member(16, 11)


def _trained_like_params(seed=3):
    p = M.init_params(seed)
    rng = np.random.default_rng(seed)
    p[M.OFF_WOUT:M.OFF_BOUT] = rng.normal(0, 0.1, M.HID)
    p[M.OFF_BOUT] = 0.01
    return p


def _grad_blocks():
    """Parameter blocks with their bars (relative max-norm error against the
    oracle, which reproduces every BF16 rounding point). The decoder's
    gradients are FP32 sums of FP32 terms. Every other block's gradient flows
    back through the layers' BF16 tensor-core products (the layer weights are
    such a product, X^T dZ, themselves), so its terms carry BF16-rounded
    operands summed in FP32 in a different order than the oracle's. Measured
    on this system: decoder at most 1.7e-6, the others at most 2.2e-4."""
    out = [("W_in", M.OFF_WIN, M.OFF_BIN, GRAD_BAR_BF16_PATH), ("b_in", M.OFF_BIN, M.OFF_LAYER, GRAD_BAR_BF16_PATH)]
    for l in range(M.LAYERS):
        base = M.OFF_LAYER + l * M.LAYER_SIZE
        out.append((f"Theta{l}", base, base + 2 * M.HID * M.HID, GRAD_BAR_BF16_PATH))
        out.append((f"beta{l}", base + 2 * M.HID * M.HID, base + M.LAYER_SIZE, GRAD_BAR_BF16_PATH))
    out += [("w_out", M.OFF_WOUT, M.OFF_BOUT, GRAD_BAR_FP32), ("b_out", M.OFF_BOUT, M.NPARAMS, GRAD_BAR_FP32)]
    return out


GRAD_BAR_BF16_PATH = 1e-3
GRAD_BAR_FP32 = 1e-5


def test_network_output_loss_and_gradient_match_oracle(torch, small_member):
    mb = small_member
    sysm = LN.make_system(mb)
    params = _trained_like_params()
    net = LN.Net(params)
    try:
        net.bind(sysm)
        net.set_step(0)
        rng = np.random.default_rng(5)
        r = rng.standard_normal(mb.A.n)
        e = rng.standard_normal(mb.A.n) * 0.05
        rd, ed = LN._dev(torch, r), LN._dev(torch, e)
        out = torch.zeros_like(rd)
        net.apply(sysm, rd.data_ptr(), out.data_ptr())
        import oracle
        port = oracle.port()
        ilu_h = port.ilu_apply(mb.L, mb.U, r, mb.cptr, mb.cnum, 16)
        g = M.Graph(mb.A.val, mb.A.cind, mb.A.rptr)
        want = M.apply(params, g, r, ilu_h, rounding=True)
        got = out.cpu().numpy()
        corr_got, corr_want = got - ilu_h, want - ilu_h
        assert rel(corr_got, corr_want) <= 1e-2
        assert rel(got, want) <= 1e-3
        # the least-squares step, element by element: K(r) = ILU(r) + alpha c with
        # alpha = (q . Ac) / (Ac . Ac), q = r - A ILU(r), in FP64 on the host
        net.set_step(1)
        out1 = torch.zeros_like(rd)
        net.apply(sysm, rd.data_ptr(), out1.data_ptr())
        got1 = out1.cpu().numpy()
        q = r - mb.A.matvec(ilu_h)
        ac = mb.A.matvec(corr_want)
        alpha = float(q @ ac / (ac @ ac))
        want1 = ilu_h + alpha * corr_want
        alpha_got = float((got1 - ilu_h) @ corr_want / (corr_want @ corr_want))
        assert abs(alpha_got - alpha) <= 1e-2 * abs(alpha), (alpha_got, alpha)
        assert rel(got1, want1) <= 1e-3
        # one application leaves no larger residual than ILU(r) alone
        assert np.linalg.norm(r - mb.A.matvec(got1)) <= np.linalg.norm(q) * (1 + 1e-6)
        for mode in (1, 0):
            net.set_loss(mode)
            loss, grad = net.loss_grad(sysm, rd.data_ptr(), ed.data_ptr())
            lw, gw = M.loss_grad(params, g, r, ilu_h, e, rounding=True, mode=mode)
            assert abs(loss - lw) <= 1e-3 * lw, (mode, loss, lw)
            for name, lo, hi, bar in _grad_blocks():
                err = rel(grad[lo:hi], gw[lo:hi])
                print(f"gradient {name} [{lo}, {hi}) mode {mode}: {err:.2e} (bar {bar:.0e})")
                assert err <= bar, (mode, name, err)
    finally:
        net.close()
        sysm.close()


def test_training_lowers_the_loss_and_flexible_gcr_converges(torch):
    net = LN.Net(seed=0)
    try:
        losses = LN.train(torch, net, 16, seeds=range(100, 116), epochs=3, lr=3e-4)
        first, last = np.mean(losses[:8]), np.mean(losses[-8:])
        assert np.isfinite(last) and last < first
        for s in (900, 901):
            mb = LN.family_member(16, s)
            c = LN.compare_gcr(net, mb, m=20)
            assert c["plain"]["converged"] and c["plain"]["true_res"] < 1e-8
            assert c["learned"]["converged"] and c["learned"]["true_res"] < 1e-8
    finally:
        net.close()


def test_least_squares_step_gcr_converges(torch):
    """K = ILU + alpha c with the least-squares alpha (senk_mpnn_set_step 1),
    computed on the device inside the GCR cycle graph: the solve converges to
    the FP64 true residual, in no more restart cycles than one over plain ILU."""
    net = LN.Net(seed=0)
    try:
        LN.train(torch, net, 16, seeds=range(100, 116), epochs=3, lr=3e-4)
        net.set_step(1)  # (the default)
        for s in (900, 901):
            c = LN.compare_gcr(net, LN.family_member(16, s), m=20)
            assert c["learned"]["converged"] and c["learned"]["true_res"] < 1e-8
            assert c["learned"]["iters"] <= c["plain"]["iters"] + 20
    finally:
        net.close()


def test_stagnating_network_falls_back_to_plain_ilu(torch):
    mb = LN.family_member(16, 902)
    p = M.init_params(1)
    p[M.OFF_WOUT:M.OFF_BOUT] = 50.0  # a large, useless correction
    net = LN.Net(p)
    net.set_step(0)  # the fixed step: the least-squares step would only shrink it
    try:
        c = LN.compare_gcr(net, mb, m=20, stall=0.9)
        assert c["learned"]["converged"] and c["learned"]["true_res"] < 1e-8
        assert c["learned"]["fallback_cycle"] >= 1
    finally:
        net.close()
