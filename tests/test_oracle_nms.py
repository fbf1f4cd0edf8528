"""The oracle's FP32/FP64 model of the learned min-sum decoder: its analytic
backward against central finite differences (double), the float copy
against the double copy, and basic invariants."""
import numpy as np
import pytest

import oracle_lib as O
from channel import frames
from cusat_gb300 import enums as E

SHORT, NORMAL = E.FECFRAME_SHORT, E.FECFRAME_NORMAL


def _llr(mod, rate, fs, B, esn0, seed):
    import cusat_gb300 as cs
    _, cw, noisy, n0, gain = frames(mod, rate, fs, B, esn0, seed=seed)
    llr = O.demap_modcod(noisy, O.modcod(mod, rate, fs), n0, gain)
    return llr, cw


def _theta(T, seed):
    rng = np.random.default_rng(seed)
    th = np.zeros((T, 32, 2))
    th[:, :, 0] = rng.uniform(0.2, 1.8, (T, 32))
    th[:, :, 1] = rng.uniform(0.6, 1.0, (T, 32))
    return th


@pytest.mark.parametrize("fs,rate,mod,esn0,iw", [(SHORT, E.RATE_1_2, E.MOD_QPSK, 1.0, None),
                                                 (SHORT, E.RATE_3_5, E.MOD_8PSK, 5.0, None),
                                                 (SHORT, E.RATE_1_2, E.MOD_QPSK, 1.0, [0.0, 0.1, 0.3, 1.0])])
def test_backward_matches_finite_differences(fs, rate, mod, esn0, iw):
    llr, cw = _llr(mod, rate, fs, 2, esn0, seed=3)
    T = 4
    th = _theta(T, 0)
    loss, g = O.nms_train(fs, rate, llr, cw, T, th, dtype=np.float64, iter_w=iw)
    assert loss > 0
    nz = np.argwhere(g != 0)
    assert len(nz) >= 8
    # a step small enough to rarely cross a kink (min/argmin switch, offset
    # threshold, 127 clamp) of the piecewise-linear model, large enough for
    # double rounding
    eps = 1e-6
    rng = np.random.default_rng(1)
    for t, d, k in nz[rng.permutation(len(nz))[:10]]:
        tp, tm = th.copy(), th.copy()
        tp[t, d, k] += eps
        tm[t, d, k] -= eps
        lp, _ = O.nms_train(fs, rate, llr, cw, T, tp, grad=False, dtype=np.float64, iter_w=iw)
        lm, _ = O.nms_train(fs, rate, llr, cw, T, tm, grad=False, dtype=np.float64, iter_w=iw)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[t, d, k]) <= 1e-4 * max(abs(fd), 1e-3 * np.abs(g).max()), (t, d, k, fd, g[t, d, k])


def test_float_copy_matches_double():
    llr, cw = _llr(E.MOD_QPSK, E.RATE_1_2, SHORT, 3, 1.2, seed=8)
    T = 5
    th = _theta(T, 2)
    l64, g64 = O.nms_train(SHORT, E.RATE_1_2, llr, cw, T, th, dtype=np.float64)
    l32, g32 = O.nms_train(SHORT, E.RATE_1_2, llr, cw, T, th.astype(np.float32), dtype=np.float32)
    # the float copy sums the loss sequentially in float (relative error
    # ~1e-4 over N x T terms)
    assert abs(l32 - l64) <= 5e-4 * l64
    assert np.allclose(g32, g64, rtol=1e-3, atol=1e-4 * np.abs(g64).max())


def test_frames_add_up_and_unused_degrees_have_no_gradient():
    llr, cw = _llr(E.MOD_QPSK, E.RATE_1_2, SHORT, 4, 1.2, seed=9)
    T = 3
    th = _theta(T, 4)
    la, ga = O.nms_train(SHORT, E.RATE_1_2, llr[:2], cw[:2], T, th, dtype=np.float64)
    lb, gb = O.nms_train(SHORT, E.RATE_1_2, llr[2:], cw[2:], T, th, dtype=np.float64)
    l, g = O.nms_train(SHORT, E.RATE_1_2, llr, cw, T, th, dtype=np.float64)
    assert abs(l - la - lb) <= 1e-12 * l
    assert np.allclose(g, ga + gb, rtol=1e-10, atol=1e-15)
    info = O.code_info(SHORT, E.RATE_1_2)
    used = np.nonzero(np.abs(g).sum(axis=(0, 2)))[0]
    assert used.max() <= info["cnl"] + 2 and used.min() >= 2


def test_noiseless_frames_have_small_loss():
    """A codeword with loud correct LLRs: the loss is tiny and the gradient
    with respect to the weights nearly zero."""
    import cusat_gb300 as cs
    fs, rate = SHORT, E.RATE_1_2
    ci = cs.code_info(fs, rate)
    rng = np.random.default_rng(0)
    cw = cs.encode_frames(fs, rate, rng.integers(0, 256, (1, ci["k_bch"] // 8), dtype=np.uint8))
    bits = np.unpackbits(cw, axis=1)[:, :ci["n_ldpc"]]
    llr = np.where(bits == 0, 60, -60).astype(np.int16)
    loss, g = O.nms_train(fs, rate, llr, cw, 3, _theta(3, 1), dtype=np.float64)
    assert loss < 1e-20
    assert np.abs(g).max() < 1e-20


def test_iteration_weights_are_linear():
    """The loss is linear in the iteration weights: uniform weights equal the
    default, and a weight vector's loss is the weighted sum of one-hot ones."""
    llr, cw = _llr(E.MOD_QPSK, E.RATE_1_2, SHORT, 2, 1.2, seed=5)
    T = 3
    th = _theta(T, 6)
    l0, g0 = O.nms_train(SHORT, E.RATE_1_2, llr, cw, T, th, dtype=np.float64)
    lu, gu = O.nms_train(SHORT, E.RATE_1_2, llr, cw, T, th, dtype=np.float64, iter_w=[1 / T] * T)
    assert abs(l0 - lu) <= 1e-12 * l0 and np.allclose(g0, gu, rtol=1e-10, atol=1e-16)
    w = np.array([0.2, 0.5, 1.5])
    lw, gw = O.nms_train(SHORT, E.RATE_1_2, llr, cw, T, th, dtype=np.float64, iter_w=w)
    ls, gs = 0.0, np.zeros_like(gw)
    for t in range(T):
        e = np.zeros(T)
        e[t] = w[t]
        lt, gt = O.nms_train(SHORT, E.RATE_1_2, llr, cw, T, th, dtype=np.float64, iter_w=e)
        ls += lt
        gs += gt
    assert abs(lw - ls) <= 1e-10 * lw and np.allclose(gw, gs, rtol=1e-9, atol=1e-15)
