"""Learned min-sum training kernels against the oracle's FP32 model.

The GPU forward/backward (cusat_nms_train_step) and the oracle's
orc_nms_train_f32 evaluate the same unrolled model; they differ only in the
order of floating-point additions (atomics on the GPU) and in expf/log1pf
rounding, so losses and gradients agree to a relative 1e-3.  The oracle's
analytic backward itself is checked against finite differences in
test_oracle_nms.py."""
import numpy as np
import pytest

import cusat_gb300 as cs
import oracle_lib as O
from channel import frames
from cusat_gb300 import enums as E
from cusat_gb300 import learned
from test_gpu_parity import oracle_llr

pytestmark = pytest.mark.gpu

NORMAL, SHORT = E.FECFRAME_NORMAL, E.FECFRAME_SHORT


def random_theta(T, seed):
    rng = np.random.default_rng(seed)
    th = np.zeros((T, 32, 2), np.float32)
    th[:, :, 0] = rng.uniform(0.0, 2.0, (T, 32))
    th[:, :, 1] = rng.uniform(0.55, 1.05, (T, 32))
    return th


def gpu_loss_grad(torch, fs, rate, llr, cw, T, theta, with_grad=True, iter_w=None):
    B = llr.shape[0]
    tr = learned.nms_trainer(fs, rate, T, B)
    d_llr = torch.from_numpy(np.ascontiguousarray(llr)).cuda()
    d_cw = torch.from_numpy(np.ascontiguousarray(cw)).cuda()
    th = torch.from_numpy(theta).cuda()
    g = torch.zeros_like(th) if with_grad else None
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    iw = None if iter_w is None else torch.tensor(np.asarray(iter_w, np.float32), device="cuda")
    tr.step(d_llr, d_cw, B, th, g, loss, torch.cuda.current_stream(), iter_w=iw)
    torch.cuda.synchronize()
    return float(loss.item()), (g.cpu().numpy() if with_grad else None), tr


@pytest.mark.parametrize("name,fs,esn0,B,T", [("qpsk1/2", SHORT, 0.8, 3, 4), ("8psk3/5", NORMAL, 5.4, 2, 3),
                                              ("16apsk3/4", NORMAL, 10.2, 2, 3), ("qpsk1/3", NORMAL, 0.3, 2, 3)])
def test_gradients_match_oracle(cuda, name, fs, esn0, B, T):
    torch = cuda
    _, mod, rate, _, _, _ = E.find_modcod(name)
    _, cw, noisy, n0, gain = frames(mod, rate, fs, B, esn0, seed=21)
    llr = oracle_llr(mod, rate, fs, noisy, n0, gain)
    theta = random_theta(T, rate)
    lg, gg, tr = gpu_loss_grad(torch, fs, rate, llr, cw, T, theta)
    lc, gc = O.nms_train(fs, rate, llr, cw, T, theta, dtype=np.float32, nthreads=16)
    assert abs(lg - lc) <= 1e-3 * abs(lc)  # the oracle sums the loss sequentially in float
    scale = np.abs(gc).max()
    assert scale > 0
    assert np.allclose(gg, gc, rtol=1e-3, atol=1e-3 * scale), np.abs(gg - gc).max() / scale
    # only the code's check degrees carry gradient
    deg = np.nonzero(np.abs(gc).sum(axis=(0, 2)))[0]
    assert deg.min() >= tr.deg_lo and deg.max() <= tr.deg_hi
    # forward only: same loss
    lf, _, _ = gpu_loss_grad(torch, fs, rate, llr, cw, T, theta, with_grad=False)
    assert abs(lf - lg) <= 1e-6 * abs(lg)


def test_iteration_weights_match_oracle(cuda):
    torch = cuda
    fs, rate, T, B = SHORT, E.RATE_1_2, 5, 3
    _, cw, noisy, n0, gain = frames(E.MOD_QPSK, rate, fs, B, 0.9, seed=9)
    llr = oracle_llr(E.MOD_QPSK, rate, fs, noisy, n0, gain)
    theta = random_theta(T, 4)
    iw = [0.0, 0.05, 0.1, 0.35, 1.0]
    lg, gg, _ = gpu_loss_grad(torch, fs, rate, llr, cw, T, theta, iter_w=iw)
    lc, gc = O.nms_train(fs, rate, llr, cw, T, theta, dtype=np.float32, iter_w=iw)
    assert abs(lg - lc) <= 1e-3 * abs(lc)
    assert np.allclose(gg, gc, rtol=1e-3, atol=1e-3 * np.abs(gc).max())


def test_plain_theta_is_exact(cuda):
    """With beta 1, alpha 1 every value of the model is an integer below 2^24:
    GPU and oracle follow the same trajectory exactly, so the gradients
    differ only by the order of their float sums."""
    torch = cuda
    fs, rate, T, B = SHORT, E.RATE_1_2, 6, 4
    _, cw, noisy, n0, gain = frames(E.MOD_QPSK, rate, fs, B, 1.0, seed=4)
    llr = oracle_llr(E.MOD_QPSK, rate, fs, noisy, n0, gain)
    theta = learned.plain_theta(T)
    lg, gg, _ = gpu_loss_grad(torch, fs, rate, llr, cw, T, theta)
    lc, gc = O.nms_train(fs, rate, llr, cw, T, theta, dtype=np.float32)
    assert abs(lg - lc) <= 1e-3 * abs(lc)
    assert np.allclose(gg, gc, rtol=1e-4, atol=1e-5 * np.abs(gc).max())


def test_training_lowers_loss_and_quantises(cuda):
    """A short training run on the GPU lowers the model's loss on held-out
    frames; the quantised table drives the integer decoder."""
    torch = cuda
    name, fs, T = "qpsk1/2", SHORT, 10
    theta, hist = learned.train(name, fs, n_iter=T, n_frames=64 * 40, batch=64, lr=0.03, seed=3, log=None)
    assert theta.shape == (T, 32, 2)
    pool = learned.ChannelPool(name, fs, 64, 99, 64, torch)
    tr = learned.nms_trainer(fs, pool.rate, T, 64)
    thr = E.find_modcod(name)[5]
    losses = {}
    for key, th in (("plain", learned.plain_theta(T)), ("learned", theta)):
        d_th = torch.from_numpy(np.ascontiguousarray(th, np.float32)).cuda()
        loss = torch.zeros(1, dtype=torch.float32, device="cuda")
        pool.gen.manual_seed(5)
        for k in range(4):
            _, llr, cw, _, _ = pool.draw(64, thr + 0.25 * k - 0.25)
            tr.step(llr, cw, 64, d_th, None, loss)
        losses[key] = float(loss.item())
    assert losses["learned"] < losses["plain"], losses
    w = learned.quantize(theta)
    assert w.dtype == np.int16 and (w[..., 1] >= 1).all()
    res = learned.frame_errors(name, fs, thr + 0.5, T, w, n_frames=512, batch=128)
    assert res["frames"] == 512 and 0 <= res["fer"] <= 1


def test_committed_weights_beat_plain(cuda):
    """The adopted weights of normal QPSK 1/3 (trained on 1e6 frames by the
    kernels above): 0.25 dB below the MODCOD's threshold the learned decoder
    capped at 20 iterations decodes frames that the plain decoder capped at 50
    loses, and at the threshold it needs fewer than half the iterations."""
    name, fs = "qpsk1/3", NORMAL
    w = learned.load_weights(name, fs)
    assert w is not None and w.shape == (20, 32, 2)
    thr = E.find_modcod(name)[5]
    low_p = learned.frame_errors(name, fs, thr - 0.25, 50, None, n_frames=512, batch=256, seed=31)
    low_l = learned.frame_errors(name, fs, thr - 0.25, 20, w, n_frames=512, batch=256, seed=31)
    assert low_p["fer"] > 0.2 and low_l["frame_errors"] <= 2, (low_p, low_l)
    at_p = learned.frame_errors(name, fs, thr, 50, None, n_frames=512, batch=256, seed=32)
    at_l = learned.frame_errors(name, fs, thr, 20, w, n_frames=512, batch=256, seed=32)
    assert at_l["frame_errors"] <= at_p["frame_errors"]
    assert at_l["mean_iterations"] < 0.5 * at_p["mean_iterations"], (at_p, at_l)
    # a weight file that lost to the plain decoder is not loaded
    assert learned.load_weights("16apsk3/4", NORMAL) is None
    assert learned.load_weights("16apsk3/4", NORMAL, adopted_only=False) is not None


def test_degree_counts_and_ties(cuda):
    tr = learned.nms_trainer(NORMAL, E.RATE_3_5, 3, 2)
    ci = cs.code_info(NORMAL, E.RATE_3_5)
    assert sum(tr.degree_counts) == ci["n_ldpc"] - ci["k_ldpc"]
    assert tr.degree_counts[11] == ci["n_ldpc"] - ci["k_ldpc"] - 1 and tr.degree_counts[10] == 1
    assert tr.tied_degrees() == {10: 11}
    short = learned.nms_trainer(SHORT, E.RATE_1_2, 3, 2)
    assert sum(short.degree_counts) == 16200 - 7200
    for d, up in short.tied_degrees().items():
        assert short.degree_counts[d] < 360 <= short.degree_counts[up]
