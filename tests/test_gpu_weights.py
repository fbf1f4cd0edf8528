"""Learned min-sum weights in the integer decoder: bit-exact with the oracle's
weighted decoder (same {beta, alpha/64} per iteration and check degree), in
the plain decoder, the fused chain and mixed batches."""
import numpy as np
import pytest

import cusat_gb300 as cs
import oracle_lib as O
from channel import frames
from cusat_gb300 import enums as E
from test_gpu_parity import assert_same, gpu_decode, oracle_llr

pytestmark = pytest.mark.gpu

NORMAL, SHORT = E.FECFRAME_NORMAL, E.FECFRAME_SHORT


def random_weights(T, seed):
    rng = np.random.default_rng(seed)
    w = np.zeros((T, 32, 2), np.int16)
    w[:, :, 0] = rng.integers(0, 4, (T, 32))
    w[:, :, 1] = rng.integers(36, 72, (T, 32))
    w[rng.random((T, 32)) < 0.1, 1] = 0  # some entries unscaled
    return w


def expand(w, T):
    return np.concatenate([w, np.repeat(w[-1:], T - len(w), axis=0)]) if len(w) < T else w[:T]


def decode_weighted(torch, fs, rate, llr, T, w):
    B = llr.shape[0]
    dec = cs.ldpc_decode_cuda(fs, rate, T, B)
    dec.set_weights(w)
    d_llr = torch.from_numpy(np.ascontiguousarray(llr)).cuda()
    hard = torch.zeros((B, dec.k_bytes()), dtype=torch.uint8, device="cuda")
    trials = torch.zeros(B, dtype=torch.int32, device="cuda")
    dec.decode_launch_async(d_llr, B, torch.cuda.current_stream(), hard, trials)
    torch.cuda.synchronize()
    return dec, hard.cpu().numpy(), trials.cpu().numpy()


@pytest.mark.parametrize("fs,rate,mod,esn0,B", [(SHORT, E.RATE_1_2, E.MOD_QPSK, 1.5, 32),
                                                (NORMAL, E.RATE_3_5, E.MOD_8PSK, 6.0, 12),
                                                (NORMAL, E.RATE_3_4, E.MOD_16APSK, 10.4, 8),
                                                (NORMAL, E.RATE_1_3, E.MOD_QPSK, 0.6, 8)])
def test_weighted_decoder_matches_oracle(cuda, fs, rate, mod, esn0, B):
    torch = cuda
    T = 20
    _, _, noisy, n0, gain = frames(mod, rate, fs, B, esn0, seed=77 + rate)
    llr = oracle_llr(mod, rate, fs, noisy, n0, gain)
    w = random_weights(T, rate)
    dec, h, t = decode_weighted(torch, fs, rate, llr, T, w)
    ho, to = O.ldpc_decode(fs, rate, llr, T, weights=w, nthreads=16)
    assert_same(h, t, ho, to)
    # fewer rows than iterations: later iterations reuse the last row
    dec.set_weights(w[:5])
    d_llr = torch.from_numpy(llr).cuda()
    hard = torch.zeros((B, dec.k_bytes()), dtype=torch.uint8, device="cuda")
    trials = torch.zeros(B, dtype=torch.int32, device="cuda")
    dec.decode_launch_async(d_llr, B, torch.cuda.current_stream(), hard, trials)
    torch.cuda.synchronize()
    ho, to = O.ldpc_decode(fs, rate, llr, T, weights=expand(w[:5], T), nthreads=16)
    assert_same(hard.cpu().numpy(), trials.cpu().numpy(), ho, to)
    # back to the plain decoder
    dec.set_weights(None)
    dec.decode_launch_async(d_llr, B, torch.cuda.current_stream(), hard, trials)
    torch.cuda.synchronize()
    ho, to = O.ldpc_decode(fs, rate, llr, T, nthreads=16)
    assert_same(hard.cpu().numpy(), trials.cpu().numpy(), ho, to)


def test_weighted_saturating_path(cuda):
    """Loud LLRs take the saturating instantiation; weights apply there too."""
    torch = cuda
    fs, rate, T = SHORT, E.RATE_1_2, 12
    rng = np.random.default_rng(5)
    info = cs.code_info(fs, rate)
    cw = O.ldpc_encode(fs, rate, rng.integers(0, 256, (6, info["k_ldpc"] // 8), dtype=np.uint8))
    bits = np.unpackbits(cw, axis=1)[:, :info["n_ldpc"]]
    llr = np.where(bits == 0, 1, -1).astype(np.int32) * rng.integers(20000, 32768, bits.shape)
    flip = rng.random(bits.shape) < 0.08
    llr = np.where(flip, -llr, llr).astype(np.int16)
    w = random_weights(T, 11)
    _, h, t = decode_weighted(torch, fs, rate, llr, T, w)
    ho, to = O.ldpc_decode(fs, rate, llr, T, weights=w, nthreads=16)
    assert_same(h, t, ho, to)


def test_weighted_chain_and_batch(cuda):
    torch = cuda
    T = 20
    cases = [("8psk3/5", NORMAL, 6), ("qpsk1/2", SHORT, 6)]
    table, data = [], []
    for name, fs, B in cases:
        _, mod, rate, _, _, thr = E.find_modcod(name)
        _, _, noisy, n0, gain = frames(mod, rate, fs, B, thr + 0.2, seed=5)
        table.append((mod, rate, fs))
        data.append((noisy, n0, gain))
    w = random_weights(T, 3)
    # fused chain, learned
    mod, rate, fs = table[0]
    noisy, n0, gain = data[0]
    rx = cs.rx_fec(mod, rate, fs, T, len(noisy))
    rx.set_weights(w)
    d = torch.from_numpy(noisy).cuda()
    hard = torch.zeros((len(noisy), rx.k_bytes), dtype=torch.uint8, device="cuda")
    trials = torch.zeros(len(noisy), dtype=torch.int32, device="cuda")
    rx.launch(d, len(noisy), n0, gain, hard, trials, None, torch.cuda.current_stream())
    torch.cuda.synchronize()
    llr0 = oracle_llr(mod, rate, fs, noisy, n0, gain)
    ho0, to0 = O.ldpc_decode(fs, rate, llr0, T, weights=w, nthreads=16)
    assert_same(hard.cpu().numpy(), trials.cpu().numpy(), ho0, to0)
    # batch: MODCOD 0 learned, MODCOD 1 plain
    b = cs.batch(table, max_trials=T, max_frames=32)
    b.set_weights(0, w)
    outs, cols = [], [[] for _ in range(7)]
    for m, ((mod, rate, fs), (noisy, n0, gain)) in enumerate(zip(table, data)):
        kb = cs.code_info(fs, rate)["k_ldpc"] // 8
        d = torch.from_numpy(noisy).cuda()
        h = torch.zeros((len(noisy), kb), dtype=torch.uint8, device="cuda")
        t = torch.zeros(len(noisy), dtype=torch.int32, device="cuda")
        outs.append((d, h, t))
        for i in range(len(noisy)):
            for c, v in zip(cols, [m, n0, gain, d[i].data_ptr(), h[i].data_ptr(), t[i].data_ptr(), None]):
                c.append(v)
    torch.cuda.synchronize()
    b.launch(cs.batch.frames(*cols), torch.cuda.current_stream())
    torch.cuda.synchronize()
    assert_same(outs[0][1].cpu().numpy(), outs[0][2].cpu().numpy(), ho0, to0)
    mod, rate, fs = table[1]
    noisy, n0, gain = data[1]
    ho1, to1 = O.ldpc_decode(fs, rate, oracle_llr(mod, rate, fs, noisy, n0, gain), T, nthreads=16)
    assert_same(outs[1][1].cpu().numpy(), outs[1][2].cpu().numpy(), ho1, to1)


def test_invalid_weights_rejected(cuda):
    dec = cs.ldpc_decode_cuda(SHORT, E.RATE_1_2, 10, 4)
    w = random_weights(10, 1)
    w[3, 7, 0] = 200
    with pytest.raises(cs.CusatError):
        dec.set_weights(w)
    w = random_weights(10, 1)
    w[0, 0, 1] = -1
    with pytest.raises(cs.CusatError):
        dec.set_weights(w)
