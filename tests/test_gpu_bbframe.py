"""Post-FEC baseband stage on the GPU against the oracle (which
test_oracle_bb.py holds equal to the reference's own code): crafted batches
with failed, corrupted and foreign frames and a short output buffer, and the
whole receive chain end to end (GSE BBFRAMEs encoded, mapped, sent through
AWGN, decoded, checked and unpacked)."""
import numpy as np
import pytest

import cusat_gb300 as cs
import oracle_lib as O
from cusat_gb300 import enums as E
from channel import awgn, es_normalised

pytestmark = pytest.mark.gpu

NORMAL, SHORT = E.FECFRAME_NORMAL, E.FECFRAME_SHORT


def _frames(kbch, B, rng, stride):
    hard = np.zeros((B, stride), np.uint8)
    for f in range(B):
        n = [0, 1, kbch - 10, int(rng.integers(1, kbch - 10))][f % 4]
        hard[f, :kbch] = O.bb_build(rng.integers(0, 256, n, dtype=np.uint8), kbch, ts_gs=3 if f % 11 == 6 else 0)
        hard[f, kbch:] = rng.integers(0, 256, stride - kbch, dtype=np.uint8)
    hard[2::9, 4] ^= 0x01                               # broken headers
    trials = np.where(np.arange(B) % 7 == 3, -1, 4).astype(np.int32)
    valid = np.where(np.arange(B) % 5 == 4, 0, 1).astype(np.int32)
    return hard, trials, valid


@pytest.mark.parametrize("fs,rate", [(NORMAL, E.RATE_3_5), (SHORT, E.RATE_1_2), (NORMAL, E.RATE_9_10)])
@pytest.mark.parametrize("B", [1, 13, 300])
def test_extract_matches_oracle(cuda, fs, rate, B):
    torch = cuda
    ci = cs.code_info(fs, rate)
    kbch, stride = ci["k_bch"] // 8, ci["k_ldpc"] // 8
    hard, trials, valid = _frames(kbch, B, np.random.default_rng(B + rate), stride)
    x = cs.bb_extractor(fs, rate)
    for max_out in (B * kbch, int(B * kbch * 0.3), 0):
        out_o, len_o, off_o = O.bb_extract(hard, kbch, trials, valid, max_out)
        d = [torch.from_numpy(a).cuda() for a in (hard, trials, valid)]
        out = torch.zeros(max(max_out, 1), dtype=torch.uint8, device="cuda")
        lengths = torch.full((B,), -9, dtype=torch.int32, device="cuda")
        offsets = torch.full((B + 1,), -9, dtype=torch.int32, device="cuda")
        x.extract(d[0], stride, d[1], d[2], B, out if max_out else None, max_out, lengths, offsets,
                  torch.cuda.current_stream())
        torch.cuda.synchronize()
        assert (lengths.cpu().numpy() == len_o).all() and (offsets.cpu().numpy() == off_o).all()
        assert (out.cpu().numpy()[:off_o[B]] == out_o).all()


def test_receive_chain_end_to_end(cuda):
    """GSE payloads -> BBFRAMEs -> BCH/LDPC -> 8PSK -> AWGN -> fused demap +
    decode + BCH check -> descramble + unpack: every payload comes back."""
    torch = cuda
    _, mod, rate, _, _, thr = E.find_modcod("8psk3/5")
    fs, B = NORMAL, 24
    ci = cs.code_info(fs, rate)
    kbch = ci["k_bch"] // 8
    rng = np.random.default_rng(4)
    payloads = [rng.integers(0, 256, int(rng.integers(1, kbch - 10)), dtype=np.uint8) for _ in range(B)]
    bbframes = np.stack([O.bb_build(p, kbch) for p in payloads])
    cw = cs.encode_frames(fs, rate, bbframes)
    noisy, n0 = awgn(es_normalised(cs.map_frames(mod, rate, fs, cw)), thr + 0.5, rng)
    rx = cs.rx_fec(mod, rate, fs, 50, B)
    d_sym = torch.from_numpy(noisy).cuda()
    hard = torch.zeros((B, rx.k_bytes), dtype=torch.uint8, device="cuda")
    trials = torch.zeros(B, dtype=torch.int32, device="cuda")
    valid = torch.zeros(B, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream()
    rx.launch(d_sym, B, n0, min(4 / n0, 1000.0), hard, trials, valid, st)
    x = cs.bb_extractor(fs, rate)
    out = torch.zeros(B * kbch, dtype=torch.uint8, device="cuda")
    lengths = torch.zeros(B, dtype=torch.int32, device="cuda")
    offsets = torch.zeros(B + 1, dtype=torch.int32, device="cuda")
    x.extract(hard, rx.k_bytes, trials, valid, B, out, B * kbch, lengths, offsets, st)
    torch.cuda.synchronize()
    assert (trials.cpu().numpy() >= 0).all() and (valid.cpu().numpy() == 1).all()
    L, Off, o = lengths.cpu().numpy(), offsets.cpu().numpy(), out.cpu().numpy()
    for f, p in enumerate(payloads):
        assert L[f] == len(p) and (o[Off[f]:Off[f] + L[f]] == p).all()


@pytest.mark.parametrize("fs,rate", [(NORMAL, E.RATE_1_2), (SHORT, E.RATE_1_2)])
def test_kernel_header_rejections(cuda, fs, rate):
    """The reference parser tests' header cases (valid, largest and empty
    DFL, every single-bit header error, oversize and fractional DFL, non-GSE
    TS/GS) through the device BB stage: the expected lengths and bytes."""
    from test_oracle_bb import header_cases
    torch = cuda
    ci = cs.code_info(fs, rate)
    kbch, stride = ci["k_bch"] // 8, ci["k_ldpc"] // 8
    cases = header_cases(kbch, np.random.default_rng(2))
    B = len(cases)
    hard = np.zeros((B, stride), np.uint8)
    hard[:, :kbch] = np.stack([c[0] for c in cases])
    want = np.array([c[1] for c in cases])
    trials = np.full(B, 5, np.int32)
    valid = np.ones(B, np.int32)
    out_o, len_o, off_o = O.bb_extract(hard, kbch, trials, valid, B * kbch)
    assert (len_o == want).all()
    d = [torch.from_numpy(a).cuda() for a in (hard, trials, valid)]
    out = torch.zeros(B * kbch, dtype=torch.uint8, device="cuda")
    lengths = torch.zeros(B, dtype=torch.int32, device="cuda")
    offsets = torch.zeros(B + 1, dtype=torch.int32, device="cuda")
    cs.bb_extractor(fs, rate).extract(d[0], stride, d[1], d[2], B, out, B * kbch, lengths, offsets,
                                      torch.cuda.current_stream())
    torch.cuda.synchronize()
    assert (lengths.cpu().numpy() == want).all()
    assert (out.cpu().numpy()[:off_o[B]] == out_o).all()
