"""The PL receiver tail kernel (cusat_pl_extract) against the oracle, bit for
bit: descrambling, pilot removal and per-slot counter-rotation of located
PLFRAMEs, and the whole receive path from scrambled PLFRAME payloads with
pilots to decoded frames."""
import numpy as np
import pytest

import cusat_gb300 as cs
import oracle_lib as O
from cusat_gb300 import enums as E

pytestmark = pytest.mark.gpu

# PLS codes: 8PSK 3/5 normal + pilots, QPSK 1/4 normal + pilots (360 slots,
# the longest payload), 16APSK 2/3 short + pilots, QPSK 1/2 short without,
# 128APSK 3/4 + pilots (103 slots), 256APSK 3/4 without pilots
CODES = [(12 << 2) | 1, (1 << 2) | 1, (18 << 2) | 3, (4 << 2) | 2, 200 | 1, 214]
GOLDS = [0, 77777, 262141]


def _slot_rot(rng, slots):
    ang = rng.uniform(-3.2, 3.2, slots)
    stp = rng.uniform(-0.02, 0.02, slots)
    g = rng.uniform(0.5, 2.0, slots)
    return np.stack([g * np.cos(ang), g * np.sin(ang), np.cos(stp), np.sin(stp)], 1).astype(np.float32).reshape(-1)


def test_extract_matches_oracle(cuda):
    torch = cuda
    rng = np.random.default_rng(4)
    x = cs.pl_extractor(GOLDS, max_frames=64)
    pays, datas, rots, codes, golds, want = [], [], [], [], [], []
    for k, code in enumerate(CODES * 2):
        l = cs.pl_layout(code)
        gold = GOLDS[k % len(GOLDS)]
        pay = (rng.standard_normal(2 * l["payload_symbols"]) * rng.uniform(0.2, 5)).astype(np.float32)
        if k == 3:
            pay[11] = np.inf
            pay[400] = np.nan
        rot = _slot_rot(rng, l["slots"]) if k % 2 else None
        r = O.pl_rotation(gold, l["payload_symbols"])
        want.append(O.pl_extract(pay, l["slots"], l["pilots"], r, rot))
        pays.append(torch.from_numpy(pay).cuda())
        datas.append(torch.full((2 * l["data_symbols"],), 7.0, dtype=torch.float32, device="cuda"))
        rots.append(None if rot is None else torch.from_numpy(rot).cuda())
        codes.append(code)
        golds.append(gold)
    frames = x.frames(pays, datas, codes, golds, rots)
    x.extract(frames, torch.cuda.current_stream())
    torch.cuda.synchronize()
    for k, w in enumerate(want):
        got = datas[k].cpu().numpy()
        assert (got.view(np.uint32) == w.view(np.uint32)).all(), f"frame {k} (PLS code {codes[k]})"


def test_plframes_through_the_receive_path(cuda):
    """Scrambled PLFRAME payloads with pilots -> cusat_pl_extract ->
    demap -> decode -> BCH equals the receive path fed with the XFECFRAMEs
    themselves (the headline frames: 8PSK 3/5 normal, 6.0 dB)."""
    torch = cuda
    import bench
    wl = dict(bench.WORKLOAD, frames=48)
    ci, msg, bufs, n0, gain = bench.make_traffic(wl, 1, bench.ProductGen())
    sym = bufs[0]
    code, gold = (12 << 2) | 1, 3
    l = cs.pl_layout(code)
    r = O.pl_rotation(gold, l["payload_symbols"])
    pays = [torch.from_numpy(O.pl_frame_payload(sym[f], l["slots"], 1, r)).cuda() for f in range(len(sym))]
    B = len(sym)
    d_data = torch.zeros((B, 2 * l["data_symbols"]), dtype=torch.float32, device="cuda")
    x = cs.pl_extractor([5, gold], max_frames=B)
    x.extract(x.frames(pays, [d_data[f] for f in range(B)], [code] * B, [gold] * B), torch.cuda.current_stream())
    torch.cuda.synchronize()
    assert np.array_equal(d_data.cpu().numpy(), sym)
    rx = cs.rx_fec(wl["mod"], wl["rate"], wl["fs"], wl["max_trials"], B)
    outs = []
    for src in (d_data, torch.from_numpy(sym).cuda()):
        hard = torch.zeros((B, ci["k_ldpc"] // 8), dtype=torch.uint8, device="cuda")
        trials = torch.zeros(B, dtype=torch.int32, device="cuda")
        valid = torch.zeros(B, dtype=torch.int32, device="cuda")
        rx.launch(src, B, n0, gain, hard, trials, valid, torch.cuda.current_stream())
        torch.cuda.synchronize()
        outs.append((hard.cpu().numpy(), trials.cpu().numpy(), valid.cpu().numpy()))
    for a, b in zip(outs[0], outs[1]):
        assert (a == b).all()
    assert (outs[0][1] >= 0).sum() > B // 2 and (outs[0][0][:, :msg.shape[1]] == msg).all(axis=1).sum() > B // 2


def test_extract_rejects_bad_frames(cuda):
    torch = cuda
    x = cs.pl_extractor([0], max_frames=2)
    buf = torch.zeros(2 * 40000, dtype=torch.float32, device="cuda")
    with pytest.raises(cs.CusatError):
        x.extract(x.frames([buf], [buf], [0], [0]))        # dummy PLFRAME: no data
    with pytest.raises(cs.CusatError):
        x.extract(x.frames([buf], [buf], [(12 << 2) | 1], [9]))  # scrambling code not in the extractor
    with pytest.raises(cs.CusatError):
        x.extract(x.frames([buf] * 3, [buf] * 3, [49] * 3, [0] * 3))  # more than max_frames
    with pytest.raises(cs.CusatError):
        cs.pl_extractor([262142])
