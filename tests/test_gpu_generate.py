"""GPU traffic generation (BCH + LDPC encode, mapping) equals this library's
host encoder and mapper bit for bit (those are held equal to the oracle's by
test_capi_host.py), for every constellation family, both frame sizes and
batch sizes around the kernels' work splits."""
import numpy as np
import pytest

import cusat_gb300 as cs
from cusat_gb300 import enums as E

pytestmark = pytest.mark.gpu

NORMAL, SHORT = E.FECFRAME_NORMAL, E.FECFRAME_SHORT
CASES = [("qpsk1/2", SHORT), ("qpsk1/4", NORMAL), ("8psk3/5", NORMAL), ("8psk3/5", SHORT), ("16apsk3/4", NORMAL),
         ("32apsk4/5", NORMAL), ("64apsk32/45", NORMAL), ("8psk9/10", NORMAL), ("16apsk2/3", SHORT),
         ("128apsk3/4", NORMAL), ("256apsk2/3", NORMAL), ("256apsk29/45", NORMAL)]


@pytest.mark.parametrize("name,fs", CASES)
@pytest.mark.parametrize("B", [1, 5, 33])
def test_generator_matches_host(cuda, name, fs, B):
    torch = cuda
    _, mod, rate, _, _, _ = E.find_modcod(name)
    g = cs.generator(mod, rate, fs, max_batch=64)
    ci = cs.code_info(fs, rate)
    assert g.msg_bytes == ci["k_bch"] // 8 and g.cw_bytes == ci["n_ldpc"] // 8
    rng = np.random.default_rng(B * 7 + rate)
    msg = rng.integers(0, 256, (B, g.msg_bytes), dtype=np.uint8)
    d_msg = torch.from_numpy(msg).cuda()
    d_cw = torch.zeros((B, g.cw_bytes), dtype=torch.uint8, device="cuda")
    d_sym = torch.zeros((B, 2 * g.xfec), dtype=torch.float32, device="cuda")
    g.generate(d_msg, B, d_cw, d_sym, torch.cuda.current_stream())
    torch.cuda.synchronize()
    cw = cs.encode_frames(fs, rate, msg)
    assert (d_cw.cpu().numpy() == cw).all()
    sym = cs.map_frames(mod, rate, fs, cw)
    assert np.array_equal(d_sym.cpu().numpy().view(np.uint32), sym.view(np.uint32))


def test_generator_edges(cuda):
    torch = cuda
    g = cs.generator(E.MOD_QPSK, E.RATE_1_2, SHORT, max_batch=4)
    d = torch.zeros((4, g.cw_bytes), dtype=torch.uint8, device="cuda")
    m = torch.zeros((4, g.msg_bytes), dtype=torch.uint8, device="cuda")
    g.generate(m, 4, d, None, torch.cuda.current_stream())   # symbols optional
    torch.cuda.synchronize()
    assert int(d.sum().item()) == 0                          # the zero message encodes to zero
    with pytest.raises(cs.CusatError):
        g.generate(m, 5, d)                                   # above max_batch
    with pytest.raises(cs.CusatError):
        cs.generator(E.MOD_QPSK, E.RATE_9_10, SHORT)          # no short 9/10 code
